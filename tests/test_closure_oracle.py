"""The closure oracle without a GPU: its analytic gradient agrees with central
finite differences (float64, without the BF16 rounding, which is piecewise
constant), and its BF16 rounding is round-to-nearest-even."""
import numpy as np

from oracle import closure_oracle as C


def test_bf16_rounding_ties_to_even():
    # 1 + 2^-8 is halfway between the BF16 neighbours 1 and 1 + 2^-7: ties go to 1
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e38, 1e-40], np.float32)
    got = C.bf16(vals)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2.0 ** -6 and got[3] == -2.5
    assert np.isfinite(got[4]) and abs(got[4] / 3.0e38 - 1) < 2 ** -8
    assert abs(got[5] - 1e-40) <= 2.0 ** -134  # half the BF16 subnormal step


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    theta = C.init_params(5).astype(np.float64)
    theta[C.NPARAMS - 3:] = rng.normal(0, 0.1, 3)
    feat = rng.normal(size=(40, C.FEAT))
    target = rng.normal(size=(40, C.OUT))
    mean = rng.normal(0, 0.1, C.FEAT)
    inv_std = rng.uniform(0.5, 2.0, C.FEAT)
    _, g = C.loss_and_grad(theta, feat, target, mean, inv_std, round_bf16=False)
    idx = rng.choice(C.NPARAMS, 60, replace=False)
    eps = 1e-6
    for k in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[k] += eps
        tm[k] -= eps
        lp, _ = C.loss_and_grad(tp, feat, target, mean, inv_std, round_bf16=False)
        lm, _ = C.loss_and_grad(tm, feat, target, mean, inv_std, round_bf16=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_parameter_layout():
    assert C.NPARAMS == 16 * 64 + 64 + 2 * (64 * 64 + 64) + 3 * 64 + 3
    theta = np.arange(C.NPARAMS, dtype=np.float64)
    assert np.array_equal(C.pack(C.unpack(theta)), theta)


def test_normalization_sums_chunk_by_chunk():
    """The training set's normalisation (cmag_gb300.closure.normalization_from)
    sums a chunk of rows at a time; any chunking gives torch's mean, unbiased
    standard deviation and target RMS."""
    torch = __import__("pytest").importorskip("torch")
    from cmag_gb300 import closure as CL
    g = torch.Generator().manual_seed(5)
    feat = torch.randn(10007, 16, generator=g) * torch.linspace(0.1, 30.0, 16) + torch.linspace(-5.0, 5.0, 16)
    tgt = torch.randn(10007, 3, generator=g) * 0.25
    want_mean = feat.double().mean(0).numpy()
    want_std = feat.double().std(0).numpy()
    want_scale = float(tgt.double().pow(2).mean().sqrt())
    for chunk in (1000, 4096, 1 << 24):
        mean, inv, scale = CL.normalization_from(feat, tgt, chunk=chunk)
        assert np.allclose(mean, want_mean, rtol=1e-6, atol=1e-6)
        assert np.allclose(1.0 / inv, want_std, rtol=1e-5)
        assert abs(scale - want_scale) <= 1e-6 * want_scale
