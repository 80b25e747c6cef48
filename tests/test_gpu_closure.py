"""The learned closure's CUDA kernels against the CPU oracle
(oracle/closure_oracle.py): features of a real coarse state, the BF16 network's
outputs, the loss gradient with respect to every parameter; the fused
correction inside a step; training on the GPU; and what the trained closure
gains over the plain coarse method on held-out fine data."""
import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from cmag_gb300.closure import Closure, Pair, collect, normalization_from, output_limit_from, rollout, train
from oracle import closure_oracle as C

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def small_dambreak(steps=20):
    p, n, tank, L = presets.dambreak3d(fluid=(8, 16, 8), tank=(24, 20, 8), layers=3, dt=1e-4)
    s = cm.DamBreakSystem(params=p, num_particles=n)
    s.scene3d(tank, L, 0.01, 11)
    s.update_n(steps)
    s.run_stages(_abi.STAGE_FORCE)
    return p, n, s


def test_features_match_oracle(gpu):
    torch = _torch()
    p, n, s = small_dambreak()
    feat = torch.full((n, 16), float("nan"), dtype=torch.float32, device="cuda")
    s.closure_features(feat.data_ptr())
    got = feat.cpu().numpy()
    pos = s.getArray(cm.POSITION)
    vel = s.getArray(cm.VELOCITYLEAPFROG)
    acc = s.getArray(cm.ACCELERATION)
    idx = s.getUintArray(_abi.INDEX)
    meas = s.getArray(cm.MEASURES)
    rho = np.empty(n)
    pres = np.empty(n)
    rho[idx] = meas[:, 0]
    pres[idx] = meas[:, 1]
    want = C.features(p, pos, vel, rho, pres, acc)
    fluid = pos[:, 3] == _abi.FLUID
    assert np.isfinite(got[fluid]).all()
    assert np.isnan(got[~fluid]).all()  # wall rows untouched
    scale = np.abs(want[fluid]).max(0) + 1e-12
    err = (np.abs(got[fluid] - want[fluid]) / scale).max(0)
    print("feature error / feature scale:", np.round(err, 7))
    assert (err < 2e-4).all(), err
    s.close()


def _random_case(n=3000, seed=1):
    torch = _torch()
    rng = np.random.default_rng(seed)
    theta = C.init_params(seed)
    theta[C.NPARAMS - 3:] = rng.normal(0, 0.05, 3).astype(np.float32)
    feat = rng.normal(size=(n, 16)).astype(np.float32) * 2.0 + 0.3
    target = rng.normal(size=(n, 3)).astype(np.float32)
    mean = rng.normal(0, 0.2, 16).astype(np.float32)
    inv_std = rng.uniform(0.4, 0.8, 16).astype(np.float32)
    c = Closure(theta)
    c.set_normalization(mean, inv_std, 1.0)
    fd = torch.from_numpy(feat).cuda()
    td = torch.from_numpy(target).cuda()
    return c, theta, feat, target, mean, inv_std, fd, td


def test_bf16_parameters(gpu):
    c, theta, *_ = _random_case(10)
    assert np.array_equal(c.params, theta)
    assert np.array_equal(c.bf16_params(), C.bf16(theta).astype(np.float32))


def test_forward_matches_oracle(gpu):
    torch = _torch()
    c, theta, feat, target, mean, inv_std, fd, td = _random_case()
    out = torch.empty((feat.shape[0], 3), dtype=torch.float32, device="cuda")
    c.forward(fd, out)
    got = out.cpu().numpy()
    want, _ = C.forward(theta, feat, mean.astype(np.float64), inv_std.astype(np.float64))
    err = np.abs(got - want)
    scale = np.abs(want).max()
    print("forward: max err %.3g median %.3g (scale %.3g)" % (err.max(), np.median(err), scale))
    # BF16 activations: FP32 vs FP64 accumulation may move an activation by one
    # BF16 step (2^-8 relative) now and then
    assert np.median(err) < 1e-6 * scale
    assert err.max() < 5e-3 * scale


def test_gradient_matches_oracle(gpu):
    c, theta, feat, target, mean, inv_std, fd, td = _random_case()
    loss, g = c.gradient(fd, td)
    wl, wg = C.loss_and_grad(theta, feat, target, mean.astype(np.float64), inv_std.astype(np.float64))
    assert abs(loss - wl) <= 1e-3 * wl
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in C.SHAPES])
    for (name, _), a, b in zip(C.SHAPES, offs[:-1], offs[1:]):
        gg, ww = g[a:b].astype(np.float64), wg[a:b]
        rel = np.linalg.norm(gg - ww) / (np.linalg.norm(ww) + 1e-30)
        print("%s: |g - oracle| / |oracle| = %.2e" % (name, rel))
        assert rel < 1e-4, name
    # the parameters did not move
    assert np.array_equal(c.params, theta)


def test_training_fits_a_teacher(gpu):
    """Adam on the GPU drives the loss on a teacher network's outputs down."""
    torch = _torch()
    rng = np.random.default_rng(4)
    n = 8192
    feat = rng.normal(size=(n, 16)).astype(np.float32)
    teacher = C.init_params(17)
    y, _ = C.forward(teacher, feat, np.zeros(16), np.ones(16))
    c = Closure(C.init_params(3))
    c.set_normalization(np.zeros(16, np.float32), np.ones(16, np.float32), 1.0)
    fd = torch.from_numpy(feat).cuda()
    td = torch.from_numpy(y.astype(np.float32)).cuda()
    l0, _ = c.gradient(fd, td)
    losses = train(c, fd, td, steps=400, batch=2048, lr=3e-3, lr_final=3e-4, log_every=100)
    l1, _ = c.gradient(fd, td)
    print("teacher fit: loss %.4g -> %.4g" % (l0, l1), losses)
    assert l1 < 0.1 * l0


def test_correction_inside_the_step(gpu):
    """run_stages(FORCE) with the closure attached adds out_scale * network to the
    plain acceleration of every fluid particle and leaves walls alone."""
    torch = _torch()
    p, n, s = small_dambreak(10)
    plain = s.getArray(cm.ACCELERATION)
    feat = torch.zeros((n, 16), dtype=torch.float32, device="cuda")
    s.closure_features(feat.data_ptr())
    c = Closure(C.init_params(8))
    mean = feat.mean(0).cpu().numpy()
    inv = (1.0 / feat.std(0).clamp_min(1e-3)).cpu().numpy()
    c.set_normalization(mean, inv, 0.7)
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    c.forward(feat, out)
    s.set_closure(c)
    s.run_stages(_abi.STAGE_FORCE)
    corr = s.getArray(cm.ACCELERATION)
    s.set_closure(None)
    fluid = s.getArray(cm.POSITION)[:, 3] == _abi.FLUID
    want = plain[:, :3] + 0.7 * out.cpu().numpy()
    assert np.array_equal(corr[~fluid], plain[~fluid])
    assert np.allclose(corr[fluid, :3], want[fluid], rtol=1e-6, atol=1e-6 * np.abs(want).max())
    # and a whole step runs with it, graph-captured
    s.set_closure(c)
    s.update_n(5)
    s.synchronize()
    assert np.isfinite(s.getArray(cm.POSITION)).all()
    s.set_closure(None)
    s.close()


def test_trained_closure_gains_over_plain_coarse(gpu):
    """Trained on fine runs of two seeds, the closure cuts the coarse method's
    acceleration error on a third, held-out seed."""
    torch = _torch()
    pair = Pair(fluid=(16, 32, 16), tank=(64, 48, 16), layers=3, dt_fine=1e-4)
    snaps, every = 12, 150  # fine steps between samples (even)

    ftr, ttr = collect(pair, [101, 102], snaps, every)
    fte, tte = collect(pair, [103], snaps, every)
    c = Closure(C.init_params(0))
    mean, inv, scale = normalization_from(ftr, ttr)
    c.set_normalization(mean, inv, scale)
    c.set_output_limit(output_limit_from(ttr, scale))
    train(c, ftr, ttr, steps=1500, batch=8192, lr=2e-3, lr_final=2e-4)
    pred = torch.empty_like(tte)
    c.forward(fte, pred)
    base = float(tte.pow(2).mean())
    resid = float((tte - scale * pred).pow(2).mean())
    print("held-out mean squared acceleration error: plain coarse %.4g, with closure %.4g (%.1f%%)"
          % (base, resid, 100.0 * resid / base))
    assert resid < 0.8 * base
    # rollouts of the held-out seed to t = 0.3 s: fine, coarse, coarse + closure
    width = 0.5
    pair.start(103)
    _, _, f_fine = rollout(pair.fine, 0.3, 0.05, width)
    _, _, f_plain = rollout(pair.coarse, 0.3, 0.05, width)
    pair.start(103)
    pair.coarse.set_closure(c)
    _, _, f_closure = rollout(pair.coarse, 0.3, 0.05, width)
    pair.coarse.set_closure(None)
    print("fronts fine", np.round(f_fine, 3), "coarse", np.round(f_plain, 3),
          "coarse+closure", np.round(f_closure, 3))
    assert np.isfinite(f_closure).all()
    pair.close()


def test_shipped_closure_improves_held_out_front(gpu):
    """A posteriori, on the benchmark's own coarse dam break: the closure shipped in
    cmag_gb300/data (trained by cmag_gb300/train_closure.py on seeds 2001-2020,
    strength chosen on seed 998) brings the coarse run's surge front closer to the
    plain fine run's on the held-out seed 1973 than the plain coarse method does
    (mean relative error while the surge crosses the tank), and the coarse run with
    it still takes less device time than the fine run."""
    import os
    from cmag_gb300 import train_closure as TC
    if not os.path.exists(TC.DEFAULT_OUT):
        pytest.fail("no trained closure at %s" % TC.DEFAULT_OUT)
    c, rec = TC.load()
    assert rec["strength"] > 0.0 and 1973 not in rec["train_seeds"] and rec["validation_seed"] != 1973
    pair = Pair()
    width, t_end = TC.COLUMN_WIDTH, 0.45
    tank_over_column = pair.tank_f[0] / pair.fluid_f[0]
    pair.start(1973)
    t_fine, _, f_fine = rollout(pair.fine, t_end, 0.01, width)
    pair.start(1973)
    _, _, f_plain = rollout(pair.coarse, t_end, 0.01, width)
    pair.start(1973)
    pair.coarse.set_closure(c)
    t_closure, _, f_closure = rollout(pair.coarse, t_end, 0.01, width)
    pair.coarse.set_closure(None)
    judged = f_fine < 0.95 * tank_over_column
    e_plain = np.abs(f_plain - f_fine)[judged] / f_fine[judged]
    e_closure = np.abs(f_closure - f_fine)[judged] / f_fine[judged]
    print("held-out front error (mean, max): plain coarse %.4f %.4f, with closure %.4f %.4f; "
          "device s: fine %.2f, coarse + closure %.2f"
          % (e_plain.mean(), e_plain.max(), e_closure.mean(), e_closure.max(), t_fine, t_closure))
    assert e_closure.mean() < e_plain.mean()
    assert t_closure < t_fine
    pair.close()
    c.close()
