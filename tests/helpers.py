"""Shared comparison helpers for the parity tests (CUDA path vs the oracle)."""
import numpy as np

from cmag_gb300 import _abi

# Tolerances, one step from an identical state, FP32.  The CUDA kernels sum the
# same terms in a different order (row runs, lane groups, FMA) and use
# multiplication chains where the reference calls powf, so floating-point
# results agree to a few ulp per term; the bounds below leave ~10x headroom.
TOL_RHO = 1e-5        # |d rho| / rho0
TOL_P = 1e-4          # |d p| <= TOL_P * max|p| + |dp/drho| * TOL_RHO * rho0
TOL_TERM = 3e-5      # |d a_i| <= TOL_TERM * sum_j |pair term ij| (per particle and
                      # component): a reordered FP32 sum of ~100 terms errs by at
                      # most ~100 ulp of the term sum, ~6e-6
TOL_POS = 1e-5        # |d x| / dx after one step


def assert_int_equal(got, want, name):
    got = np.asarray(got)
    want = np.asarray(want)
    if not np.array_equal(got, want):
        bad = np.flatnonzero(got != want)
        raise AssertionError("%s differs at %d of %d entries, first %s: got %s want %s"
                             % (name, bad.size, got.size, bad[:5], got[bad[:5]], want[bad[:5]]))


def cell_tables_equal(gpu_start, gpu_end, ref_start, ref_end):
    assert_int_equal(gpu_start, ref_start, "cellStart")
    occ = ref_start != 0xFFFFFFFF
    assert_int_equal(gpu_end[occ], ref_end[occ], "cellEnd (occupied cells)")


def rel_err(got, want, scale):
    d = np.abs(got.astype(np.float64) - want.astype(np.float64))
    return float(d.max() / scale) if d.size else 0.0


def eos_slope(p):
    """|dp/drho| at rest density."""
    if p.eos == _abi.EOS_TAIT or p.system == _abi.DAMBREAK:
        return 7.0 * float(p.B) / float(p.rest_density) * 1.2 ** 6
    if p.system == _abi.POISEUILLE:
        return float(p.soundspeed) ** 2
    return 50.0 * float(p.soundspeed)


def compare_step(gpu_state, ref, check_forces=True, label=""):
    """Compare one step's outputs; returns a dict of the measured errors."""
    p = ref.p
    out = {}
    assert_int_equal(gpu_state["hash"], ref.hash, label + "hash")
    assert_int_equal(gpu_state["idx"], ref.idx, label + "index")
    assert_int_equal(gpu_state["spos"].view(np.uint32), ref.spos.view(np.uint32), label + "sortedPos")
    assert_int_equal(gpu_state["svel"].view(np.uint32), ref.svel.view(np.uint32), label + "sortedVel")
    rho0 = float(p.rest_density)
    out["rho"] = rel_err(gpu_state["meas"][:, 0], ref.meas[:, 0], rho0)
    assert out["rho"] <= TOL_RHO, "%sdensity error %g" % (label, out["rho"])
    pmax = float(np.abs(ref.meas[:, 1]).max()) + 1e-30
    dp = np.abs(gpu_state["meas"][:, 1].astype(np.float64) - ref.meas[:, 1]).max()
    bound = TOL_P * pmax + eos_slope(p) * TOL_RHO * rho0
    out["p"] = float(dp / pmax)
    assert dp <= bound, "%spressure error %g > %g" % (label, dp, bound)
    dt = float(p.delta_time)
    acc_err = np.zeros((ref.n, 3))
    acc_scale = np.zeros((ref.n, 3))
    if check_forces:
        sa, sb = ref.force_scale()
        if p.system == _abi.PERISTALSIS:
            pairs = (("vforce", ref.vforce, sa), ("pforce", ref.pforce, sb))
        else:
            pairs = (("acc", ref.acc, sa),)
        for name, want, sc in pairs:
            err = np.abs(gpu_state[name][:, :3].astype(np.float64) - want[:, :3])
            scale = sc[:, :3].astype(np.float64)
            # per particle and component: |error| <= TOL_TERM * sum |term| + tiny
            floor = 1e-30 + 1e-12 * float(scale.max())
            out[name] = float((err / (scale + floor)).max())
            assert out[name] <= TOL_TERM, "%s%s error %g of the term sum" % (label, name, out[name])
            acc_err += err
            acc_scale += scale
    dx = 2.0 * float(p.particle_radius)
    out["pos"] = rel_err(gpu_state["pos"][:, :3], ref.pos[:, :3], dx)
    assert out["pos"] <= TOL_POS, "%sposition error %g dx" % (label, out["pos"])
    # v' = v + (g + a) dt: the velocity error is the force error times dt plus
    # the rounding of the update itself
    dv = np.abs(gpu_state["vel"][:, :3].astype(np.float64) - ref.vel[:, :3])
    vbound = TOL_TERM * acc_scale * dt + 4e-7 * (np.abs(ref.vel[:, :3]) + np.abs(np.asarray(p.gravity)) * dt) + 1e-30
    out["vel"] = float((dv / vbound).max())
    assert out["vel"] <= 1.0, "%svelocity error %g of its bound" % (label, out["vel"])
    return out
