"""Shared comparison helpers for the parity tests (CUDA path vs the oracle)."""
import numpy as np

from cmag_gb300 import _abi

# Tolerances, one step from an identical state, FP32.  The CUDA kernels sum the
# same terms in a different order (row runs, lane groups, FMA) and use
# multiplication chains where the reference calls powf, so floating-point
# results agree to a few ulp per term; the bounds below leave ~10x headroom.
TOL_RHO = 1e-5        # |d rho| / rho0
TOL_P = 1e-4          # |d p| <= TOL_P * max|p| + |dp/drho| * TOL_RHO * rho0
TOL_FORCE = 2e-4      # |d a| <= TOL_FORCE * scale, scale = max|a| over the scene
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
    if check_forces:
        if p.system == _abi.PERISTALSIS:
            pairs = (("vforce", ref.vforce), ("pforce", ref.pforce))
        else:
            pairs = (("acc", ref.acc),)
        for name, want in pairs:
            scale = float(np.abs(want[:, :3]).max()) + 1e-30
            out[name] = rel_err(gpu_state[name][:, :3], want[:, :3], scale)
            assert out[name] <= TOL_FORCE, "%s%s error %g (scale %g)" % (label, name, out[name], scale)
    dx = 2.0 * float(p.particle_radius)
    out["pos"] = rel_err(gpu_state["pos"][:, :3], ref.pos[:, :3], dx)
    assert out["pos"] <= TOL_POS, "%sposition error %g dx" % (label, out["pos"])
    vscale = float(np.abs(ref.vel[:, :3]).max()) + 1e-30
    out["vel"] = rel_err(gpu_state["vel"][:, :3], ref.vel[:, :3], vscale)
    assert out["vel"] <= TOL_FORCE, "%svelocity error %g" % (label, out["vel"])
    return out
