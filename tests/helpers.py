"""Shared comparison helpers for the parity tests (CUDA path vs the oracle).

A step is compared stage by stage from identical inputs:
  * hash, sort, cell ranges and the sorted gathers: bit for bit;
  * density: |d rho| <= TOL_RHO max(rho0, |rho|) (rounding scales with the sum:
    a pile of coincident particles, such as the parked gate of a released dam
    break, reaches tens of rho0);
  * pressure: the density bound carried through the equation of state
    (near rest density the Tait form amplifies density rounding ~7/(x-1) times);
  * forces: the oracle recomputes them on the GPU's own measures, and the
    difference must stay within TOL_TERM of the force's conditioning scale (per
    particle and component, the sum over pair terms of the product of the
    magnitudes of their factors -- the bound on rounding for any summation
    order and formula arrangement);
  * integration: the oracle integrates the pre-step state with the GPU's own
    forces; the difference is a few ulp of the magnitudes involved.
"""
import numpy as np

from cmag_gb300 import _abi

TOL_RHO = 1e-5       # |d rho| / rho0
TOL_P = 1e-4         # |d p| <= TOL_P * max|p| + |dp/drho| * TOL_RHO * rho0
TOL_TERM = 3e-5      # |d a_i| <= TOL_TERM * conditioning scale_i
TOL_ULP = 5e-7       # integration: a few float32 ulp of the operand magnitudes


def assert_int_equal(got, want, name):
    got = np.asarray(got)
    want = np.asarray(want)
    if not np.array_equal(got, want):
        bad = np.flatnonzero(got != want)
        raise AssertionError("%s differs at %d of %d entries, first %s: got %s want %s"
                             % (name, bad.size, got.size, bad[:5], got.ravel()[bad[:5]],
                                want.ravel()[bad[:5]]))


def cell_tables_equal(gpu_start, gpu_end, ref_start, ref_end):
    assert_int_equal(gpu_start, ref_start, "cellStart")
    occ = ref_start != 0xFFFFFFFF
    assert_int_equal(gpu_end[occ], ref_end[occ], "cellEnd (occupied cells)")


def rel_err(got, want, scale):
    d = np.abs(got.astype(np.float64) - want.astype(np.float64))
    return float(d.max() / scale) if d.size else 0.0


def rho_err(got, want, rho0):
    """Largest density difference relative to max(rho0, |rho|) of the particle."""
    want = want.astype(np.float64)
    d = np.abs(got.astype(np.float64) - want) / np.maximum(rho0, np.abs(want))
    return float(d.max()) if d.size else 0.0


def eos_slope(p):
    """|dp/drho| up to 1.2 rho0."""
    if p.eos == _abi.EOS_TAIT or p.system == _abi.DAMBREAK:
        return 7.0 * float(p.B) / float(p.rest_density) * 1.2 ** 6
    if p.system == _abi.POISEUILLE:
        return float(p.soundspeed) ** 2
    return 50.0 * float(p.soundspeed)


def configured_walls(pre):
    """True when the step after `pre` moves the Peristalsis walls with
    configureBoundary (sinf) before hashing."""
    p = pre.p
    return (p.system == _abi.PERISTALSIS and p.is_boundary_configuration
            and pre.phase[3] < np.float32(p.amplitude))


def compare_step(gpu, pre, post, label="", threads=1):
    """gpu: dict of the GPU arrays after one step from `pre`; post: the oracle's
    state after the same step (threads: host threads of the oracle's force
    recomputation).  Returns the measured error ratios."""
    from oracle import oracle as O
    p = post.p
    out = {}
    walls_moved = configured_walls(pre)
    assert_int_equal(gpu["hash"], post.hash, label + "hash")
    assert_int_equal(gpu["idx"], post.idx, label + "index")
    if walls_moved:  # walls placed with the GPU's sinf: fluid exact, walls within 1e-5 r
        fluid = post.spos[:, 3] == 0
        assert_int_equal(gpu["spos"][fluid].view(np.uint32), post.spos[fluid].view(np.uint32),
                         label + "sortedPos (fluid)")
        assert np.abs(gpu["spos"][:, :3] - post.spos[:, :3]).max() <= 1e-5 * p.particle_radius
    else:
        assert_int_equal(gpu["spos"].view(np.uint32), post.spos.view(np.uint32), label + "sortedPos")
    assert_int_equal(gpu["svel"].view(np.uint32), post.svel.view(np.uint32), label + "sortedVel")

    rho0 = float(p.rest_density)
    out["rho"] = rho_err(gpu["meas"][:, 0], post.meas[:, 0], rho0)
    assert out["rho"] <= TOL_RHO, "%sdensity error %g" % (label, out["rho"])
    pmax = float(np.abs(post.meas[:, 1]).max()) + 1e-30
    dp = np.abs(gpu["meas"][:, 1].astype(np.float64) - post.meas[:, 1]).max()
    bound = TOL_P * pmax + eos_slope(p) * TOL_RHO * rho0
    out["p"] = float(dp / bound)
    assert dp <= bound, "%spressure error %g > %g" % (label, dp, bound)

    a, b, sa, sb = post.forces_on(gpu["meas"], spos=gpu["spos"], threads=threads)
    if p.system == _abi.PERISTALSIS:
        pairs = (("vforce", a, sa), ("pforce", b, sb))
    else:
        pairs = (("acc", a, sa),)
    for name, want, sc in pairs:
        err = np.abs(gpu[name][:, :3].astype(np.float64) - want[:, :3])
        scale = sc[:, :3].astype(np.float64) + 1e-30
        out[name] = float((err / scale).max())
        assert out[name] <= TOL_TERM, "%s%s error %g of its conditioning scale" % (label, name, out[name])

    zeros = np.zeros_like(gpu["pos"])
    pos, vel, vlf = O.integrate_from(pre, post, gpu.get("acc", zeros), gpu.get("vforce", zeros),
                                     gpu.get("pforce", zeros))
    dt = float(p.delta_time)
    g = np.abs(np.asarray(list(p.gravity), np.float64))
    accm = sum(np.abs(gpu[k][:, :3].astype(np.float64)) for k in ("acc", "vforce", "pforce") if k in gpu)
    vmag = np.abs(pre.vel[:, :3].astype(np.float64)) + (g + accm) * dt
    for name, want, mag in (("vel", vel, vmag), ("vlf", vlf, vmag),
                            ("pos", pos, np.abs(pre.pos[:, :3].astype(np.float64)) + vmag * dt)):
        err = np.abs(gpu[name][:, :3].astype(np.float64) - want[:, :3])
        if name == "pos" and walls_moved:
            mag = mag + p.particle_radius * 20.0  # walls placed with the GPU's sinf
        out[name] = float((err / (TOL_ULP * mag + 1e-30)).max())
        assert out[name] <= 1.0, "%s%s error %g of its bound" % (label, name, out[name])
    return out


def compare_step_kept(gpu, pre, post, label="", threads=1):
    """compare_step for a solver on kept neighbour lists (cmag_system_set_verlet):
    its sorted arrays keep the order of the last list rebuild, so density and
    pressure are compared per particle (original order, through each side's
    sorted index) and the oracle recomputes the forces on the GPU's measures
    brought into the oracle's sorted order.  gpu: a state() dict."""
    from oracle import oracle as O
    p = post.p
    out = {}
    n = post.n
    meas_orig = np.zeros((n, 4), np.float32)
    meas_orig[gpu["idx"]] = gpu["meas"]
    want_orig = np.zeros((n, 4), np.float32)
    want_orig[post.idx] = post.meas
    # the gathers in the rebuild's order hold the step's positions and velocities
    spos_orig = np.zeros((n, 4), np.float32)
    spos_orig[gpu["idx"]] = gpu["spos"]
    assert_int_equal(spos_orig.view(np.uint32), pre.pos.view(np.uint32), label + "gathered positions")
    svel_orig = np.zeros((n, 4), np.float32)
    svel_orig[gpu["idx"]] = gpu["svel"]
    assert_int_equal(svel_orig.view(np.uint32), pre.vlf.view(np.uint32), label + "gathered leap-frog velocities")

    rho0 = float(p.rest_density)
    out["rho"] = rho_err(meas_orig[:, 0], want_orig[:, 0], rho0)
    assert out["rho"] <= TOL_RHO, "%sdensity error %g" % (label, out["rho"])
    pmax = float(np.abs(want_orig[:, 1]).max()) + 1e-30
    dp = np.abs(meas_orig[:, 1].astype(np.float64) - want_orig[:, 1]).max()
    bound = TOL_P * pmax + eos_slope(p) * TOL_RHO * rho0
    out["p"] = float(dp / bound)
    assert dp <= bound, "%spressure error %g > %g" % (label, dp, bound)

    meas_oracle_order = np.ascontiguousarray(meas_orig[post.idx])
    a, b, sa, sb = post.forces_on(meas_oracle_order, threads=threads)
    if p.system == _abi.PERISTALSIS:
        pairs = (("vforce", a, sa), ("pforce", b, sb))
    else:
        pairs = (("acc", a, sa),)
    for name, want, sc in pairs:
        err = np.abs(gpu[name][:, :3].astype(np.float64) - want[:, :3])
        scale = sc[:, :3].astype(np.float64) + 1e-30
        out[name] = float((err / scale).max())
        assert out[name] <= TOL_TERM, "%s%s error %g of its conditioning scale" % (label, name, out[name])

    zeros = np.zeros_like(gpu["pos"])
    pos, vel, vlf = O.integrate_from(pre, post, gpu.get("acc", zeros), gpu.get("vforce", zeros),
                                     gpu.get("pforce", zeros))
    dt = float(p.delta_time)
    g = np.abs(np.asarray(list(p.gravity), np.float64))
    accm = sum(np.abs(gpu[k][:, :3].astype(np.float64)) for k in ("acc", "vforce", "pforce") if k in gpu)
    vmag = np.abs(pre.vel[:, :3].astype(np.float64)) + (g + accm) * dt
    for name, want, mag in (("vel", vel, vmag), ("vlf", vlf, vmag),
                            ("pos", pos, np.abs(pre.pos[:, :3].astype(np.float64)) + vmag * dt)):
        err = np.abs(gpu[name][:, :3].astype(np.float64) - want[:, :3])
        out[name] = float((err / (TOL_ULP * mag + 1e-30)).max())
        assert out[name] <= 1.0, "%s%s error %g of its bound" % (label, name, out[name])
    return out
