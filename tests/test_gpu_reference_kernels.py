"""The library against the reference's own CUDA kernels on the GPU.

DamBreak.Core/fluid_kernel.cu, compiled for the GB300 (oracle/ref/Makefile,
target gpu-cubin) and driven in the order of DamBreakSystem::update
(oracle/ref/ref_gpu_launch.cu, thrust::sort_by_key as the reference), takes one
step from the same state as the library on the reference's own 2-D dam break
(reference physics): sort order and cell order agree exactly, densities within
1e-5 rho0 and accelerations within the force tolerance of tests/helpers.py
(measured against the oracle's per-particle conditioning scale; the reference
build fuses multiply-adds where nvcc chooses, the library only where it writes
them out).  Skipped where the reference cubin was not built (it is built from
the reference sources, so it exists only where they were)."""
import os

import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from oracle import oracle as O
from oracle import ref_gpu as RG

from helpers import TOL_RHO, TOL_TERM, assert_int_equal, rho_err

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def reference_scene(num):
    """The reference's dam break (XFrontTest.h:17-23) with a num x 2num column.  The
    reference's particle mass (fluidSystem.cpp:49) and dt (1e-4) belong to its
    num = 128 column: the mass scales with the particle area and dt with the
    spacing, so every size has the reference's rest density and CFL number."""
    kw = presets.dambreak_xfront(num)
    p = presets.dambreak_params(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    p.particle_mass = np.float32(float(p.particle_mass) * (128.0 / num) ** 2)
    p.delta_time = np.float32(1e-4 * 128 / num)
    s = cm.DamBreakSystem(params=p)
    s.reset()
    return s, p


@pytest.mark.parametrize("num", [64, 256])
def test_library_equals_reference_kernels_one_step(gpu, num):
    if not RG.available():
        pytest.skip("reference GPU kernels not built (no reference tree where the cubin is made)")
    s, p = reference_scene(num)
    s.removeRightBoundary()
    s.update_n(50)  # a moving state: the column has started to collapse
    st = s.state()
    ref = RG.RefGpu(s.params, st["pos"])
    for name, a in (("vel", cm.VELOCITY), ("vlf", cm.VELOCITYLEAPFROG), ("meas", cm.MEASURES)):
        ref.set(a, st[name])
    ref.steps(1)
    s.update()
    s.synchronize()
    got = s.state()
    assert_int_equal(got["idx"], ref.index(), "sorted index")
    assert_int_equal(got["spos"].view(np.uint32), ref.get(cm.SORTEDPOSITION).view(np.uint32), "sortedPos")
    # the reference's pair terms are NaN (0 * inf) for coincident particles (the
    # parked gate particles, which the library skips); those rows are left out
    ref_meas, ref_acc = ref.get(cm.MEASURES), ref.get(cm.ACCELERATION)
    assert np.isfinite(got["meas"]).all() and np.isfinite(got["acc"]).all()
    ok = np.isfinite(ref_meas[:, 0])
    nan_rows = int((~ok).sum())
    u, c = np.unique(got["spos"][:, :3], axis=0, return_counts=True)
    assert nan_rows <= int(c[c > 1].sum()), "NaN rows of the reference beyond its coincident particles"
    drho = rho_err(got["meas"][ok, 0], ref_meas[ok, 0], float(p.rest_density))
    assert drho <= TOL_RHO, "density differs from the reference kernels by %g" % drho
    # accelerations: both within the tolerance of the exact sum, measured on the
    # oracle's conditioning scale for this step
    ora = O.OracleState(s.params, s.getNumParticles())
    ora.pos[:], ora.vel[:], ora.vlf[:], ora.meas[:] = st["pos"], st["vel"], st["vlf"], st["meas"]
    ora.p.right_boundary = s.params.right_boundary
    ora.step(stop_after=_abi.STAGE_FORCE, threads=THREADS)
    _, _, sa, _ = ora.forces_on(got["meas"], threads=THREADS)
    fluid = (got["pos"][:, 3] == _abi.FLUID) & np.isfinite(ref_acc).all(axis=1)
    err = np.abs(got["acc"][fluid, :3].astype(np.float64) - ref_acc[fluid, :3])
    worst = float((err / (sa[fluid, :3] + 1e-30)).max())
    assert worst <= 2 * TOL_TERM, "accelerations differ from the reference kernels by %g of the scale" % worst
    # positions after the step: the acceleration differences above times dt^2,
    # i.e. a few ulp of the coordinates
    ref_pos = ref.get(cm.POSITION)
    fin = np.isfinite(ref_pos).all(axis=1)
    dpos = np.abs(got["pos"][fin, :3].astype(np.float64) - ref_pos[fin, :3])
    ulps = float((dpos / (np.spacing(np.abs(ref_pos[fin, :3])).astype(np.float64) + 1e-30)).max())
    print("num=%d: |drho|/rho %.2e, acc %.2e of scale, position %.1f ulp, reference NaN rows %d"
          % (num, drho, worst, ulps, nan_rows))
    assert ulps <= 4.0
    ref.close()
    s.close()


def test_dambreak_front_follows_the_reference_kernels(gpu):
    """XFrontTest's quantity (the surge front, XFrontTest.h:64-86: the largest fluid x,
    here in column widths from the world origin) on the reference's own 2-D dam
    break (a 64 x 128 column released at t = 0), the library against the
    reference's kernels run side by side on the GPU: the fronts agree within 1 % of
    the column width while the surge crosses the tank (the two runs round
    differently, so they drift apart only through the flow's own sensitivity)."""
    if not RG.available():
        pytest.skip("reference GPU kernels not built (no reference tree where the cubin is made)")
    s, p = reference_scene(64)
    s.removeRightBoundary()
    ref = RG.RefGpu(s.params, s.getArray(cm.POSITION))
    width = 64 * 2.0 * float(p.particle_radius)
    fronts = []
    for k in range(30):
        s.update_n(100)
        ref.steps(100)
        a = s.getArray(cm.POSITION)
        b = ref.get(cm.POSITION)
        fa = a[a[:, 3] == _abi.FLUID, 0].max() / width
        fb = np.nanmax(b[b[:, 3] == _abi.FLUID, 0]) / width
        fronts.append((fa, fb))
    fronts = np.array(fronts)
    dev = np.abs(fronts[:, 0] - fronts[:, 1])
    print("fronts (library, reference kernels) every 0.01 s:", np.round(fronts, 3).tolist())
    assert fronts[-1, 0] - fronts[0, 0] > 1.5, "the surge did not advance"
    assert dev.max() < 0.01, "fronts differ by %.3f column widths" % dev.max()
    ref.close()
    s.close()
