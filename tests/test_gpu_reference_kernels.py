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

from helpers import TOL_RHO, TOL_TERM, assert_int_equal

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def reference_scene(num):
    kw = presets.dambreak_xfront(num)
    p = presets.dambreak_params(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
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
    rho_err = np.abs(got["meas"][:, 0].astype(np.float64) - ref.get(cm.MEASURES)[:, 0]).max() / float(p.rest_density)
    assert rho_err <= TOL_RHO, "density differs from the reference kernels by %g rho0" % rho_err
    # accelerations: both within the tolerance of the exact sum, measured on the
    # oracle's conditioning scale for this step
    ora = O.OracleState(s.params, s.getNumParticles())
    ora.pos[:], ora.vel[:], ora.vlf[:], ora.meas[:] = st["pos"], st["vel"], st["vlf"], st["meas"]
    ora.p.right_boundary = s.params.right_boundary
    ora.step(stop_after=_abi.STAGE_FORCE, threads=THREADS)
    _, _, sa, _ = ora.forces_on(got["meas"], threads=THREADS)
    fluid = got["pos"][:, 3] == _abi.FLUID
    err = np.abs(got["acc"][fluid, :3].astype(np.float64) - ref.get(cm.ACCELERATION)[fluid, :3])
    worst = float((err / (sa[fluid, :3] + 1e-30)).max())
    assert worst <= 2 * TOL_TERM, "accelerations differ from the reference kernels by %g of the scale" % worst
    pos_err = np.abs(got["pos"][:, :3] - ref.get(cm.POSITION)[:, :3]).max() / (2.0 * float(p.particle_radius))
    print("num=%d: |drho|/rho0 %.2e, acc %.2e of scale, |dx|/dx %.2e" % (num, rho_err, worst, pos_err))
    assert pos_err < 1e-5
    ref.close()
    s.close()
