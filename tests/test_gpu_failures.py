"""Failure reporting without a GPU fault, and update(dt).

* A look-back wait of the radix sort that runs out: with the spin limit set to 0
  (cmag_testing_set_sort_spin_limit) every wait that finds its predecessor tile
  unpublished gives up at once, so a multi-tile sort reports CMAG_ERR_DEVICE
  with the look-back bit; with the default limit restored the next call sorts
  correctly.  The waits end by themselves and every scatter stays in bounds.
* A planar particle moved out of its z layer behind the solver's back (through
  the borrowed device pointer) is hashed outside the scanned cell table; the
  step completes and cmag_system_synchronize reports CMAG_DEVERR_RANGE.
* update(dt) (the reference's update() with dt in its parameter block) equals
  setting delta_time and stepping, bit for bit.
"""
import ctypes

import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from cmag_gb300._lib import LIB_PATH, c_u32p, lib

pytestmark = pytest.mark.gpu


def _sort(keys, vals, bits):
    import torch
    k = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    v = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    torch.cuda.synchronize()
    rc = lib().cmag_sort_particles(ctypes.cast(k.data_ptr(), c_u32p), ctypes.cast(v.data_ptr(), c_u32p),
                                   keys.size, bits, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def test_sort_lookback_timeout_is_reported_and_recovers(gpu):
    L = lib()
    rng = np.random.default_rng(7)
    n, bits = 1 << 20, 24  # 256 tiles, three passes
    keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    timed_out = False
    try:
        assert L.cmag_testing_set_sort_spin_limit(0) == 0
        for _ in range(5):  # tiles race their predecessors; one miss is enough
            rc, _, _ = _sort(keys, vals, bits)
            if rc == _abi.CMAG_ERR_DEVICE:
                timed_out = True
                assert b"look-back" in L.cmag_last_error()
                break
            assert rc == 0
    finally:
        assert L.cmag_testing_set_sort_spin_limit(-1) == 0
    assert timed_out, "no look-back wait ran out with a spin limit of 0"
    rc, k, v = _sort(keys, vals, bits)
    assert rc == 0, L.cmag_last_error()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


def test_planar_particle_leaving_its_layer_is_reported(gpu):
    kw = presets.poiseuille_dump(16, 64, 3)
    s = cm.PoiseuilleFlowSystem(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    s.reset()
    s.update()
    s.synchronize()
    assert s.device_error_bits() == 0
    # move particle 0 two cells up in z through the device pointer: the solver
    # still treats the scene as planar (one z layer scanned)
    pos = s.getArray(cm.POSITION)
    z = np.array([pos[0, 2] + 4.0 * float(s.params.particle_radius)], np.float32)
    cudart = ctypes.CDLL(LIB_PATH)  # resolves the CUDA runtime the library links
    cudart.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    dst = s.getCudaPosVBO() + 8  # .z of row 0
    assert cudart.cudaMemcpy(ctypes.c_void_p(dst), z.ctypes.data_as(ctypes.c_void_p), 4, 1) == 0
    s.update()
    with pytest.raises(cm.CmagError):
        s.synchronize()
    assert s.device_error_bits() & _abi.CMAG_DEVERR_RANGE
    assert b"outside the scanned cell range" in lib().cmag_system_last_error(s._h)
    s.close()


@pytest.mark.parametrize("family", ["dambreak", "peristalsis"])
def test_update_dt_equals_params_dt(gpu, family):
    if family == "dambreak":
        make = lambda: cm.DamBreakSystem((16, 32, 1), 1, (64, 64, 4), 1.0 / 256)  # noqa: E731
    else:
        kw = presets.peristalsis_report()
        kw.update(fluid_size=(64, 26, 1), grid_size=(64, 64, 4))

        def make():
            return cm.PeristalsisSystem(kw["dt"], kw["fluid_size"], kw["amplitude"], kw["wave_speed"],
                                        kw["soundspeed"], kw["gravity"], kw["boundary_offset"],
                                        kw["grid_size"], kw["radius"])
    a, b = make(), make()
    a.reset()
    b.reset()
    dt = 0.5 * float(a.params.delta_time)
    q = b.params
    q.delta_time = dt
    b.set_params(q)
    for _ in range(5):
        a.update(dt)
        b.update()
    a.synchronize()
    b.synchronize()
    assert float(a.params.delta_time) == np.float32(dt)
    assert a.getElapsedTime() == b.getElapsedTime()
    for arr in (cm.POSITION, cm.VELOCITY, cm.VELOCITYLEAPFROG):
        assert np.array_equal(a.getArray(arr).view(np.uint32), b.getArray(arr).view(np.uint32))
    a.update()  # dt stays
    assert float(a.params.delta_time) == np.float32(dt)
    a.close()
    b.close()
