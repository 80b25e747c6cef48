"""The C ABI library without a GPU: it loads, exports every entry point that
include/cmag_sph.h declares, and its host-side logic (reference parameter
derivations, particle counts, scene generators, the Peristalsis lattice mass sum)
equals the oracle's bit for bit."""
import ctypes
import os
import re

import numpy as np
import pytest

from cmag_gb300 import _abi, presets
from cmag_gb300._lib import SIGNATURES, c_f32p, check, lib
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "cmag_sph.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cmag_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    L = lib()
    names = header_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(SIGNATURES), set(names) ^ set(SIGNATURES)
    assert lib().cmag_version().startswith(b"cmag_gb300")


def test_params_struct_layout(built):
    # the ctypes mirror must have the layout the library was compiled with
    assert ctypes.sizeof(_abi.SphParams) == lib().cmag_sph_params_size()


REF_SCENES = [
    ("dambreak", lambda: presets.dambreak_params((128, 256, 1), 1, (512, 256, 4), 1 / 256),
     lambda: O.dambreak_params((128, 256, 1), 1, (512, 256, 4), 1 / 256)),
    ("dambreak_off3", lambda: presets.dambreak_params((32, 48, 1), 3, (128, 64, 4), 1 / 256),
     lambda: O.dambreak_params((32, 48, 1), 3, (128, 64, 4), 1 / 256)),
    ("poiseuille", lambda: presets.poiseuille_params(**_pf()), lambda: O.poiseuille_params(**_pf())),
    ("peristalsis", lambda: presets.peristalsis_params(**presets.peristalsis_report()),
     lambda: O.peristalsis_params(**presets.peristalsis_report())),
]


def _pf():
    kw = presets.poiseuille_dump()
    return dict(fluid_size=kw["fluid_size"], boundary_offset=kw["boundary_offset"],
                grid_size=kw["grid_size"], radius=kw["radius"])


@pytest.mark.parametrize("name,prod,orc", REF_SCENES, ids=[s[0] for s in REF_SCENES])
def test_host_params_and_scenes_match_oracle(built, name, prod, orc):
    pp, po = prod(), orc()
    assert bytes(pp) == bytes(po), {k: (v, po.as_dict()[k]) for k, v in pp.as_dict().items()
                                    if v != po.as_dict()[k]}
    n = presets.reference_count(pp)
    assert n == O.particle_count(po)
    pos = np.zeros((n, 4), np.float32)
    check(lib().cmag_reference_scene(ctypes.byref(pp), pos.ctypes.data_as(c_f32p), n))
    assert np.array_equal(pos.view(np.uint32), O.scene(po, n).view(np.uint32))
    if pp.system == _abi.PERISTALSIS:
        out = ctypes.c_float()
        check(lib().cmag_peristalsis_mass_sum(ctypes.byref(pp), pos.ctypes.data_as(c_f32p), n,
                                              ctypes.byref(out)))
        assert out.value == lib_mass(po, pos)


def lib_mass(p, pos):
    return O.lib().orc_peristalsis_mass_sum(ctypes.byref(p), O.fp(pos), pos.shape[0])


def test_reference_constructor_values(built):
    """Spot values of the DamBreak constructor (fluidSystem.cpp:44-75) for the
    XFrontTest scene, computed independently in float32."""
    p = presets.dambreak_params((128, 256, 1), 1, (512, 256, 4), 1 / 256)
    f = np.float32
    r = f(1 / 256)
    assert p.smoothing_radius == f(3) * r
    assert p.particle_mass == f(1000.0 / 16327.6)
    B = f(f(f(200) * f(1000)) * f(9.8)) * f(f(f(2) * r) * f(256)) / f(7)
    assert p.B == B
    assert p.soundspeed == np.sqrt(f(f(p.B * f(7)) / f(1000)))
    assert list(p.world_origin) == [-(f(512) * r), -(f(256) * r), -(f(4) * r)]


def test_dambreak3d_scene_counts(built):
    p, n, tank, L = presets.dambreak3d()
    assert n == 524288 + 430572
    assert list(p.grid_size) == [264, 245, 72]
    small, ns, ts, Ls = presets.dambreak3d(fluid=(8, 16, 8), tank=(32, 24, 8))
    pos = np.zeros((ns, 4), np.float32)
    check(lib().cmag_dambreak3d_scene_host(ctypes.byref(small), _abi.u3(ts), Ls, 0.01, 1973,
                                           pos.ctypes.data_as(c_f32p), ns))
    assert np.array_equal(pos.view(np.uint32), O.dambreak3d_scene(small, ts, Ls, 0.01, 1973).view(np.uint32))
    assert (pos[:, 3] == _abi.FLUID).sum() == 8 * 16 * 8


def test_create_reports_errors_without_exiting(built):
    """Invalid parameters come back as a status code and a message."""
    p = presets.dambreak_params((16, 32, 1), 1, (64, 64, 4), 1 / 256)
    p.grid_size[0] = 5  # narrower than the 2*cell_count+1 searched cells
    h = ctypes.c_void_p()
    rc = lib().cmag_system_create(ctypes.byref(p), 100, ctypes.byref(h))
    assert rc == _abi.CMAG_ERR_INVALID
    assert b"2*cell_count+1" in lib().cmag_last_error()
    p.grid_size[0] = 64
    rc = lib().cmag_system_create(ctypes.byref(p), 0, ctypes.byref(h))
    assert rc == _abi.CMAG_ERR_INVALID


def test_batch_create_reports_errors_without_exiting(built):
    """Batch creation checks every scene before touching the device."""
    good = presets.dambreak_params((16, 32, 1), 1, (64, 64, 4), 1 / 256)
    bad = presets.dambreak_params((16, 32, 1), 1, (64, 64, 4), 1 / 256)
    bad.grid_size[1] = 3
    arr = (_abi.SphParams * 2)(good, bad)
    counts = (ctypes.c_uint32 * 2)(100, 100)
    h = ctypes.c_void_p()
    assert lib().cmag_batch_create(arr, counts, 2, ctypes.byref(h)) == _abi.CMAG_ERR_INVALID
    assert lib().cmag_last_error().startswith(b"scene 1:")
    assert lib().cmag_batch_create(arr, counts, 0, ctypes.byref(h)) == _abi.CMAG_ERR_INVALID
    counts[0] = 0
    assert lib().cmag_batch_create(arr, counts, 1, ctypes.byref(h)) == _abi.CMAG_ERR_INVALID
    assert not h.value


def test_batched_workload_sizes(built):
    """The batched benchmark's scenes: counts log-uniform in the stated range,
    families split in half, cell tables small enough for 32-bit sort keys."""
    P, N, F, D = presets.batched_scenes()
    assert len(P) == 256 and [d[0] for d in D] == ["poiseuille"] * 128 + ["dambreak"] * 128
    assert min(F) >= 0.9 * 4096 and max(F) <= 1.1 * 262144
    assert all(n > f for n, f in zip(N, F))  # walls on top of the fluid
    cells = sum(int(p.grid_size[0]) * int(p.grid_size[1]) for p in P)
    assert cells < 2 ** 32
    for p, d in zip(P, D):
        if d[0] == "poiseuille":
            assert abs(float(p.mu) - 1000 * d[3]) <= 1e-6 * float(p.mu)
            assert 1e-6 * 0.99 <= d[3] <= 1e-4 * 1.01
