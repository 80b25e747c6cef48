"""The neighbour walk of the density and force passes (cmag_gb300/csrc/
neighbor_walk.cuh) against brute force, on the host.

tests/walk_host/walk_check.cpp compiles the product's walk header for the host
(with host restatements of the few device intrinsics it uses), hashes and sorts a
scene like the hash/sort stages, and checks that for every particle and every lane
group the walk visits each particle inside the support exactly once, through the
periodic image shift that gives its true distance.  Seeded scenes of every family
and search shape: planar and 3-D, trimmed and untrimmed rows, 1/2/4 lanes, power
of two and other grid sizes down to the smallest allowed (2c + 1 cells), particles
on cell faces, at the grid's far edges, stacked in one cell, and (DamBreak)
outside the grid, some more than one grid period away."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from cmag_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "walk_host", "walk_check.cpp")
OUT = os.path.join(HERE, "walk_host", "_build", "libwalk_check.so")
CSRC = os.path.join(os.path.dirname(HERE), "cmag_gb300", "csrc")
DEPS = [SRC, os.path.join(CSRC, "neighbor_walk.cuh"), os.path.join(CSRC, "sph_common.cuh"),
        os.path.join(os.path.dirname(HERE), "include", "cmag_sph.h")]


def _cuda_include():
    for root in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "cuda_runtime.h")):
            return os.path.join(root, "include")
    return None


@pytest.fixture(scope="module")
def walk_lib():
    gxx, inc = shutil.which("g++"), _cuda_include()
    if not gxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(d) for d in DEPS):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-Wno-attributes",
                        "-I" + inc, "-I" + CSRC, "-o", OUT, SRC], check=True)
    lib = ctypes.CDLL(OUT)
    lib.walk_check.restype = ctypes.c_int64
    lib.walk_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_float),
                               ctypes.c_float, ctypes.c_float, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_float), ctypes.c_uint32,
                               ctypes.POINTER(ctypes.c_uint64)]
    return lib


def _run(lib, system, planar, trim, lanes, grid, h, pos, cell=1.0):
    c = int(np.ceil(2 * h / cell - 1e-9))
    g = (ctypes.c_uint32 * 3)(*grid)
    o = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
    pos = np.ascontiguousarray(pos, np.float32)
    visited = ctypes.c_uint64()
    bad = lib.walk_check(system, int(planar), int(trim), lanes, g, o, cell, h, c,
                         pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), pos.shape[0],
                         ctypes.byref(visited))
    return bad, visited.value


def _scene(rng, grid, planar, n, outside=False):
    """Random particles in the grid, plus particles on cell faces, at the far edges,
    stacked in one cell and (outside=True) beyond the grid."""
    gx, gy, gz = grid
    w = np.array([gx, gy, gz], np.float64)
    p = rng.uniform(0, 1, (n, 3)) * w
    faces = rng.integers(0, [gx, gy, gz], (n // 8, 3)).astype(np.float64)
    faces[:, 2] += rng.uniform(0, 1, n // 8)
    edges = np.column_stack([np.full(6, gx - 1e-4), rng.uniform(0, gy, 6), rng.uniform(0, gz, 6)])
    edges = np.vstack([edges, np.column_stack([np.full(6, 1e-6), rng.uniform(0, gy, 6), rng.uniform(0, gz, 6)])])
    stack = np.tile(np.array([[gx / 2 + 0.3, gy / 2 + 0.6, gz / 2 + 0.5]]), (9, 1))
    parts = [p, faces, edges, stack]
    if outside:
        parts.append(np.array([[-2.5, 3.3, 1.2], [-0.4, 3.7, 1.6], [gx + 1.5, 2.2, 1.5],
                               [4.5, 2.3 * gy, 1.5], [2.5, -1.2 * gy, 2.5], [-1.7 * gx, 5.5, 0.5]]))
    q = np.vstack(parts)
    if planar:
        q[:, 2] = 2.5 if gz > 2 else 0.5
    else:
        q[:, 2] = np.mod(q[:, 2], gz)
    out = np.zeros((q.shape[0], 4), np.float32)
    out[:, :3] = q
    return out


CASES = [
    # family, planar, trim, grid, h (cells), n, outside
    (_abi.DAMBREAK, True, True, (16, 16, 4), 1.3, 700, True),
    (_abi.DAMBREAK, True, False, (16, 16, 4), 1.3, 700, True),
    (_abi.DAMBREAK, False, True, (13, 11, 9), 1.3, 900, True),
    (_abi.DAMBREAK, False, False, (12, 10, 8), 1.3, 700, True),
    (_abi.DAMBREAK, False, True, (7, 9, 7), 1.3, 500, False),
    (_abi.POISEUILLE, True, True, (16, 32, 4), 1.3, 900, False),
    (_abi.POISEUILLE, True, True, (7, 13, 4), 1.3, 400, False),
    (_abi.PERISTALSIS, True, True, (16, 16, 4), 1.3, 800, False),
    (_abi.PERISTALSIS, True, True, (7, 9, 4), 1.3, 400, False),
    (_abi.PERISTALSIS, False, True, (9, 8, 7), 1.3, 700, False),
    (_abi.DAMBREAK, False, True, (10, 9, 8), 0.65, 900, True),
    (_abi.PERISTALSIS, True, True, (8, 8, 4), 0.5, 500, False),
]


@pytest.mark.parametrize("lanes", [1, 2, 4])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_walk_visits_every_neighbour_once(walk_lib, case, lanes):
    system, planar, trim, grid, h, n, outside = CASES[case]
    rng = np.random.default_rng(1000 + case)
    pos = _scene(rng, grid, planar, n, outside)
    bad, visited = _run(walk_lib, system, planar, trim, lanes, grid, h, pos)
    assert bad == 0, "%d particles with a wrong neighbour set (case %d, lanes %d)" % (bad, case, lanes)
    assert visited > 0


def test_trim_visits_fewer_candidates(walk_lib):
    """The trimmed walk visits a subset of the full cell box's candidates (about
    half in 3-D) and still finds every neighbour."""
    rng = np.random.default_rng(7)
    grid = (13, 11, 9)
    pos = _scene(rng, grid, False, 900)
    bad_t, vis_t = _run(walk_lib, _abi.DAMBREAK, False, True, 1, grid, 1.3, pos)
    bad_f, vis_f = _run(walk_lib, _abi.DAMBREAK, False, False, 1, grid, 1.3, pos)
    assert bad_t == 0 and bad_f == 0
    assert vis_t < 0.7 * vis_f, (vis_t, vis_f)


def test_harness_detects_a_missed_neighbour(walk_lib):
    """The check has teeth: a support larger than the searched box (h = 1.3 cells
    with c = 2, searched 2 cells out for a 2.6-cell support) misses neighbours."""
    rng = np.random.default_rng(3)
    grid = (16, 16, 4)
    pos = _scene(rng, grid, True, 700)
    g = (ctypes.c_uint32 * 3)(*grid)
    o = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
    visited = ctypes.c_uint64()
    bad = walk_lib.walk_check(_abi.DAMBREAK, 1, 0, 1, g, o, 1.0, 1.3, 2,
                              pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), pos.shape[0],
                              ctypes.byref(visited))
    assert bad > 0


@pytest.mark.parametrize("grid,c", [((264, 245, 72), 3), ((16, 16, 4), 3), ((13, 11, 9), 3), ((5, 6, 7), 1),
                                    ((5, 6, 7), 2), ((4, 4, 4), 3), ((9, 33, 10), 2)])
def test_wall_cache_fluid_test_matches_brute_force(walk_lib, grid, c):
    """The kept wall densities' test for fluid in a wall particle's cell box
    (neighbor_walk.cuh: fluid_near) against every cell of the wrapped box: grids
    that are and are not multiples of the 4-cell blocks, boxes wider than the
    grid, cells outside the grid."""
    walk_lib.wall_near_check.restype = ctypes.c_int64
    walk_lib.wall_near_check.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int, ctypes.c_uint32,
                                         ctypes.c_uint64]
    g = (ctypes.c_uint32 * 3)(*grid)
    bad = walk_lib.wall_near_check(g, c, 4000, 1234 + c)
    assert bad == 0, "%d of 4000 cell boxes judged wrongly" % bad
