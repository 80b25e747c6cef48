"""Kept densities of dam-break walls (cmag_system_set_wall_cache).

A non-fluid particle with no fluid particle in its searched cell box gets the
density its cell walk gave on an earlier step of the same epoch.  The walk would
visit the same non-fluid particles in the same runs and order, so the solver
must produce the same bits with and without the cache, step after step, while
the surge reaches new walls, after the gate is removed and after positions are
set from the host."""
import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets

pytestmark = pytest.mark.gpu

ARRAYS = (cm.POSITION, cm.VELOCITY, cm.VELOCITYLEAPFROG, cm.MEASURES, cm.ACCELERATION)


def same_bits(a, b, label):
    for arr in ARRAYS:
        x, y = a.getArray(arr), b.getArray(arr)
        bad = np.flatnonzero((x.view(np.uint32) != y.view(np.uint32)).any(axis=1))
        assert bad.size == 0, "%s: array %d differs in %d rows (first %s)" % (label, arr, bad.size, bad[:5])


def dambreak3d_pair(fluid=(12, 24, 10), tank=(40, 32, 12), dt=None):
    p, n, tank, L = presets.dambreak3d(fluid=fluid, tank=tank, layers=3)
    if dt:
        p.delta_time = np.float32(dt)
    out = []
    for on in (True, False):
        s = cm.DamBreakSystem(params=p, num_particles=n)
        s.scene3d(tank, L, 0.01, 1973)
        s.set_wall_cache(on)
        assert s.wall_cache() == on
        out.append(s)
    return out


@pytest.mark.parametrize("lists", [True, False], ids=["lists", "walk"])
def test_wall_cache_same_bits_3d(gpu, lists):
    """The 3-D column collapses onto the tank floor and runs to the far wall:
    walls come near the fluid and leave it again."""
    a, b = dambreak3d_pair(dt=2e-4)  # a quarter of the CFL limit of this coarse column
    for s in (a, b):
        s.set_neighbor_lists(lists)
    for k in range(8):
        a.update_n(100)
        b.update_n(100)
        same_bits(a, b, "3-D dam break, %d steps" % (100 * (k + 1)))
    lo, hi = a.fluid_extent()
    dx = 2 * float(a.params.particle_radius)
    # the 12 dx column has spread along the floor past 16 dx of the 40 dx tank
    assert hi[0] > 16 * dx, "the surge front is at %.1f dx" % (hi[0] / dx)
    a.close()
    b.close()


def test_wall_cache_follows_host_writes(gpu):
    """A wall particle moved through setArray (no parameter change), then turned
    into fluid: the hash pass sees the changed non-fluid particle and starts a new
    epoch."""
    a, b = dambreak3d_pair()
    a.update_n(20)
    b.update_n(20)
    pos = a.getArray(cm.POSITION)
    walls = np.flatnonzero(pos[:, 3] != _abi.FLUID)
    far = walls[np.argmax(pos[walls, 0])]  # a wall particle at the far end of the tank
    pos[far, 1] += 0.25 * float(a.params.particle_radius)
    for s in (a, b):
        s.setArray(cm.POSITION, pos)
        s.update_n(5)
    same_bits(a, b, "after moving a far wall particle")
    # the same particle turned into fluid
    pos = a.getArray(cm.POSITION)
    pos[far, 3] = _abi.FLUID
    for s in (a, b):
        s.setArray(cm.POSITION, pos)
        s.update_n(3)
    same_bits(a, b, "after a wall particle became fluid")
    a.close()
    b.close()


def test_wall_cache_same_bits_2d_gate(gpu):
    """The reference's 2-D dam break with its gate: held for 200 steps, then
    removed (the gate particles jump away), then released."""
    kw = presets.dambreak_xfront(64)
    out = []
    for on in (True, False):
        p = presets.dambreak_params(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
        p.particle_mass = np.float32(float(p.particle_mass) * 4.0)
        p.delta_time = np.float32(2e-4)
        s = cm.DamBreakSystem(params=p)
        s.reset()
        s.set_wall_cache(on)
        out.append(s)
    a, b = out
    for s in (a, b):
        s.update_n(200)
    same_bits(a, b, "2-D dam break behind the gate")
    for s in (a, b):
        s.removeRightBoundary()
        s.update_n(300)
    same_bits(a, b, "2-D dam break released")
    a.close()
    b.close()


def test_wall_cache_full_size(gpu):
    """The benchmarked 954,860-particle dam break: 300 steps from rest on
    interaction lists, then 20 on the two-lane walk (a new lane count starts a new
    epoch)."""
    a, b = dambreak3d_pair(fluid=(64, 128, 64), tank=(256, 192, 64))
    for s in (a, b):
        s.set_neighbor_lists(True)
        s.update_n(300)
    same_bits(a, b, "full-size dam break, 300 steps")
    for s in (a, b):
        s.set_neighbor_lists(False)
        s.set_groups(2, 2)
        s.update_n(20)
    same_bits(a, b, "full-size dam break, 2 lanes")
    a.close()
    b.close()


def test_wall_cache_refused_elsewhere(gpu):
    kw = presets.poiseuille_dump(16, 64, 3)
    s = cm.PoiseuilleFlowSystem(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    assert not s.wall_cache()
    with pytest.raises(Exception):
        s.set_wall_cache(True)
    s.set_wall_cache(False)
    s.close()


def test_wall_cache_batch_same_bits(gpu):
    """A reduced copy of the benchmark's batch (16 scenes: channels and released
    2-D dam breaks, whose gate particles are parked on one point) with and
    without the kept wall densities, then after a change of one group's lanes."""
    from cmag_gb300.batch import Batch
    P, N, _, _ = presets.batched_scenes(scenes=16, seed=7, lo=2048, hi=16384)
    pair = []
    for on in (True, False):
        b = Batch(P, N)
        for k, p in enumerate(P):
            b.reset(k)
            if p.system == _abi.DAMBREAK:
                b.dambreak_remove_right_boundary(k)
        assert b.wall_cache()
        b.set_wall_cache(on)
        assert b.wall_cache() == on
        b.set_graphs(True, 5)
        pair.append(b)
    a, b = pair

    def same(label):
        for arr in ARRAYS:
            x, y = a.get_array_all(arr), b.get_array_all(arr)
            bad = np.flatnonzero((x.view(np.uint32) != y.view(np.uint32)).any(axis=1))
            assert bad.size == 0, "%s: array %d differs in %d rows" % (label, arr, bad.size)

    for s in (a, b):
        s.update_n(60)
    same("batch, 60 steps")
    g = next(k for k, gr in enumerate(a.groups()) if gr["system"] == _abi.DAMBREAK)
    for s in (a, b):
        s.set_group_lanes(g, 2, 2)
        s.update_n(20)
    same("batch, 20 steps at two lanes")
    a.close()
    b.close()
