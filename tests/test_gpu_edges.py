"""Edge cases of the step against the oracle.

* Particles outside the grid: their cells wrap by residue, as the reference's
  mask does on power-of-two grids (calcGridHash, fluid_kernel.cu:28-30), also
  more than one grid period away; hash, sort, cell ranges and gathers stay bit for
  bit, the step within the tolerances of tests/helpers.py.
* Coincident particles: equal cell keys keep index order in the sort; the
  reference's pair term of two particles at one position is 0/0 (NaN), which the
  force loop skips, so every force stays finite and all other particles match.
* Scenes of one to three particles."""
import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from oracle import oracle as O

from helpers import TOL_RHO, TOL_TERM, assert_int_equal, cell_tables_equal, compare_step, rel_err

pytestmark = pytest.mark.gpu

FLUID, OFF, GRID, R = (16, 32, 1), 1, (64, 64, 4), 1.0 / 256


def _dambreak():
    s = cm.DamBreakSystem(FLUID, OFF, GRID, R)
    s.reset()
    ref = O.OracleState(O.dambreak_params(FLUID, OFF, GRID, R), s.getNumParticles())
    return s, ref.reset_reference()


def _poiseuille():
    kw = presets.poiseuille_dump(16, 64, 3)
    args = (kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    s = cm.PoiseuilleFlowSystem(*args)
    s.reset()
    ref = O.OracleState(O.poiseuille_params(*args), s.getNumParticles())
    return s, ref.reset_reference()


def _set_mode(s, mode):
    if mode == "lists":
        s.set_groups(1, 1)
        s.set_neighbor_lists(True)
    else:
        lanes = int(mode[-1])
        s.set_groups(lanes, lanes)
        s.set_neighbor_lists(False)


def _stages_bit_exact(s, ref, label):
    s.load_state(ref)
    s.run_stages(_abi.STAGE_REORDER)
    r = O.OracleState(ref.p, ref.n).set_state(ref)
    r.step(stop_after=_abi.STAGE_REORDER)
    assert_int_equal(s.getUintArray(_abi.HASH), r.hash, label + "sorted hash")
    assert_int_equal(s.getUintArray(_abi.INDEX), r.idx, label + "sorted index")
    cell_tables_equal(s.getUintArray(_abi.CELLSTART), s.getUintArray(_abi.CELLEND),
                      r.cell_start, r.cell_end)
    assert_int_equal(s.getArray(cm.SORTEDPOSITION).view(np.uint32), r.spos.view(np.uint32),
                     label + "sortedPos")
    return r


def _one_step(s, ref):
    s.load_state(ref)
    pre = O.OracleState(ref.p, ref.n).set_state(ref)
    nxt = O.OracleState(ref.p, ref.n).set_state(ref)
    s.update()
    nxt.step()
    return s.state(), pre, nxt


@pytest.mark.parametrize("mode", ["walk1", "walk2", "lists"])
def test_dambreak_particles_outside_the_grid(gpu, mode):
    s, ref = _dambreak()
    _set_mode(s, mode)
    p = ref.p
    ox, oy = float(p.world_origin[0]), float(p.world_origin[1])
    cs = float(p.cell_size[0])
    wx, wy = GRID[0] * cs, GRID[1] * cs
    fluid = np.flatnonzero(ref.pos[:, 3] == _abi.FLUID)
    k = fluid[[3, 40, 77, 120, 200, 260, 300]]
    y_mid = oy + 20.5 * cs
    places = [(ox - 2.5 * cs, y_mid),                # left of the grid: cells wrap to the right edge
              (ox - 3.4 * cs, y_mid),                # ... and a neighbour of it
              (ox - 2.5 * cs, y_mid + 0.8 * cs),     # ... and another
              (ox + wx + 1.5 * cs, y_mid),           # right of the grid
              (ox + 5.5 * cs, oy + 2.3 * wy),        # more than two periods above
              (ox + 7.5 * cs, oy - 1.2 * wy),        # more than one period below
              (ox - 1.7 * wx, oy + 30.5 * cs)]       # more than one period to the left
    for j, (x, y) in zip(k, places):
        ref.pos[j, 0] = np.float32(x)
        ref.pos[j, 1] = np.float32(y)
    _stages_bit_exact(s, ref, "outside (%s): " % mode)
    g, pre, nxt = _one_step(s, ref)
    print(mode, compare_step(g, pre, nxt, label="outside (%s): " % mode))
    s.close()


def test_poiseuille_particle_above_the_grid(gpu):
    """A Poiseuille particle past the top of the grid: its cell wraps in y (no image
    shift in y), while its x neighbours still carry the periodic x shift."""
    s, ref = _poiseuille()
    p = ref.p
    cs = 2.0 * float(p.particle_radius)
    top = float(p.world_origin[1]) + int(p.grid_size[1]) * cs
    fluid = np.flatnonzero(ref.pos[:, 3] != 1.0)  # Poiseuille walls have w = 1
    # a fluid particle at the x edge, lifted past the top of the grid
    j = fluid[np.argmin(ref.pos[fluid, 0])]
    ref.pos[j, 1] = np.float32(top + 1.5 * cs)
    _stages_bit_exact(s, ref, "poiseuille above: ")
    g, pre, nxt = _one_step(s, ref)
    print(compare_step(g, pre, nxt, label="poiseuille above: "))
    s.close()


def test_coincident_particles(gpu):
    s, ref = _dambreak()
    for _ in range(2):
        ref.step()
    fluid = np.flatnonzero(ref.pos[:, 3] == _abi.FLUID)
    groups = [fluid[[10, 11]], fluid[[100, 140]], fluid[[205, 206, 207]], fluid[[300, 20]]]
    for grp in groups:
        for j in grp[1:]:
            ref.pos[j, :3] = ref.pos[grp[0], :3]
    coincident = np.concatenate([grp for grp in groups])
    r = _stages_bit_exact(s, ref, "coincident: ")
    # equal keys keep index order: each group sits in one cell, ascending
    where = np.argsort(r.idx)
    for grp in groups:
        pos_in_sort = np.sort(where[grp])
        assert np.array_equal(r.idx[pos_in_sort], np.sort(grp))
        assert len(set(r.hash[pos_in_sort])) == 1
    g, pre, nxt = _one_step(s, ref)
    assert_int_equal(g["hash"], nxt.hash, "hash")
    assert_int_equal(g["idx"], nxt.idx, "index")
    assert rel_err(g["meas"][:, 0], nxt.meas[:, 0], float(ref.p.rest_density)) <= TOL_RHO
    a, _, sa, _ = nxt.forces_on(g["meas"], spos=g["spos"])
    assert np.isfinite(g["acc"][:, :3]).all() and np.isfinite(g["pos"][:, :3]).all()
    nan_rows = ~np.isfinite(a[:, :3]).all(axis=1)
    # the reference's NaN appears exactly at the coincident fluid particles
    # (forces in original particle order)
    assert set(np.flatnonzero(nan_rows).tolist()) == set(coincident.tolist())
    ok = ~nan_rows
    err = np.abs(g["acc"][ok, :3].astype(np.float64) - a[ok, :3]) / (sa[ok, :3].astype(np.float64) + 1e-30)
    assert err.max() <= TOL_TERM, err.max()
    s.close()


@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_scenes(gpu, n):
    """One fluid particle alone, a fluid pair, a fluid pair with a wall particle."""
    p = O.dambreak_params(FLUID, OFF, GRID, R)
    cs = float(p.cell_size[0])
    ox, oy, oz = (float(p.world_origin[a]) for a in range(3))
    ref = O.OracleState(p, n)
    fl, wall = float(_abi.FLUID), float(_abi.FIRST_TYPE)
    pts = [(ox + 20.5 * cs, oy + 30.25 * cs, fl), (ox + 21.75 * cs, oy + 30.5 * cs, fl),
           (ox + 21.0 * cs, oy + 29.0 * cs, wall)][:n]
    z = oz + 2.5 * cs
    for j, (x, y, w) in enumerate(pts):
        ref.pos[j] = (x, y, z, w)
    ref.meas[:, 0] = p.rest_density
    s = cm.DamBreakSystem(params=p, num_particles=n)
    _stages_bit_exact(s, ref, "n=%d: " % n)
    g, pre, nxt = _one_step(s, ref)
    print(n, compare_step(g, pre, nxt, label="n=%d: " % n))
    s.close()


def test_multi_array_transfer_equals_single_arrays(gpu):
    """setArrays / getArrays (one synchronisation for several arrays) leave the
    solver in the state the per-array calls leave: the same trajectory bit for
    bit, and a z velocity uploaded with the positions still switches a 2-D scene
    off its single-layer search."""
    a, _ = _dambreak()
    b, _ = _dambreak()
    for s in (a, b):
        s.removeRightBoundary()
        s.update_n(20)
    ids = (cm.POSITION, cm.VELOCITY, cm.VELOCITYLEAPFROG)
    host = {k: a.getArray(k) for k in ids}
    got = b.getArrays({k: None for k in ids})
    for k in ids:
        assert np.array_equal(got[k].view(np.uint32), host[k].view(np.uint32))
    # a small z velocity on one fluid particle: both must take the 3-D walk
    host[cm.VELOCITY][5, 2] = 1e-3
    for k in ids:
        a.setArray(k, host[k])
    b.setArrays(host)
    for s in (a, b):
        s.update()
    # the 3-D walk scans the whole grid: its dense cell offsets cover every cell
    # (a single-layer scan window holds one z layer of them)
    for s in (a, b):
        assert len(s.getUintArray(_abi.CELLOFFSET, count=s.numGridCells + 1)) == s.numGridCells + 1
    for s in (a, b):
        s.update_n(4)
    got = b.getArrays({k: None for k in ids})
    for k in ids:
        assert np.array_equal(got[k].view(np.uint32), a.getArray(k).view(np.uint32)), k
    with pytest.raises(Exception):
        b.setArrays({cm.POSITION: host[cm.POSITION][:-1]})
    a.close()
    b.close()
