"""CUDA path vs the oracle, one step at a time from identical states.

For each family a small seeded scene is advanced by the oracle; at several
points of that trajectory the CUDA solver is loaded with the oracle's state and
both take one step.  Hash, sort, cell ranges and the sorted gathers must match
bit for bit; density, pressure, forces and the integrated state within the
tolerances in tests/helpers.py."""
import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from oracle import oracle as O

from helpers import assert_int_equal, cell_tables_equal, compare_step

pytestmark = pytest.mark.gpu


def _dambreak(fluid=(16, 32, 1), off=1, grid=(64, 64, 4), r=1.0 / 256):
    s = cm.DamBreakSystem(fluid, off, grid, r)
    s.reset()
    ref = O.OracleState(O.dambreak_params(fluid, off, grid, r), s.getNumParticles())
    return s, ref.reset_reference()


def _poiseuille(grid_x=16, grid_y=64, off=3):
    kw = presets.poiseuille_dump(grid_x, grid_y, off)
    s = cm.PoiseuilleFlowSystem(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    s.reset()
    ref = O.OracleState(O.poiseuille_params(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"],
                                            kw["radius"]), s.getNumParticles())
    return s, ref.reset_reference()


def _peristalsis(fluid=(64, 26, 1), grid=(64, 64, 4)):
    kw = presets.peristalsis_report()
    kw.update(fluid_size=fluid, grid_size=grid)
    kw["amplitude"] = 5 * kw["radius"]
    s = cm.PeristalsisSystem(kw["dt"], kw["fluid_size"], kw["amplitude"], kw["wave_speed"],
                             kw["soundspeed"], kw["gravity"], kw["boundary_offset"], kw["grid_size"],
                             kw["radius"])
    s.reset()
    p = O.peristalsis_params(kw["dt"], kw["fluid_size"], kw["amplitude"], kw["wave_speed"],
                             kw["soundspeed"], kw["gravity"], kw["boundary_offset"], kw["grid_size"],
                             kw["radius"])
    ref = O.OracleState(p, s.getNumParticles())
    return s, ref.reset_reference()


def _dambreak3d():
    p, n, tank, L = presets.dambreak3d(fluid=(12, 24, 10), tank=(40, 32, 12), layers=3)
    s = cm.DamBreakSystem(params=p, num_particles=n)
    s.scene3d(tank, L, 0.01, 1973)
    ref = O.OracleState(p, n)
    ref.pos[:] = O.dambreak3d_scene(p, tank, L, 0.01, 1973)
    ref.meas[:, 0] = p.rest_density
    return s, ref


SCENES = {"dambreak": _dambreak, "poiseuille": _poiseuille, "peristalsis": _peristalsis,
          "dambreak3d": _dambreak3d}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_reset_matches_oracle(gpu, name):
    s, ref = SCENES[name]()
    assert s.getNumParticles() == ref.n
    assert_int_equal(s.getArray(cm.POSITION).view(np.uint32), ref.pos.view(np.uint32), "positions")
    assert s.params.particle_mass == np.float32(ref.p.particle_mass)
    s.close()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_stages_bit_exact(gpu, name):
    """hash -> sort -> reorder outputs equal the oracle's exactly.  (Peristalsis runs
    released: during the configuration phase configureBoundary moves the walls with
    sinf before the hash, and the GPU's sinf may differ from the host's by an ulp;
    the wall law is checked with a tolerance in test_peristalsis_phase_machine.)"""
    s, ref = SCENES[name]()
    if name == "peristalsis":
        ref.p.is_boundary_configuration = 0
    for _ in range(3):
        ref.step()
    s.load_state(ref)
    s.run_stages(_abi.STAGE_HASH)
    r = O.OracleState(ref.p, ref.n).set_state(ref)
    r.step(stop_after=_abi.STAGE_HASH)
    assert_int_equal(s.getUintArray(_abi.HASH), r.hash, "hash (unsorted)")
    s.load_state(ref)
    s.run_stages(_abi.STAGE_REORDER)
    r = O.OracleState(ref.p, ref.n).set_state(ref)
    r.step(stop_after=_abi.STAGE_REORDER)
    assert_int_equal(s.getUintArray(_abi.HASH), r.hash, "sorted hash")
    assert_int_equal(s.getUintArray(_abi.INDEX), r.idx, "sorted index")
    cell_tables_equal(s.getUintArray(_abi.CELLSTART), s.getUintArray(_abi.CELLEND),
                      r.cell_start, r.cell_end)
    assert_int_equal(s.getArray(cm.SORTEDPOSITION).view(np.uint32), r.spos.view(np.uint32), "sortedPos")
    s.synchronize()
    s.close()


@pytest.mark.parametrize("lanes", [1, 2, 4])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_one_step_along_trajectory(gpu, name, lanes):
    """At several points of an oracle trajectory, one GPU step equals one oracle step."""
    s, ref = SCENES[name]()
    s.set_groups(lanes, lanes)
    checkpoints = {0, 5, 20}
    errs = []
    for k in range(21):
        if k in checkpoints:
            s.load_state(ref)
            pre = O.OracleState(ref.p, ref.n).set_state(ref)
            nxt = O.OracleState(ref.p, ref.n).set_state(ref)
            s.update()
            nxt.step()
            errs.append(compare_step(s.state(), pre, nxt, label="%s step %d: " % (name, k)))
        ref.step()
    s.synchronize()
    s.close()
    print(name, errs)


def test_peristalsis_moving_walls_step(gpu):
    """One step with the walls in motion (after the configuration phase)."""
    s, ref = _peristalsis()
    ref.p.is_boundary_configuration = 0
    for _ in range(12):
        ref.step()
    s.load_state(ref)
    pre = O.OracleState(ref.p, ref.n).set_state(ref)
    ref.step()
    s.update()
    compare_step(s.state(), pre, ref, label="peristalsis moving: ")
    s.close()


def test_peristalsis_noslip_walls_step(gpu):
    """The no-slip extrapolation into the moving walls (wall_noslip = 1, an option
    of this build): one step with the walls in motion against the oracle's
    restatement (wall distance by Newton's method, wall velocity from the law)."""
    s, ref = _peristalsis()
    ref.p.is_boundary_configuration = 0
    ref.p.wall_noslip = 1
    sp = s.params
    sp.wall_noslip = 1
    s.set_params(sp)
    for _ in range(12):
        ref.step()
    s.load_state(ref)
    pre = O.OracleState(ref.p, ref.n).set_state(ref)
    plain = O.OracleState(ref.p, ref.n).set_state(ref)
    plain.p.wall_noslip = 0
    plain.step()
    ref.step()
    s.update()
    out = compare_step(s.state(), pre, ref, label="peristalsis no-slip: ")
    # the option changes the viscous force next to the walls and nowhere else
    d = np.abs(ref.vforce[:, :2] - plain.vforce[:, :2]).max(axis=1)
    near = d > 0
    assert near.any() and (~near).any()
    print("no-slip step:", out, "particles changed:", int(near.sum()))
    s.close()


@pytest.mark.parametrize("cap", [None, 40, 4])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_interaction_lists_equal_the_walk(gpu, name, cap):
    """With interaction lists the force pass reads the pairs the density pass
    recorded: 15 steps give the one-lane walk's state bit for bit, also when some
    (cap 40) or all (cap 4) particles overflow their list and walk the cells."""
    s1, _ = SCENES[name]()
    s2, _ = SCENES[name]()
    s1.set_groups(1, 1)
    s2.set_groups(1, 1)
    s2.set_neighbor_lists(True, cap)
    assert s2.neighbor_lists()[0]
    s1.update_n(15)
    s2.update_n(15)
    s2.synchronize()
    for a in (cm.POSITION, cm.VELOCITY, cm.MEASURES):
        assert_int_equal(s2.getArray(a).view(np.uint32), s1.getArray(a).view(np.uint32), "%s array %d" % (name, a))
    s2.set_neighbor_lists(False)
    assert not s2.neighbor_lists()[0]
    s1.close()
    s2.close()


@pytest.mark.parametrize("name", ["dambreak", "peristalsis"])
def test_state_round_trip_through_host_buffers(gpu, name):
    """A planar scene reloaded through setArray (whose z checks run on the device)
    keeps its one-layer search: it steps bit for bit like its twin; getArray fills a
    caller buffer with the same rows it returns."""
    s1, _ = SCENES[name]()
    s2, _ = SCENES[name]()
    s1.set_groups(1, 1)
    s2.set_groups(1, 1)
    s1.update_n(3)
    s2.update_n(3)
    s2.load_state(s1.state())
    s2.set_elapsed_time(s1.getElapsedTime())
    s1.update_n(5)
    s2.update_n(5)
    for a in (cm.POSITION, cm.VELOCITY, cm.MEASURES):
        assert_int_equal(s2.getArray(a).view(np.uint32), s1.getArray(a).view(np.uint32), "%s array %d" % (name, a))
    buf = np.full((s1.getNumParticles(), 4), np.nan, np.float32)
    out = s1.getArray(cm.POSITION, out=buf)
    assert out is buf and np.array_equal(buf, s1.getArray(cm.POSITION))
    with pytest.raises(ValueError):
        s1.getArray(cm.POSITION, out=np.zeros((3, 4), np.float32))
    s1.close()
    s2.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_graph_replay_equals_plain_launches(gpu, graphs):
    """A captured-and-replayed step produces the same bits as plain launches."""
    a, ref = _dambreak()
    b, _ = _dambreak()
    a.set_graphs(True)
    b.set_graphs(graphs)
    a.reset()
    b.reset()
    a.update_n(10)
    for _ in range(10):
        b.update()
    for arr in (cm.POSITION, cm.VELOCITY, cm.MEASURES):
        assert_int_equal(a.getArray(arr).view(np.uint32), b.getArray(arr).view(np.uint32), "array %d" % arr)
    assert a.getElapsedTime() == b.getElapsedTime()
    a.close()
    b.close()


def test_multi_step_short_horizon(gpu):
    """10 steps of free evolution stay within a short-horizon bound of the oracle."""
    s, ref = _dambreak()
    s.reset()
    for _ in range(10):
        s.update()
        ref.step()
    got = s.getArray(cm.POSITION)
    dx = 2 * ref.p.particle_radius
    assert np.abs(got[:, :3] - ref.pos[:, :3]).max() / dx < 1e-4
    assert s.getElapsedTime() == np.float32(ref.phase[0])
    s.close()


def test_peristalsis_phase_machine(gpu):
    """Boundary-configuration ramp, relax and release follow PeristalsisSystem::Update."""
    s, ref = _peristalsis(fluid=(32, 16, 1), grid=(32, 32, 4))
    p = ref.p
    p.amplitude = np.float32(3e-10)  # 3 ramp steps at dt*1e-3 per step
    ref.p = p
    s.set_params(p)
    s.reset()
    ref.reset_reference()
    for k in range(1010):
        s.update()
        ref.step()
    ph = s.phase()
    assert ph["is_boundary_configuration"] == ref.p.is_boundary_configuration
    assert np.float32(ph["time_shift"]) == ref.phase[1]
    assert np.float32(ph["current_wave_height"]) == ref.phase[3]
    got = s.getArray(cm.POSITION)
    walls = ref.pos[:, 3] != 0
    assert np.abs(got[walls, 1] - ref.pos[walls, 1]).max() < 1e-4 * ref.p.particle_radius
    s.close()
