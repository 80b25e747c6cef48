"""Batched scenes vs the same scenes run alone.

A batch runs every scene with the single-scene kernels' arithmetic (same
parameters, same lanes per particle, same neighbour order), so each scene of a
batch must equal a cmag_system with the same parameters bit for bit: the hash,
sort and cell tables (scene-local), densities, forces and the integrated state
after many steps.  The single-scene solver itself is checked against the oracle
in test_gpu_parity.py."""
import ctypes

import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from cmag_gb300._lib import c_f32p, check, lib
from cmag_gb300.batch import Batch
from cmag_gb300.systems import DamBreakSystem, PeristalsisSystem, PoiseuilleFlowSystem

from helpers import assert_int_equal

pytestmark = pytest.mark.gpu

F4 = [cm.POSITION, cm.VELOCITY, cm.VELOCITYLEAPFROG, cm.MEASURES, cm.ACCELERATION]


def _peristalsis_params():
    kw = presets.peristalsis_report()
    kw.update(fluid_size=(64, 26, 1), grid_size=(64, 64, 4))
    kw["amplitude"] = 5 * kw["radius"]
    return presets.peristalsis_params(kw["dt"], kw["fluid_size"], kw["amplitude"], kw["wave_speed"],
                                      kw["soundspeed"], kw["gravity"], kw["boundary_offset"],
                                      kw["grid_size"], kw["radius"])


def _dambreak3d_state():
    p, n, tank, L = presets.dambreak3d(fluid=(12, 24, 10), tank=(40, 32, 12), layers=3)
    pos = np.zeros((n, 4), np.float32)
    check(lib().cmag_dambreak3d_scene_host(ctypes.byref(p), _abi.u3(tank), L, 0.01, 1973,
                                           pos.ctypes.data_as(c_f32p), n))
    return p, n, pos


def mixed_scenes():
    """Families interleaved (the batch regroups them), power-of-two and tight
    grids, one 3-D scene.  Returns [(params, count, positions or None)]."""
    out = []
    kw = presets.poiseuille_dump(16, 64, 3)
    out.append(presets.poiseuille_params(kw["fluid_size"], 3, kw["grid_size"], kw["radius"]))
    out.append(presets.dambreak_params((16, 32, 1), 1, (64, 64, 4), 1.0 / 256))
    out.append(_peristalsis_params())
    p3, n3, pos3 = _dambreak3d_state()
    out.append(p3)
    kw = presets.poiseuille_dump(24, 48, 3)
    p = presets.poiseuille_params(kw["fluid_size"], 3, (24, 54, 4), kw["radius"])
    p.mu = np.float32(2e-3)
    out.append(p)
    out.append(presets.dambreak_params((24, 40, 1), 1, (96, 80, 4), 1.0 / 256))
    scenes = []
    for k, p in enumerate(out):
        if k == 3:
            scenes.append((p, n3, pos3))
        else:
            scenes.append((p, presets.reference_count(p), None))
    return scenes


def single_for(p, n):
    cls = {_abi.DAMBREAK: DamBreakSystem, _abi.POISEUILLE: PoiseuilleFlowSystem,
           _abi.PERISTALSIS: PeristalsisSystem}[p.system]
    return cls(params=p, num_particles=n)


def load_scene(batch, k, single, p, n, pos):
    """The scene's initial state in the batch and in its single-scene twin."""
    if pos is None:
        batch.reset(k)
        single.reset()
    else:
        meas = np.zeros((n, 4), np.float32)
        meas[:, 0] = p.rest_density
        zero = np.zeros((n, 4), np.float32)
        for s_set in (lambda a, d: batch.set_array(k, a, d), lambda a, d: single.setArray(a, d)):
            s_set(cm.POSITION, pos)
            s_set(cm.MEASURES, meas)
            for a in (cm.VELOCITY, cm.VELOCITYLEAPFROG, cm.ACCELERATION):
                s_set(a, zero)


def build_pair(scenes=None):
    scenes = scenes or mixed_scenes()
    batch = Batch([s[0] for s in scenes], [s[1] for s in scenes])
    singles = []
    for k, (p, n, pos) in enumerate(scenes):
        s = single_for(p, n)
        load_scene(batch, k, s, p, n, pos)
        singles.append(s)
    # same lanes per particle as each scene's launch group
    for k, s in enumerate(singles):
        g = batch.groups()[batch.scene_group(k)]
        s.set_groups(g["density_lanes"], g["force_lanes"])
    return batch, singles, scenes


def assert_scene_equal(batch, k, single, arrays=F4, what=""):
    for a in arrays:
        got = batch.get_array(k, a)
        want = single.getArray(a)
        assert_int_equal(got.view(np.uint32), want.view(np.uint32), "scene %d array %d %s" % (k, a, what))


def test_batch_layout_and_groups(gpu):
    batch, singles, scenes = build_pair()
    assert batch.num_particles == sum(s[1] for s in scenes)
    ranges = [batch.scene_range(k) for k in range(len(scenes))]
    # scenes tile the particle arrays without gaps, grouped by family
    spans = sorted(ranges)
    pos = 0
    for a, n in spans:
        assert a == pos
        pos += n
    groups = batch.groups()
    assert sum(g["scenes"] for g in groups) == len(scenes)
    assert sum(g["particles"] for g in groups) == batch.num_particles
    fam = [g["system"] for g in groups]
    assert fam == sorted(fam)
    g3 = groups[batch.scene_group(3)]
    assert g3["planar"] == 0 and g3["system"] == _abi.DAMBREAK
    for k in (0, 1, 2, 4, 5):
        assert groups[batch.scene_group(k)]["planar"] == 1
    for k in range(len(scenes)):
        assert_scene_equal(batch, k, singles[k], what="after load")
    batch.close()


def test_batch_stages_bit_exact(gpu):
    """hash, sort, cell tables, gathers, densities and forces of one step."""
    batch, singles, scenes = build_pair()
    batch.run_stages(_abi.STAGE_FORCE)
    for s in singles:
        s.run_stages(_abi.STAGE_FORCE)
    for k, s in enumerate(singles):
        n = scenes[k][1]
        for a in (_abi.HASH, _abi.INDEX):
            assert_int_equal(batch.get_uint_array(k, a), s.getUintArray(a), "scene %d uint %d" % (k, a))
        for a in (_abi.CELLSTART, _abi.CELLEND):
            assert_int_equal(batch.get_uint_array(k, a), s.getUintArray(a), "scene %d cells %d" % (k, a))
        arrays = [cm.SORTEDPOSITION, cm.SORTEDVELOCITY, cm.MEASURES]
        arrays += [cm.VISCOUSFORCE, cm.PRESSUREFORCE] if scenes[k][0].system == _abi.PERISTALSIS else [cm.ACCELERATION]
        assert_scene_equal(batch, k, s, arrays, "stages")
        assert n == s.getNumParticles()
    assert batch.device_error_bits() == 0
    batch.close()


@pytest.mark.parametrize("graphs,steps_per_graph", [(False, 1), (True, 1), (True, 4)])
def test_batch_trajectory_bit_exact(gpu, graphs, steps_per_graph):
    """30 steps: every scene's state equals its twin's, eager or graph-replayed
    (several steps per graph included)."""
    batch, singles, scenes = build_pair()
    batch.set_graphs(graphs, steps_per_graph)
    # dam breaks released part-way, as the Report harnesses do
    batch.update_n(10)
    for s in singles:
        s.update_n(10)
    for k, (p, _, pos) in enumerate(scenes):
        if p.system == _abi.DAMBREAK and pos is None:
            batch.dambreak_remove_right_boundary(k)
            singles[k].removeRightBoundary()
    batch.update_n(20)
    for s in singles:
        s.update_n(20)
    batch.synchronize()
    for k, s in enumerate(singles):
        assert_scene_equal(batch, k, s, what="after 30 steps")
        assert batch.elapsed_time(k) == s.getElapsedTime()
    lo, hi = batch.fluid_extents()
    for k, s in enumerate(singles):
        slo, shi = s.fluid_extent()
        assert np.array_equal(lo[k], slo) and np.array_equal(hi[k], shi), k
    batch.close()


def test_batch_autotuned_lanes(gpu):
    """After autotuning, with the twins on the tuned lanes, trajectories still agree."""
    batch, singles, scenes = build_pair()
    batch.update_n(2)
    batch.autotune(2)
    for g in batch.groups():
        assert g["density_lanes"] in (1, 2, 4) and g["force_lanes"] in (1, 2, 4)
    # restart both from the initial state on the tuned lanes
    for k, (p, n, pos) in enumerate(scenes):
        load_scene(batch, k, singles[k], p, n, pos)
        g = batch.groups()[batch.scene_group(k)]
        singles[k].set_groups(g["density_lanes"], g["force_lanes"])
    batch.update_n(8)
    for s in singles:
        s.update_n(8)
    for k, s in enumerate(singles):
        assert_scene_equal(batch, k, s, what="tuned lanes")
    batch.close()


def test_batch_interaction_lists_bit_exact(gpu):
    """Every launch group on interaction lists: each scene equals its twin on the
    one-lane cell walk after 20 graph-replayed steps (dam breaks released part-way)."""
    batch, singles, scenes = build_pair()
    for gi in range(len(batch.groups())):
        batch.set_group_lists(gi, True)
    for g in batch.groups():
        assert g["lists"] == 1 and g["density_lanes"] == 1 and g["force_lanes"] == 1
    for s in singles:
        s.set_groups(1, 1)
    batch.set_graphs(True, 4)
    batch.update_n(8)
    for s in singles:
        s.update_n(8)
    for k, (p, _, pos) in enumerate(scenes):
        if p.system == _abi.DAMBREAK and pos is None:
            batch.dambreak_remove_right_boundary(k)
            singles[k].removeRightBoundary()
    batch.update_n(12)
    for s in singles:
        s.update_n(12)
    batch.synchronize()
    for k, s in enumerate(singles):
        assert_scene_equal(batch, k, s, what="lists")
    assert batch.device_error_bits() == 0
    # back to the walk
    batch.set_group_lists(0, False)
    assert batch.groups()[0]["lists"] == 0
    batch.close()


def test_batch_whole_arrays(gpu):
    """set_array_all / get_array_all move every scene's rows (scene order) and agree
    with the per-scene calls; a planar scene's z is checked on the device."""
    batch, singles, scenes = build_pair()
    batch.update_n(3)
    n = batch.num_particles
    for a in (cm.POSITION, cm.VELOCITY, cm.VELOCITYLEAPFROG, cm.ACCELERATION):
        whole = batch.get_array_all(a)
        per = np.concatenate([batch.get_array(k, a) for k in range(len(scenes))])
        assert whole.shape == (n, 4) and np.array_equal(whole.view(np.uint32), per.view(np.uint32))
    # round trip through the whole-batch upload
    pos = batch.get_array_all(cm.POSITION)
    vel = batch.get_array_all(cm.VELOCITY)
    batch.set_array_all(cm.POSITION, pos)
    batch.set_array_all(cm.VELOCITY, vel)
    assert np.array_equal(batch.get_array_all(cm.POSITION), pos)
    # a planar scene's particle off its z layer, or with a z velocity: rejected
    first = sum(s[1] for s in scenes[:1])  # scene 1 (planar dam break) starts here
    bad = pos.copy()
    bad[first + 5, 2] += 0.01
    with pytest.raises(cm.CmagError):
        batch.set_array_all(cm.POSITION, bad)
    batch.set_array_all(cm.POSITION, pos)
    badv = vel.copy()
    badv[first + 5, 2] = 1.0
    with pytest.raises(cm.CmagError):
        batch.set_array_all(cm.VELOCITY, badv)
    batch.set_array_all(cm.VELOCITY, vel)
    batch.update_n(2)
    assert np.isfinite(batch.get_array_all(cm.POSITION)).all()
    batch.close()


def test_batch_set_params_and_planar_checks(gpu):
    scenes = mixed_scenes()
    batch = Batch([s[0] for s in scenes], [s[1] for s in scenes])
    p = batch.params(0)
    p.gravity[0] = np.float32(2e-4)
    batch.set_params(0, p)
    assert batch.params(0).gravity[0] == np.float32(2e-4)
    bad = batch.params(0)
    bad.grid_size[0] = 32
    with pytest.raises(cm.CmagError):
        batch.set_params(0, bad)
    # a planar 2-D scene keeps one z layer
    n = scenes[1][1]
    pos = np.zeros((n, 4), np.float32)
    pos[1, 2] = 0.01
    with pytest.raises(cm.CmagError):
        batch.set_array(1, cm.POSITION, pos)
    vel = np.zeros((n, 4), np.float32)
    vel[0, 2] = 1.0
    with pytest.raises(cm.CmagError):
        batch.set_array(1, cm.VELOCITY, vel)
    with pytest.raises(cm.CmagError):
        batch.scene_range(len(scenes))
    batch.close()


def test_batched_workload_runs(gpu):
    """A reduced copy of the benchmark's batch (16 scenes, counts up to 16k):
    every scene's twin agrees after a few graph-replayed steps, and the hash
    range check stays clean."""
    P, N, _, _ = presets.batched_scenes(scenes=16, seed=7, lo=2048, hi=16384)
    batch = Batch(P, N)
    singles = []
    for k, (p, n) in enumerate(zip(P, N)):
        s = single_for(p, n)
        batch.reset(k)
        s.reset()
        if p.system == _abi.DAMBREAK:
            batch.dambreak_remove_right_boundary(k)
            s.removeRightBoundary()
        singles.append(s)
    batch.set_graphs(True, 5)
    batch.update_n(10)
    for s in singles:
        s.update_n(10)
    batch.synchronize()
    for k, s in enumerate(singles):
        assert_scene_equal(batch, k, s, (cm.POSITION, cm.VELOCITY), "workload")
    batch.close()
