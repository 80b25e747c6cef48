"""CUDA path vs the oracle at the sizes bench.py times.

One step from an identical state, compared stage by stage with the tolerances
of tests/helpers.py (hash, index, cell order and the sorted gathers bit for bit;
density, pressure, forces and the integrated state within their bounds):

  * 3-D dam break, 64x128x64 fluid + 3-layer walls (954,860 particles), at t = 0
    and from a developed flow (the GPU's own state after 2000 steps, t = 0.1 s,
    surge front well into the tank), with interaction lists at their default
    capacity and with the cell walk;
  * 2-D peristaltic channel, 2048x512 fluid + moving walls (1,060,864
    particles), released, at t = 0 and after 200 steps;
  * 2-D Poiseuille, exactly 64x64 fluid + 3 wall rows each side (4,480
    particles), with the reference's physics and with the cubic-spline / Tait
    option, along an oracle trajectory;
  * the 256-scene batch: the smallest, median and largest scene of each family,
    stepping inside the batch, against the oracle run on that scene alone.

The oracle's force recomputation runs on all host cores; every case finishes in
well under a minute.
"""
import os

import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi, presets
from cmag_gb300.batch import Batch
from oracle import oracle as O

from helpers import compare_step

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def oracle_from(s):
    """An oracle state holding a solver's current arrays, parameters and time."""
    st = s.state()
    ref = O.OracleState(s.params, s.getNumParticles())
    for k in ("pos", "vel", "vlf", "meas", "acc", "vforce", "pforce"):
        if k in st:
            getattr(ref, k)[:] = st[k]
    ref.phase[0] = s.getElapsedTime()
    if ref.p.system == _abi.PERISTALSIS:
        ph = s.phase()
        ref.phase[1] = ph["time_shift"]
        ref.phase[2] = ph["time_relax"]
        ref.phase[3] = ph["current_wave_height"]
    return ref


def one_step(s, ref, label):
    """Load `ref` into the solver, step both once and compare."""
    s.load_state(ref)
    pre = O.OracleState(ref.p, ref.n).set_state(ref)
    post = O.OracleState(ref.p, ref.n).set_state(ref)
    s.update()
    post.step(threads=THREADS)
    s.synchronize()
    return compare_step(s.state(), pre, post, label=label, threads=THREADS)


# ---------------------------------------------------------------- dam break --

def dambreak3d_full():
    p, n, tank, L = presets.dambreak3d()
    s = cm.DamBreakSystem(params=p, num_particles=n)
    s.scene3d(tank, L, 0.01, 1973)
    return s, p, n


@pytest.mark.parametrize("lists", [True, False], ids=["lists", "walk"])
def test_dambreak3d_full_size_t0(gpu, lists):
    s, p, n = dambreak3d_full()
    assert n == 954_860
    s.set_groups(1, 1)
    s.set_neighbor_lists(lists)
    ref = oracle_from(s)
    err = one_step(s, ref, "dambreak3d t=0 %s: " % ("lists" if lists else "walk"))
    print("dambreak3d t=0", err)
    s.close()


@pytest.mark.parametrize("lists", [True, False], ids=["lists", "walk"])
def test_dambreak3d_full_size_developed(gpu, lists):
    """After 2000 steps (t = 0.1 s) the surge has left the column: lists near
    the front hold the most entries, and particles pile against the walls."""
    s, p, n = dambreak3d_full()
    s.set_neighbor_lists(True)
    s.update_n(2000)
    lo, hi = s.fluid_extent()
    assert hi[0] > 0.6, "surge front %g m: the flow has not developed" % hi[0]
    s.set_groups(1, 1)
    s.set_neighbor_lists(lists)
    ref = oracle_from(s)
    err = one_step(s, ref, "dambreak3d t=0.1 %s: " % ("lists" if lists else "walk"))
    print("dambreak3d t=0.1", err)
    s.close()


# -------------------------------------------------------------- peristalsis --

def test_peristalsis_full_size(gpu):
    p = presets.peristalsis_c3()
    s = cm.PeristalsisSystem(params=p)
    s.reset()
    assert s.getNumParticles() == 1_060_864
    # released (the reference's configuration ramp runs 1.5 s of simulated time)
    q = s.params
    q.is_boundary_configuration = 0
    s.set_params(q)
    s.set_groups(1, 1)
    s.set_neighbor_lists(True)
    for steps, label in ((0, "t=0"), (200, "200 steps")):
        s.update_n(steps)
        ref = oracle_from(s)
        err = one_step(s, ref, "peristalsis %s: " % label)
        print("peristalsis", label, err)
    s.close()


# --------------------------------------------------------------- poiseuille --

@pytest.mark.parametrize("reference_physics", [True, False], ids=["reference", "spline_tait"])
def test_poiseuille_64x64(gpu, reference_physics):
    p = presets.poiseuille_c1(reference_physics=reference_physics)
    assert tuple(p.fluid_size)[:2] == (64, 64)
    s = cm.PoiseuilleFlowSystem(params=p)
    s.reset()
    assert s.getNumParticles() == 4_480
    ref = O.OracleState(p, s.getNumParticles()).reset_reference()
    for k in range(201):
        if k in (0, 50, 200):
            err = one_step(s, ref, "poiseuille 64x64 step %d: " % k)
            print("poiseuille", reference_physics, k, err)
        ref.step(threads=THREADS)
    s.close()


# ------------------------------------------------------------------ batched --

def test_batched_scenes_against_oracle(gpu):
    """Each picked scene steps inside the full 256-scene batch (shared arrays,
    one sort for all scenes, per-group neighbour launches) and must equal the
    oracle run on that scene alone, from the same state after 20 batch steps."""
    P, N, F, D = presets.batched_scenes()
    b = Batch(P, N)
    for k, p in enumerate(P):
        b.reset(k)
        if p.system == _abi.DAMBREAK:
            b.dambreak_remove_right_boundary(k)
    b.autotune(2)
    b.update_n(20)
    picks = []
    for fam in ("poiseuille", "dambreak"):
        ks = sorted([k for k, d in enumerate(D) if d[0] == fam], key=lambda k: N[k])
        picks += sorted({ks[0], ks[len(ks) // 2], ks[-1]})
    names = {"pos": cm.POSITION, "vel": cm.VELOCITY, "vlf": cm.VELOCITYLEAPFROG,
             "meas": cm.MEASURES, "acc": cm.ACCELERATION}
    pre = {}
    for k in picks:
        ref = O.OracleState(b.params(k), N[k])
        for name, a in names.items():
            getattr(ref, name)[:] = b.get_array(k, a)
        ref.phase[0] = b.elapsed_time(k)
        pre[k] = ref
    b.update()
    b.synchronize()
    for k in picks:
        post = O.OracleState(pre[k].p, N[k]).set_state(pre[k]).step(threads=THREADS)
        got = {name: b.get_array(k, a) for name, a in names.items()}
        got["spos"] = b.get_array(k, cm.SORTEDPOSITION)
        got["svel"] = b.get_array(k, cm.SORTEDVELOCITY)
        got["hash"] = b.get_uint_array(k, _abi.HASH)
        got["idx"] = b.get_uint_array(k, _abi.INDEX)
        err = compare_step(got, pre[k], post, label="batch scene %d (%s, %d particles): " % (k, D[k][0], N[k]),
                           threads=THREADS)
        print("batch scene", k, D[k][0], N[k], err)
    b.close()
