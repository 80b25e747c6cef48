"""Generate the golden fixtures from the reference's own kernels.

Runs the reference kernel sources compiled for the CPU (oracle/_ref, built from
the reference tree by oracle/ref/Makefile) on small seeded scenes of each family
and stores the state before and after one step.  Scenes and parameters come from
the reference constructors and reset() (restated, since the reference host
classes need OpenGL).  Run where the reference tree exists:

    python tests/golden/make_golden.py [scene ... | channel]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def scenes():
    r = 1.0 / (2 * 16 * 1000)
    yield "dambreak", O.dambreak_params((16, 32, 1), 1, (64, 64, 4), 1.0 / 256), 40, False
    yield "dambreak_off3", O.dambreak_params((12, 16, 1), 3, (32, 32, 4), 1.0 / 256), 25, False
    yield ("poiseuille", O.poiseuille_params((16, 26, 1), 3, (16, 32, 4), 1.0 / (2 * 26 * 1000)),
           30, False)
    p = O.peristalsis_params(1e-4, (32, 16, 1), 4 * r, 1e-2, 1e-4, (0.0, 0.0, 0.0), 3, (32, 32, 4), r)
    yield "peristalsis_config", p, 10, False
    yield "peristalsis_moving", p, 10, True


FIELDS = ("pos", "vel", "vlf", "meas", "acc", "vforce", "pforce")


def make(name, p, warm, release):
    n = O.particle_count(p)
    ref = O.RefState(p, n)
    ref.reset_reference()
    if release:  # skip the boundary-configuration phase: walls move from step 1
        ref.p.is_boundary_configuration = 0
    for _ in range(warm):
        ref.step()
    before = {k: getattr(ref, k).copy() for k in FIELDS}
    phase_before = ref.phase.copy()
    params_before = np.frombuffer(bytes(ref.p), np.uint8).copy()
    ref.step()
    out = {"params": params_before, "phase": phase_before, "n": np.array([n])}
    for k, v in before.items():
        out["in_" + k] = v
    for k in FIELDS + ("spos", "svel", "hash", "idx"):
        out["out_" + k] = getattr(ref, k).copy()
    occ = ref.cell_start != 0xFFFFFFFF
    out["out_cell_occupied"] = np.flatnonzero(occ).astype(np.uint32)
    out["out_cell_start"] = ref.cell_start[occ]
    out["out_cell_end"] = ref.cell_end[occ]
    out["out_phase"] = ref.phase.copy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return n


CHANNEL_TIMES = (0.0225, 0.045, 0.1125, 0.225)


def channel_profile():
    """Peristalsis.Report/poiseuille_velocity_profile.h:13-94 on the reference
    kernels: the Peristalsis solver with wall amplitude 0 and body force 1e-4 in
    x; leap-frog u_x and height above the lower wall of the fluid particles in the
    first column of cells at each report time (about 2,250 reference steps)."""
    off, sizex, c = 3, 64, 1e-4
    r = 1.0 / (2 * (sizex - 2 * off) * 1000)
    p = O.peristalsis_params(1e-4, (64, 58, 1), 0.0, 0.0, c, (1e-4, 0.0, 0.0), off, (64, 64, 4), r)
    n = O.particle_count(p)
    ref = O.RefState(p, n)
    ref.reset_reference()
    out = {"times": np.array(CHANNEL_TIMES)}
    bottom = np.float32(p.world_origin[1]) + np.float32(2 * r * off)
    for k, t in enumerate(CHANNEL_TIMES):
        while ref.elapsed < t:
            ref.step()
        pos = ref.pos
        m = (pos[:, 0] > 0) & (pos[:, 0] < 2 * r) & (pos[:, 1] > bottom) & (pos[:, 1] < bottom + 58 * 2 * r)
        y = pos[m, 1] - np.float32(p.world_origin[1]) - np.float32(off * 2 * r)
        order = np.argsort(y)
        out["y%d" % k] = y[order].astype(np.float32)
        out["u%d" % k] = ref.vlf[m, 0][order].astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "peristalsis_channel_profile.npz"), **out)
    return n


if __name__ == "__main__":
    if not O.ref_available():
        if not O.build_ref():
            sys.exit("the reference tree is needed to build oracle/_ref")
    only = sys.argv[1:]
    for name, p, warm, release in scenes():
        if only and name not in only:
            continue
        n = make(name, p, warm, release)
        print("%-20s %6d particles, step %d" % (name, n, warm + 1))
    if not only or "channel" in only:
        print("peristalsis channel profile: %d particles" % channel_profile())
