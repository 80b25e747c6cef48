"""Generate the golden fixtures from the reference's own kernels.

Runs the reference kernel sources compiled for the CPU (oracle/_ref, built from
the reference tree by oracle/ref/Makefile) on small seeded scenes of each family
and stores the state before and after one step.  Scenes and parameters come from
the reference constructors and reset() (restated, since the reference host
classes need OpenGL).  Run where the reference tree exists:

    python tests/golden/make_golden.py
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


if __name__ == "__main__":
    if not O.ref_available():
        if not O.build_ref():
            sys.exit("the reference tree is needed to build oracle/_ref")
    for name, p, warm, release in scenes():
        n = make(name, p, warm, release)
        print("%-20s %6d particles, step %d" % (name, n, warm + 1))
