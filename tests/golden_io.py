"""Load the golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py
from the reference's own kernels) into oracle states."""
import glob
import os

import numpy as np

from cmag_gb300._abi import SphParams

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# one-step fixtures (the channel profile fixture has its own test)
NAMES = sorted(os.path.splitext(os.path.basename(f))[0] for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not f.endswith("_profile.npz"))
IN_FIELDS = ("pos", "vel", "vlf", "meas", "acc", "vforce", "pforce")


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = SphParams.from_buffer_copy(d["params"].tobytes())
    return p, d


def oracle_input(name):
    """Oracle state loaded with the fixture's pre-step state."""
    from oracle import oracle as O
    p, d = load(name)
    st = O.OracleState(p, int(d["n"][0]))
    for k in IN_FIELDS:
        getattr(st, k)[:] = d["in_" + k]
    st.phase[:4] = d["phase"][:4]
    return st, d
