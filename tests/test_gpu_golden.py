"""CUDA path vs the golden fixtures made by the reference's own kernels: the
fixture's pre-step state is loaded through the C ABI, one step runs on the GPU,
and the result must equal the fixture (integer stages and gathers bit for bit,
floating point within the tolerances of tests/helpers.py, measured against the
oracle, which reproduces the fixture -- see test_oracle_golden.py)."""
import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import _abi

from golden_io import NAMES, oracle_input
from helpers import assert_int_equal, compare_step

pytestmark = pytest.mark.gpu

CLASSES = {_abi.DAMBREAK: cm.DamBreakSystem, _abi.POISEUILLE: cm.PoiseuilleFlowSystem,
           _abi.PERISTALSIS: cm.PeristalsisSystem}


@pytest.mark.parametrize("lanes", [1, 2, 4])
@pytest.mark.parametrize("name", NAMES)
def test_gpu_step_matches_golden(gpu, name, lanes):
    st, d = oracle_input(name)
    s = CLASSES[st.p.system](params=st.p, num_particles=st.n)
    s.set_groups(lanes, lanes)
    s.load_state(st)
    s.update()
    got = s.state()
    assert_int_equal(got["hash"], d["out_hash"], "hash")
    assert_int_equal(got["idx"], d["out_idx"], "index")
    cs = s.getUintArray(_abi.CELLSTART)
    ce = s.getUintArray(_abi.CELLEND)
    occ = d["out_cell_occupied"]
    assert_int_equal(np.flatnonzero(cs != 0xFFFFFFFF), occ, "occupied cells")
    assert_int_equal(cs[occ], d["out_cell_start"], "cellStart")
    assert_int_equal(ce[occ], d["out_cell_end"], "cellEnd")
    from oracle import oracle as O
    pre = O.OracleState(st.p, st.n).set_state(st)
    st.step()
    errs = compare_step(got, pre, st, label=name + ": ")
    assert np.float32(s.getElapsedTime()) == d["out_phase"][0]
    s.synchronize()
    s.close()
    print(name, errs)
