"""Pin the oracle: it must reproduce the golden fixtures made by the reference's
own kernels (integer stages, gathers and density bit for bit; forces to the
rounding of the reference host build, which evaluates pow(float, int) in double
where the GPU -- and the oracle -- evaluate it in float)."""
import numpy as np
import pytest

from golden_io import NAMES, oracle_input

FORCE_TOL = 1e-6  # of the per-particle term sum


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(built, name):
    st, d = oracle_input(name)
    st.cell_end[:] = 0
    st.step()
    for k in ("hash", "idx"):
        assert np.array_equal(getattr(st, k), d["out_" + k]), k
    occ = d["out_cell_occupied"]
    assert np.array_equal(np.flatnonzero(st.cell_start != 0xFFFFFFFF), occ)
    assert np.array_equal(st.cell_start[occ], d["out_cell_start"])
    assert np.array_equal(st.cell_end[occ], d["out_cell_end"])
    for k in ("spos", "svel", "meas"):
        assert np.array_equal(getattr(st, k).view(np.uint32), d["out_" + k].view(np.uint32)), k
    sa, sb = st.force_scale()
    forces = (("vforce", sa), ("pforce", sb)) if st.p.system == 2 else (("acc", sa),)
    total = np.zeros((st.n, 3))
    for k, sc in forces:
        err = np.abs(getattr(st, k)[:, :3].astype(np.float64) - d["out_" + k][:, :3])
        assert (err <= FORCE_TOL * sc[:, :3] + 1e-30).all(), k
        total += sc[:, :3]
    dt = float(st.p.delta_time)
    for k in ("vel", "vlf"):
        got, want = getattr(st, k)[:, :3].astype(np.float64), d["out_" + k][:, :3]
        bound = FORCE_TOL * total * dt + 2.4e-7 * np.abs(want) + 1e-30
        assert (np.abs(got - want) <= bound).all(), k
    got, want = st.pos[:, :3].astype(np.float64), d["out_pos"][:, :3]
    bound = FORCE_TOL * total * dt * dt + 1.2e-7 * np.abs(want) + 1e-30
    assert (np.abs(got - want) <= bound).all(), "pos"
    assert np.array_equal(st.phase[:4], d["out_phase"][:4])


def test_reference_kernels_match_oracle_stepwise(built):
    """Where the reference tree is present: oracle and the reference's kernels run
    side by side for several steps of each family."""
    from oracle import oracle as O
    if not O.ref_available():
        if not O.build_ref():
            pytest.skip("reference tree not present on this host")
    r = 1.0 / (2 * 16 * 1000)
    cases = [O.dambreak_params((16, 32, 1), 1, (64, 64, 4), 1.0 / 256),
             O.poiseuille_params((16, 16, 1), 3, (16, 32, 4), r),
             O.peristalsis_params(1e-4, (32, 16, 1), 5 * r, 1e-2, 1e-4, (0, 0, 0), 3, (32, 32, 4), r)]
    for p in cases:
        n = O.particle_count(p)
        a = O.OracleState(p, n).reset_reference()
        for _ in range(8):
            b = O.RefState(a.p, n).set_state(a)  # identical input state
            a.step()
            b.step()
            assert np.array_equal(a.hash, b.hash) and np.array_equal(a.idx, b.idx)
            assert np.array_equal(a.meas.view(np.uint32), b.meas.view(np.uint32))
            sa, sb = a.force_scale()
            for k, sc in (("acc", sa), ("vforce", sa), ("pforce", sb)):
                err = np.abs(getattr(a, k)[:, :3].astype(np.float64) - getattr(b, k)[:, :3])
                assert (err <= FORCE_TOL * sc[:, :3] + 1e-30).all(), k


def test_oracle_parameter_mirror_matches_the_product(built):
    """The oracle keeps its own ctypes mirror of cmag_sph_params (so its users never
    import the product); field names, types and offsets equal the product's."""
    from cmag_gb300 import _abi
    from oracle import params as OP
    a, b = _abi.SphParams, OP.SphParams
    assert [(f, str(t)) for f, t in a._fields_] == [(f, str(t)) for f, t in b._fields_]
    assert [getattr(a, f).offset for f, _ in a._fields_] == [getattr(b, f).offset for f, _ in b._fields_]
    import ctypes
    assert ctypes.sizeof(a) == ctypes.sizeof(b)


@pytest.mark.parametrize("name", ["dambreak3d", "peristalsis", "poiseuille", "poiseuille_ref"])
def test_oracle_workloads_equal_the_presets(built, name):
    """bench.py's CPU arms derive the workloads on the oracle alone: same bytes as
    the product's presets (which derive them through the library)."""
    from cmag_gb300 import presets
    from oracle import workloads as W
    if name == "dambreak3d":
        a, na, _, _ = presets.dambreak3d()
        b, nb, _, _ = W.dambreak3d()
        assert na == nb == 954_860
    elif name == "peristalsis":
        a, b = presets.peristalsis_c3(), W.peristalsis_c3()
    else:
        ref = name == "poiseuille_ref"
        a, b = presets.poiseuille_c1(reference_physics=ref), W.poiseuille_c1(reference_physics=ref)
    assert bytes(a) == bytes(b)


def test_oracle_batched_scenes_equal_the_presets(built):
    from cmag_gb300 import presets
    from oracle import workloads as W
    a, b = presets.batched_scenes(), W.batched_scenes()
    assert a[1] == b[1] and a[2] == b[2] and a[3] == b[3]
    assert all(bytes(x) == bytes(y) for x, y in zip(a[0], b[0]))
    alphas = [float(p.av_alpha) for p, d in zip(a[0], a[3]) if d[0] == "dambreak"]
    assert 0.11 < min(alphas) < max(alphas) < 1.21
