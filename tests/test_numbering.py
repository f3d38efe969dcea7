"""DOF dictionary order, Hilbert numbering and CSR pattern of the host mirror
against the oracle, and the oracle against the reference's own robin_hood.h
and Hilbert.cpp (oracle/_ref) where that build exists."""
import numpy as np
import pytest


def configs(femg):
    return {
        "c1_m8": femg.config_c1(m=8),
        "c1_m16_p1mesh": femg.config(dim=2, m=16, mesh_order=1, gauss=2, dirichlet=1, source=1),
        "c2_m3": femg.config_c2(m=3),
        "c2_m2_p4": femg.config_c2(m=2, order=4),
        "c2_m3_p2": femg.config_c2(m=3, order=2),
        "tet_lagrange_p2": femg.config(dim=3, m=2, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4),
        "c5_m2": femg.config_c5(m=2),
    }


CASES = ["c1_m8", "c1_m16_p1mesh", "c2_m3", "c2_m2_p4", "c2_m3_p2", "tet_lagrange_p2", "c5_m2"]


def _product_order(prob):
    cr = prob.created_dofs()
    rd = prob.raw_dofs()
    key = {(int(t), int(e)): i for i, (t, e) in enumerate(zip(cr["num_type"], cr["entity"]))}
    return cr, rd, np.array([key[(int(t), int(e))] for t, e in zip(rd["num_type"], rd["entity"])], np.uint32)


@pytest.mark.parametrize("case", CASES)
def test_pattern_matches_oracle(femg, oracle, case):
    prob = femg.Problem(configs(femg)[case])
    a = prob.arrays()
    ai, aj = oracle.pattern(a["edof"], a["etype"], a["n_rows"])
    assert np.array_equal(ai, a["ai"])
    assert np.array_equal(aj, a["aj"])
    # columns sorted and unique per row (finalizePattern output)
    for r in range(0, int(a["n_rows"]), max(1, int(a["n_rows"]) // 50)):
        row = aj[ai[r]:ai[r + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0)


@pytest.mark.parametrize("case", CASES)
def test_dictionary_order_matches_oracle(femg, oracle, case):
    prob = femg.Problem(configs(femg)[case])
    cr, rd, prod = _product_order(prob)
    at, arg = prob.reserve_log()
    kinds, args = oracle.robin_script(len(cr["num_type"]), at, arg)
    mine = oracle.robin_order(kinds, args, cr["num_type"], cr["entity"])
    assert np.array_equal(prod, mine)
    if oracle.ref() is not None:
        ref = oracle.robin_order(kinds, args, cr["num_type"], cr["entity"], use_ref=True)
        assert np.array_equal(mine, ref)


@pytest.mark.parametrize("case", CASES)
def test_numbering_matches_oracle(femg, oracle, case):
    prob = femg.Problem(configs(femg)[case])
    a = prob.arrays()
    rd = prob.raw_dofs()
    atp = rd["assemble_type"]
    nu = int(np.sum((atp == 2) | (atp == 3)))
    nb = int(np.sum(atp == 3))
    assert nu == a["n_rows"]
    nd = oracle.reorder_hilbert(a["dim"], prob.bbox(), rd["xyz"], atp, nu, nb)
    mask = (atp == 2) | (atp == 3)
    assert np.array_equal(nd[mask], rd["num_dof"][mask])
    # a permutation of 1..nu, bubbles last
    assert np.array_equal(np.sort(rd["num_dof"][mask]), np.arange(1, nu + 1, dtype=np.uint64))
    if nb:
        assert rd["num_dof"][atp == 3].min() == nu - nb + 1
    # fixed DOFs keep their creation numbering 1..n_fixed
    fx = atp == 1
    assert np.array_equal(np.sort(rd["num_dof"][fx]), np.arange(1, fx.sum() + 1, dtype=np.uint64))


@pytest.mark.parametrize("dim", [2, 3])
def test_hilbert_oracle_matches_reference(oracle, dim):
    if oracle.ref() is None:
        pytest.skip("reference numbering driver not built here")
    rng = np.random.default_rng(7 + dim)
    pts = rng.random((5000, dim), dtype=np.float32)
    pts[100:200] = pts[0]  # ties keep input order (stable)
    mn = np.full(dim, -1e-6, np.float32)
    mx = np.full(dim, 1 + 1e-6, np.float32)
    assert np.array_equal(oracle.hilbert_order(dim, pts, mn, mx), oracle.ref_hilbert_order(dim, pts, mn, mx))


def test_c1_sizes(femg):
    """Full-size 2D workload: 16,641 DOFs, 512 fixed, nnz 182,325."""
    prob = femg.Problem(femg.config_c1())
    a = prob.arrays()
    assert a["E"] == 8192
    assert a["n_fixed"] == 512
    assert a["n_rows"] == 16129
    assert prob.nnz == 182325


def test_tet_dof_counts(femg):
    # (p m + 1)^3 DOFs on the Kuhn cube for hierarchical order p
    for p, m in ((1, 3), (2, 3), (3, 3), (4, 2)):
        prob = femg.Problem(femg.config_c2(m=m, order=p))
        assert prob.arrays()["n_rows"] == (p * m + 1) ** 3
