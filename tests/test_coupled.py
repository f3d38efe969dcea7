"""Terms that couple two fields (a BilinearTerm whose unknown and test fields
differ, src/term/BilinearTerm.cpp:156-273), on the CPU:
  * the reference's own assembly (oracle/_ref/ref_assemble) against the host
    mirror: the CSR pattern and both fields' DOF dictionaries with the
    numbering, bit for bit (the reference numbers the two fields' DOFs
    together, in the order of its unordered_set of fields);
  * the oracle's block-by-block assembly (oracle.assemble_blocks) against
    the reference's values and right-hand side at 1e-13;
  * the blocks the mirror forms, and the oracle's refusal of a lifting that
    the reference reads outside the element matrix."""
import numpy as np
import pytest

from coupled_cases import coupled_configs, lifting_undefined_config
from oracle import reference

TOL = 1e-13


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.skipif(not reference.available(), reason="reference program not built (no reference tree)")
@pytest.mark.parametrize("name", ["tri_lagrange_p2_dirichlet", "tri_h1_p3_p2", "tet_h1_p2_p1", "tet_h1_p1_p3"])
def test_coupled_matches_reference(femg, oracle, name):
    cfg = coupled_configs(femg)[name]
    ref = reference.run(cfg, threads=2)
    prob = femg.Problem(cfg)
    a = prob.arrays()
    assert ref["fields"] == 2 and prob.n_fields() == 2
    assert ref["n_rows"] == int(a["n_rows"])
    assert np.array_equal(ref["ai"], a["ai"]) and np.array_equal(ref["aj"], a["aj"])
    rd = prob.raw_dofs()
    for k in ("num_type", "entity", "num_dof", "assemble_type"):
        assert np.array_equal(ref["dof_" + k], rd[k]), k
    v, b = oracle.assemble_blocks(prob)
    assert np.linalg.norm(ref["values"]) > 0
    assert rel(v, ref["values"]) <= TOL, rel(v, ref["values"])
    if np.linalg.norm(ref["rhs"]) > 0:
        assert rel(b, ref["rhs"]) <= TOL, rel(b, ref["rhs"])
    else:
        assert np.linalg.norm(b) == 0
    prob.close()


def test_coupled_blocks_and_fields(femg):
    prob = femg.Problem(coupled_configs(femg)["tri_h1_p3_p2"])
    blocks = [(t, u, n) for t, u, _, n in prob.blocks()]
    # (u, u): grad, mass, source; (v, v): grad, mass, source; v rows with u
    # columns: mass and advection; u rows with v columns: grad-grad
    assert blocks == [(0, 0, 3), (1, 1, 3), (1, 0, 2), (0, 1, 1)]
    _, _, tp, nt = prob.blocks()[2]
    kinds = sorted(tp[k].kind for k in range(nt))
    assert kinds == sorted([femg.FG_TERM_MASS, femg.FG_TERM_ADVECTION])
    su, iu, tu = prob.field(0)
    sv, iv, tv = prob.field(1)
    assert (su.n_basis, sv.n_basis) == (10, 6)  # order 3 and 2 on triangles
    assert iu.shape == (prob.E, 10) and iv.shape == (prob.E, 6)
    # the two fields number disjoint sets of rows that cover all unknowns
    rows = np.concatenate([iu[tu == femg.FG_AT_UNKNOWN], iu[tu == femg.FG_AT_UNKNOWN_BUBBLE],
                           iv[tv == femg.FG_AT_UNKNOWN], iv[tv == femg.FG_AT_UNKNOWN_BUBBLE]])
    assert np.array_equal(np.unique(rows), np.arange(int(prob.sys.n_rows)))
    assert not set(np.unique(iu[tu >= femg.FG_AT_UNKNOWN])) & set(np.unique(iv[tv >= femg.FG_AT_UNKNOWN]))


def test_coupled_lifting_without_defined_value(femg, oracle):
    prob = femg.Problem(lifting_undefined_config(femg))
    assert prob.sys.n_fixed > 0
    with pytest.raises(ValueError):
        oracle.assemble_blocks(prob)
    # the values alone are defined
    v, _ = oracle.assemble_blocks(prob, with_rhs=False)
    assert np.linalg.norm(v) > 0


def test_coupled_needs_scalar_fields(femg):
    # the two-field problem takes scalar H1 spaces (Lagrange or hierarchical)
    with pytest.raises(femg.FgError):
        femg.Problem(femg.config(kind=femg.FG_PROBLEM_COUPLED, dim=2, m=2, mesh_order=1, space=femg.FG_SPACE_HCURL))
