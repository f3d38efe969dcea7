"""The reference's own assembly against this project's oracle and host
mirror, on the CPU.

oracle/_ref/ref_assemble is GmshFEM's library compiled from its sources with
the project's gmsh stand-in (meshes, quadrature, bases, keys); it runs the
reference's real Formulation::pre() and assemble(). For each problem the
tests check, against that output:
  * the CSR pattern (ai, aj) of the host mirror's pre(), bit for bit;
  * the DOF dictionary (keys, assemble types and the Hilbert numbering, in
    iteration order), bit for bit;
  * the oracle's CSR values and right-hand side, to 1e-13 relative Frobenius
    (the reference adds with OpenMP atomics in no fixed order).
The GPU tests compare the GPU path with the oracle, so this pins the GPU
path to the reference. Skipped where the reference tree is absent (the
program is then not built)."""
import numpy as np
import pytest

from oracle import reference

pytestmark = pytest.mark.skipif(not reference.available(), reason="reference program not built (no reference tree)")

TOL = 1e-13


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def cases(femg):
    c = {
        "c1_full": femg.config_c1(),
        "c1_m16_dirichlet1": femg.config_c1(m=16),
        "tri_p1_lagrange": femg.config(dim=2, m=12, mesh_order=1, space=femg.FG_SPACE_LAGRANGE, gauss=2, dirichlet=1,
                                       dirichlet_value=2.0, source=1, k=4.0),
        "tri_h1_p3": femg.config(dim=2, m=10, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=3, gauss=6, k=5.0,
                                 source=1),
        "tri_h1_p4_bubbles": femg.config(dim=2, m=4, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=4, gauss=8),
        "c2_p1_m8": femg.config_c2(m=8, order=1),
        "c2_p2_m8": femg.config_c2(m=8, order=2),
        "c2_m8": femg.config_c2(m=8),
        "c2_p4_m5": femg.config_c2(m=5, order=4),
        "c3_m10": femg.config_c3(m=10),
        "c5_m5": femg.config_c5(m=5),
        "maxwell_2d": femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=2, m=8, mesh_order=1, space=femg.FG_SPACE_HCURL,
                                  order=0, gauss=2, jitter=0.15, seed=7, k=3.0, coef_mode=1),
        "maxwell_3d": femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=3, m=4, mesh_order=1, space=femg.FG_SPACE_HCURL,
                                  order=0, gauss=2, jitter=0.15, seed=7, k=3.0),
        "upper_c3_m4": femg.config_c3(m=4),
        "upper_tri_p4_bubbles": femg.config(dim=2, m=4, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=4,
                                            gauss=8),
    }
    c["c1_m16_dirichlet1"].dirichlet_value = 1.0
    c["upper_c3_m4"].upper = 1
    c["upper_tri_p4_bubbles"].upper = 1
    return c


NAMES = ["c1_full", "c1_m16_dirichlet1", "tri_p1_lagrange", "tri_h1_p3", "tri_h1_p4_bubbles", "c2_p1_m8", "c2_p2_m8",
         "c2_m8", "c2_p4_m5", "c3_m10", "c5_m5", "maxwell_2d", "maxwell_3d", "upper_c3_m4", "upper_tri_p4_bubbles"]


@pytest.mark.parametrize("name", NAMES)
def test_reference_matches_mirror_and_oracle(femg, oracle, name):
    cfg = cases(femg)[name]
    ref = reference.run(cfg, threads=4)
    prob = femg.Problem(cfg)
    a = prob.arrays()
    # pattern and numbering: bit for bit
    assert ref["n_rows"] == int(a["n_rows"])
    assert np.array_equal(ref["ai"], a["ai"])
    assert np.array_equal(ref["aj"], a["aj"])
    rd = prob.raw_dofs()
    assert np.array_equal(ref["dof_num_type"], rd["num_type"])
    assert np.array_equal(ref["dof_entity"], rd["entity"])
    assert np.array_equal(ref["dof_num_dof"], rd["num_dof"])
    assert np.array_equal(ref["dof_assemble_type"], rd["assemble_type"])
    # values: the oracle's restatement of assemble()
    t, nt = prob.terms()
    v, b = oracle.assemble(a, t, nt)
    assert np.linalg.norm(ref["values"]) > 0
    assert rel(v, ref["values"]) <= TOL, rel(v, ref["values"])
    if np.linalg.norm(ref["rhs"]) > 0:
        assert rel(b, ref["rhs"]) <= TOL, rel(b, ref["rhs"])
    else:
        assert np.linalg.norm(b) == 0
    prob.close()
