"""Terms with non-symmetric element matrices in the oracle, against the
reference's own assembly (oracle/_ref/ref_assemble with coefficient
programs): a general TensorFunction D in integral(D grad(dof u), grad(tf u)),
the advection integral(b . grad(dof u), tf(u)) with a VectorFunction b, its
transpose integral(b dof(u), grad(tf u)) and a vector source
integral(f, grad(tf u)),
with a Dirichlet boundary of value 1, so that the lifting's transposed read
of the element matrix (addValuesDC, src/system/VectorFactory.cpp:184) shows
in the right-hand side. CSR values and right-hand side to 1e-13."""
import numpy as np
import pytest

from coef_programs import nonsym_configs, nonsym_terms
from oracle import reference

TOL = 1e-13


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.skipif(not reference.available(), reason="reference program not built (no reference tree)")
@pytest.mark.parametrize("what", ["full", "advect", "both", "vdof", "vsrc", "vector"])
@pytest.mark.parametrize("geom", ["tri_p2_dirichlet1", "tri_h1_p3", "tet_h1_p2"])
def test_nonsymmetric_terms_match_reference(femg, oracle, geom, what):
    cfg = nonsym_configs(femg)[geom]
    prob = femg.Problem(cfg)
    a = prob.arrays()
    t, nt, programs, keep = nonsym_terms(femg, what)
    ref = reference.run(cfg, threads=2, programs=programs)
    assert np.array_equal(ref["ai"], a["ai"]) and np.array_equal(ref["aj"], a["aj"])
    v, b = oracle.assemble(a, t, nt)
    assert rel(v, ref["values"]) <= TOL, rel(v, ref["values"])
    assert rel(b, ref["rhs"]) <= TOL, rel(b, ref["rhs"])
    # the element matrices are not symmetric: A differs from its transpose
    ai, aj = a["ai"].astype(np.int64), a["aj"].astype(np.int64)
    n = len(ai) - 1
    rows = np.repeat(np.arange(n), np.diff(ai))
    A = {(int(r), int(c)): val for r, c, val in zip(rows, aj, v)}
    asym = max(abs(A[(r, c)] - A.get((c, r), 0)) for (r, c) in A)
    if what != "vsrc":  # a vector source alone leaves the (mass) matrix symmetric
        assert asym > 1e-3
