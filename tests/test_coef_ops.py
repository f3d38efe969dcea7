"""The coefficient language's scalar operators (sqrt, exp, ln, log, pow,
cbrt, the trigonometric and hyperbolic functions and their inverses, abs,
conj, real, imag, atan2, heaviside) in the oracle, against the reference's
own expression trees and assembly (oracle/_ref/ref_assemble with coefficient
programs): mass and source terms whose coefficient is the operator applied
to a complex, point-dependent argument. CSR values and right-hand side to
1e-13 relative Frobenius."""
import numpy as np
import pytest

from coef_programs import OPS, configs, terms
from oracle import reference

TOL = 1e-13


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.skipif(not reference.available(), reason="reference program not built (no reference tree)")
@pytest.mark.parametrize("geom", ["tri_p2", "tet_h1_p2"])
@pytest.mark.parametrize("op", OPS)
def test_operator_matches_reference(femg, oracle, geom, op):
    if op == "ATAN2":
        pytest.skip("the reference's atan2 takes real scalars only; the complex formulation has no atan2")
    cfg = configs(femg)[geom]
    prob = femg.Problem(cfg)
    a = prob.arrays()
    t, nt, programs = terms(femg, op)
    ref = reference.run(cfg, threads=2, programs=programs)
    assert np.array_equal(ref["ai"], a["ai"]) and np.array_equal(ref["aj"], a["aj"])
    v, b = oracle.assemble(a, t, nt)
    assert rel(v, ref["values"]) <= TOL, rel(v, ref["values"])
    assert rel(b, ref["rhs"]) <= TOL, rel(b, ref["rhs"])


@pytest.mark.parametrize("op", OPS)
def test_operator_values_match_numpy(femg, oracle, op):
    """The operators themselves on the oracle, against numpy's complex
    functions at the points of a small mesh (the mass term of a P1 mesh with
    one-point quadrature gives c(centroid) |T| on the diagonal blocks)."""
    cfg = femg.config(dim=2, m=3, mesh_order=1, space=femg.FG_SPACE_LAGRANGE, gauss=1, jitter=0.2, seed=5)
    prob = femg.Problem(cfg)
    a = prob.arrays()
    t, nt, _ = terms(femg, op)
    t[0].coef.code[0].re = 0.0  # no stiffness: the mass term alone
    v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    # expected: sum over elements of c(x_c) |T| / 9 on each (i, j) pair (P1, one point)
    xyz, en = a["xyz"], a["enodes"]
    x = xyz[en].mean(axis=1)
    arg = 0.4 + 0.3 * x[:, 0] + 0.2 * x[:, 1] + 0.1j * (x[:, 0] - x[:, 1])
    f = {"SQRT": np.sqrt, "EXP": np.exp, "LN": np.log, "LOG10": np.log10, "POW2": lambda z: z * z,
         "POW5": lambda z: np.abs(z) ** 5 * np.exp(5j * np.angle(z)), "CBRT": lambda z: np.abs(z) ** (1 / 3) * np.exp(1j * np.angle(z) / 3),
         "SIN": np.sin, "COS": np.cos, "TAN": np.tan, "SINH": np.sinh, "COSH": np.cosh, "TANH": np.tanh,
         "ASIN": np.arcsin, "ACOS": np.arccos, "ATAN": np.arctan, "ASINH": np.arcsinh, "ACOSH": lambda z: np.arccosh(z + 1),
         "ATANH": np.arctanh, "ABS": lambda z: np.abs(z) + 0j, "CONJ": np.conj, "REAL": lambda z: z.real + 0j,
         "IMAG": lambda z: z.imag + 0j, "ATAN2": lambda z: np.arctan2(z.real, 0.7 + x[:, 1]) + 0j,
         "HEAVISIDE": lambda z: np.where(z.real - 0.6 > 0, 1.0, np.where(z.real - 0.6 < 0, 0.0, 0.5)) + 0j}[op]
    c = f(arg)
    p = xyz[en]
    area = 0.5 * np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    n_rows = int(a["n_rows"])
    dense = np.zeros((n_rows, n_rows), complex)
    ed = a["edof"].astype(np.int64)
    for e in range(len(c)):
        for i in range(3):
            for j in range(3):
                dense[ed[e, i], ed[e, j]] += c[e] * area[e] / 9.0
    ai, aj = a["ai"].astype(np.int64), a["aj"].astype(np.int64)
    want = np.array([dense[r, aj[k]] for r in range(n_rows) for k in range(ai[r], ai[r + 1])])
    assert rel(v, want) <= 1e-13, rel(v, want)
