"""Tensor coefficients on HCurl fields (the Maxwell PML form:
integral(D_c * curl(dof(E)), curl(tf(E))) and integral(D_m * dof(E), tf(E))
with symmetric tensors) in the oracle, pinned by identities that do not use
its tensor code:
- D = d I gives the scalar terms with coefficients times d;
- a constant field E0 (the discrete gradient of E0 . x) has mass energy
  c_m E0^T D E0 |Omega|;
- the field F = (w x x) / 2, whose edge values are F(midpoint) . (x_hi - x_lo)
  (exact for this linear field, lowest-order edge functions span it), has
  constant curl w and curl-curl energy w^T D w |Omega|."""
import ctypes as C

import numpy as np
import pytest

from test_hcurl import EDGES, csr_apply, edge_values, maxwell
from test_tensor_coef import ORDER, const_expr


def hcurl_tensor_terms(femg, prob, Dc=None, Dm=None, keep=(0, 1)):
    """The problem's curl-curl (kind GRAD_GRAD) and mass terms, those in keep
    (0: curl-curl, 1: mass), each in its tensor form when its tensor is given;
    the coefficients stay the problem's."""
    t, nt = prob.terms()
    kinds = {femg.FG_TERM_GRAD_GRAD: 0, femg.FG_TERM_MASS: 1}
    idx = [i for i in range(nt) if t[i].kind in kinds and kinds[int(t[i].kind)] in keep]
    arr = (femg.TermDesc * len(idx))()
    arr._keep = []
    for k, i in enumerate(idx):
        C.memmove(C.byref(arr[k]), C.byref(t[i]), C.sizeof(femg.TermDesc))
        D = Dc if t[i].kind == femg.FG_TERM_GRAD_GRAD else Dm
        if D is None:
            continue
        arr[k].kind = femg.FG_TERM_GRAD_GRAD_TENSOR if t[i].kind == femg.FG_TERM_GRAD_GRAD else femg.FG_TERM_MASS_TENSOR
        tens = (femg.Expr * 6)()
        for q, (a, b) in enumerate(ORDER):
            const_expr(femg, tens[q], float(np.real(D[a][b])), float(np.imag(D[a][b])))
        arr[k].tensor = C.cast(tens, C.POINTER(femg.Expr))
        arr._keep.append(tens)
    return arr, len(idx)


def scaled_terms(femg, prob, dc, dm):
    """The problem's curl-curl and mass terms with coefficients times dc, dm."""
    t, nt = prob.terms()
    idx = [i for i in range(nt) if t[i].kind in (femg.FG_TERM_GRAD_GRAD, femg.FG_TERM_MASS)]
    arr = (femg.TermDesc * len(idx))()
    for k, i in enumerate(idx):
        C.memmove(C.byref(arr[k]), C.byref(t[i]), C.sizeof(femg.TermDesc))
        ex = arr[k].coef
        n = ex.n_code
        ex.code[n].op, ex.code[n].arg = femg.FG_OP_CONST, 0
        ex.code[n].re, ex.code[n].im = (dc if t[i].kind == femg.FG_TERM_GRAD_GRAD else dm), 0.0
        ex.code[n + 1].op = femg.FG_OP_MUL
        ex.n_code = n + 2
    return arr, len(idx)


def rotation_field(a, w):
    """edge values of F = (w x x) / 2"""
    dim = int(a["dim"])
    xyz = a["xyz"]
    u = np.zeros(int(a["n_rows"]))
    en = a["enodes"].astype(np.int64)
    for k, (p, q) in enumerate(EDGES[dim]):
        na, nb = en[:, p], en[:, q]
        lo, hi = np.minimum(na, nb), np.maximum(na, nb)
        mid = 0.5 * (xyz[lo] + xyz[hi])
        F = 0.5 * np.cross(w, mid)
        u[a["edof"][:, k].astype(np.int64)] = np.sum(F * (xyz[hi] - xyz[lo]), axis=1)
    return u


def spd(seed, cplx=False, dim=3):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((3, 3))
    D = M @ M.T + 2 * np.eye(3)
    if cplx:
        D = D + 1j * np.diag([0.4, -0.3, 0.2])
    if dim == 2:
        D[2, :2] = D[:2, 2] = 0.0
    return D


@pytest.mark.parametrize("dim,m", [(2, 4), (3, 2)])
def test_isotropic_tensors_are_the_scalar_terms(femg, oracle, dim, m):
    prob = maxwell(femg, dim, m)
    a = prob.arrays()
    t1, n1 = hcurl_tensor_terms(femg, prob, 1.5 * np.eye(3), 0.75 * np.eye(3))
    t2, n2 = scaled_terms(femg, prob, 1.5, 0.75)
    v1, _ = oracle.assemble(a, t1, n1, with_rhs=False)
    v2, _ = oracle.assemble(a, t2, n2, with_rhs=False)
    assert np.abs(v1 - v2).max() <= 1e-13 * np.abs(v2).max()


@pytest.mark.parametrize("dim,m", [(2, 4), (3, 2)])
@pytest.mark.parametrize("cplx", [False, True])
def test_constant_field_mass_energy(femg, oracle, dim, m, cplx):
    k = 3.0
    prob = maxwell(femg, dim, m, k=k)
    a = prob.arrays()
    D = spd(1, cplx, dim)
    t, nt = hcurl_tensor_terms(femg, prob, None, D, keep=(1,))
    v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    E0 = np.array([1.0, -2.0, 0.5]) if dim == 3 else np.array([1.0, -2.0, 0.0])
    u = edge_values(a, a["xyz"] @ E0)
    energy = np.dot(u, csr_apply(a, v, u))
    expect = -k * k * (E0 @ D @ E0)
    assert abs(energy - expect) <= 1e-11 * abs(expect)


@pytest.mark.parametrize("dim,m", [(2, 4), (3, 2)])
@pytest.mark.parametrize("cplx", [False, True])
def test_rotation_field_curl_energy(femg, oracle, dim, m, cplx):
    prob = maxwell(femg, dim, m)
    a = prob.arrays()
    D = spd(2, cplx, dim)
    t, nt = hcurl_tensor_terms(femg, prob, D, None, keep=(0,))
    v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    w = np.array([0.3, -1.1, 0.8]) if dim == 3 else np.array([0.0, 0.0, 1.3])
    u = rotation_field(a, w)
    energy = np.dot(u, csr_apply(a, v, u))
    expect = w @ D @ w  # the curl-curl coefficient is 1
    assert abs(energy - expect) <= 1e-11 * abs(expect)
