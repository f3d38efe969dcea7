"""Hierarchical HCurl of order 1 (the reference's FunctionSpaceHierarchicalHCurl
with gmsh "HcurlLegendre1", here the stand-in basis of refelem.h: per edge
the Whitney function and grad(lambda_a lambda_b), per face lambda_c w_ab and
lambda_a w_bc), on the CPU:
  * the reference's own assembly (oracle/_ref/ref_assemble) against the host
    mirror's pattern and numbering (bit for bit) and the oracle's values
    (1e-13), in 2D (interior functions are bubbles) and 3D (shared faces);
  * exact de Rham identities that pin the basis without the oracle's HCurl
    code: the gradient of an order-2 hierarchical H1 function u has the
    order-1 coefficients (u_hi - u_lo) on each edge's Whitney function and
    u_e on its gradient function, lies in the kernel of the curl-curl
    matrix, and has the mass energy of u's Laplace energy in H1 order 2."""
import ctypes as C

import numpy as np
import pytest

from oracle import reference

EDGES = {2: [(0, 1), (1, 2), (2, 0)], 3: [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]}


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def maxwell1(femg, dim, m, coef_mode=0, k=3.0, seed=7):
    return femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=dim, m=m, mesh_order=1, space=femg.FG_SPACE_HCURL, order=1,
                       gauss=4, jitter=0.15, seed=seed, k=k, coef_mode=coef_mode)


def csr_apply(a, v, u):
    ai = a["ai"].astype(np.int64)
    rows = np.repeat(np.arange(len(ai) - 1), np.diff(ai))
    out = np.zeros(len(ai) - 1, np.complex128)
    np.add.at(out, rows, v * u[a["aj"].astype(np.int64)])
    return out


def only(femg, prob, kind):
    t, nt = prob.terms()
    idx = [i for i in range(nt) if t[i].kind == kind]
    arr = (femg.TermDesc * len(idx))()
    for j, i in enumerate(idx):
        C.memmove(C.byref(arr[j]), C.byref(t[i]), C.sizeof(femg.TermDesc))
    return arr, len(idx)


@pytest.mark.parametrize("dim,m", [(2, 4), (3, 2)])
def test_structure(femg, dim, m):
    prob = femg.Problem(maxwell1(femg, dim, m))
    a = prob.arrays()
    assert a["form"] == femg.FG_FORM_1
    assert a["nb"] == (8 if dim == 2 else 20)  # 2 per edge + 2 per face
    if dim == 2:  # the two interior functions of every triangle are bubbles
        rd = prob.raw_dofs()
        assert int((rd["assemble_type"] == femg.FG_AT_UNKNOWN_BUBBLE).sum()) == 2 * prob.E


@pytest.mark.skipif(not reference.available(), reason="reference program not built (no reference tree)")
@pytest.mark.parametrize("dim,m,coef_mode", [(2, 4, 1), (3, 2, 0), (3, 3, 1)])
def test_order1_matches_reference(femg, oracle, dim, m, coef_mode):
    cfg = maxwell1(femg, dim, m, coef_mode)
    ref = reference.run(cfg, threads=2)
    prob = femg.Problem(cfg)
    a = prob.arrays()
    assert np.array_equal(ref["ai"], a["ai"]) and np.array_equal(ref["aj"], a["aj"])
    rd = prob.raw_dofs()
    for k in ("num_type", "entity", "num_dof", "assemble_type"):
        assert np.array_equal(ref["dof_" + k], rd[k]), k
    t, nt = prob.terms()
    v, _ = oracle.assemble(a, t, nt)
    assert rel(v, ref["values"]) <= 1e-13, rel(v, ref["values"])


def gradient_coefficients(femg, a, h1, u_h1):
    """HCurl order-1 coefficients of grad u for u in H1 order 2 on the same mesh."""
    dim = int(a["dim"])
    b = h1.arrays()
    assert np.array_equal(b["xyz"], a["xyz"]) and np.array_equal(b["enodes"], a["enodes"])
    c = np.full(int(a["n_rows"]), np.nan)
    en = a["enodes"].astype(np.int64)
    nv = dim + 1
    for k, (p, q) in enumerate(EDGES[dim]):
        na, nb = en[:, p], en[:, q]
        lo_is_p = na < nb  # vertex tags are node index + 1
        up = u_h1[b["edof"][:, p].astype(np.int64)]
        uq = u_h1[b["edof"][:, q].astype(np.int64)]
        c[a["edof"][:, 2 * k].astype(np.int64)] = np.where(lo_is_p, uq - up, up - uq)
        c[a["edof"][:, 2 * k + 1].astype(np.int64)] = u_h1[b["edof"][:, nv + k].astype(np.int64)]
    # face (or interior) functions: no part in a gradient
    c[np.isnan(c)] = 0.0
    return c


@pytest.mark.parametrize("dim,m", [(2, 4), (3, 2)])
def test_gradients_of_order2_functions(femg, oracle, dim, m):
    k = 2.0
    prob = femg.Problem(maxwell1(femg, dim, m, k=k))
    a = prob.arrays()
    h1 = femg.Problem(femg.config(dim=dim, m=m, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=2, gauss=4,
                                  jitter=0.15, seed=7, k=k))
    b = h1.arrays()
    rng = np.random.default_rng(11)
    u = rng.standard_normal(int(b["n_rows"]))
    c = gradient_coefficients(femg, a, h1, u)
    # in the kernel of the curl-curl matrix
    tc, nc = only(femg, prob, femg.FG_TERM_GRAD_GRAD)
    vc, _ = oracle.assemble(a, tc, nc)
    assert np.linalg.norm(csr_apply(a, vc, c)) <= 1e-11 * np.abs(vc).max() * np.linalg.norm(c)
    # mass energy of grad u = Laplace energy of u
    tm, nm = only(femg, prob, femg.FG_TERM_MASS)
    vm, _ = oracle.assemble(a, tm, nm)
    e_hcurl = np.dot(c, csr_apply(a, vm, c).real) / (-k * k)
    t1, n1 = only(femg, h1, femg.FG_TERM_GRAD_GRAD)
    v1, _ = oracle.assemble(b, t1, n1)
    e_h1 = np.dot(u, csr_apply(b, v1, u).real)
    assert abs(e_hcurl - e_h1) <= 1e-12 * abs(e_h1), (e_hcurl, e_h1)
