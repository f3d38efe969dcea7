"""Hierarchical HCurl of any order (the reference's FunctionSpaceHierarchicalHCurl
with gmsh "HcurlLegendre<p>", src/field/FunctionSpaceHierarchicalHCurl.cpp:35,
:81-120; here the stand-in basis of refelem.h), on the CPU:
  * the reference-element basis spans the first-kind Nedelec space of degree
    p + 1 exactly: every function is a polynomial of degree p + 1 whose
    degree-(p+1) part q has x . q = 0, the functions are linearly independent
    and there are as many as the space's dimension; the curls are the curls
    of the values;
  * the assembled field is conforming: with random global coefficients, the
    tangential components seen from the two elements of every interior face
    (edge in 2D) agree, through the mirror's DOF keys, orientations and the
    covariant map;
  * the reference's own assembly (oracle/_ref/ref_assemble) against the host
    mirror's pattern and numbering (bit for bit) and the oracle's values."""
import itertools

import numpy as np
import pytest

from oracle import reference


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def nedelec_dim(dim, p):
    return (p + 1) * (p + 3) if dim == 2 else (p + 1) * (p + 3) * (p + 4) // 2


def maxwell(femg, dim, m, p, coef_mode=0, seed=7):
    return femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=dim, m=m, mesh_order=1, space=femg.FG_SPACE_HCURL, order=p,
                       gauss=2 * p + 2, jitter=0.15, seed=seed, k=3.0, coef_mode=coef_mode)


CASES = [(2, p) for p in range(0, 6)] + [(3, p) for p in range(0, 4)]


@pytest.mark.parametrize("dim,p", CASES)
def test_basis_spans_nedelec_space(femg, dim, p):
    rng = np.random.default_rng(100 * dim + p)
    pts = rng.random((2000, dim))
    pts = pts[pts.sum(1) < 1][:300]
    uvw = np.zeros((len(pts), 3))
    uvw[:, :dim] = pts
    ncode = 2 ** (3 * (dim - 1)) * (6 ** 4 if dim == 3 and p > 0 else 1)
    code = int(rng.integers(ncode))
    val, cur = femg.basis_eval(femg.FG_SPACE_HCURL, p, dim, code, uvw)
    n = val.shape[1]
    assert n == nedelec_dim(dim, p)
    mon = [m for m in itertools.product(range(p + 2), repeat=dim) if sum(m) <= p + 1]
    A = np.array([[np.prod(x ** np.array(m)) for m in mon] for x in pts])
    coef = np.linalg.lstsq(A, val[:, :, :dim].reshape(len(pts), -1), rcond=None)[0]  # [monomial][n * dim]
    assert np.abs(A @ coef - val[:, :, :dim].reshape(len(pts), -1)).max() <= 1e-11 * np.abs(val).max()
    coef = coef.T.reshape(n, dim, len(mon))
    scale = np.abs(coef).max()
    # x . q = 0 for the top-degree part q
    for i in range(n):
        acc = {}
        for c in range(dim):
            for k, m in enumerate(mon):
                if sum(m) == p + 1:
                    mm = list(m)
                    mm[c] += 1
                    acc[tuple(mm)] = acc.get(tuple(mm), 0.0) + coef[i, c, k]
        assert max(abs(v) for v in acc.values()) <= 1e-8 * scale
    sv = np.linalg.svd(coef.reshape(n, -1), compute_uv=False)
    assert sv[-1] > 1e-8 * sv[0]
    # curls of the values (central differences)
    h = 1e-6
    for q in range(4):
        J = np.zeros((n, 3, 3))
        for d in range(dim):
            e = np.zeros(3)
            e[d] = h
            vp, _ = femg.basis_eval(femg.FG_SPACE_HCURL, p, dim, code, (uvw[q] + e)[None])
            vm, _ = femg.basis_eval(femg.FG_SPACE_HCURL, p, dim, code, (uvw[q] - e)[None])
            J[:, :, d] = (vp[0] - vm[0]) / (2 * h)
        fd = np.stack([J[:, 2, 1] - J[:, 1, 2], J[:, 0, 2] - J[:, 2, 0], J[:, 1, 0] - J[:, 0, 1]], 1)
        assert np.abs(fd - cur[q]).max() <= 1e-6 * max(1.0, np.abs(cur[q]).max())


@pytest.mark.parametrize("dim,m,p", [(2, 3, 1), (2, 3, 3), (2, 2, 5), (3, 2, 1), (3, 2, 2), (3, 1, 3)])
def test_tangential_continuity(femg, dim, m, p):
    prob = femg.Problem(maxwell(femg, dim, m, p))
    a = prob.arrays()
    xyz, en = a["xyz"], a["enodes"].astype(np.int64)
    edof, etype = a["edof"].astype(np.int64), a["etype"]
    assert np.all((etype == femg.FG_AT_UNKNOWN) | (etype == femg.FG_AT_UNKNOWN_BUBBLE))
    rng = np.random.default_rng(3)
    c = rng.standard_normal(int(a["n_rows"]))
    nv = dim + 1
    sides = {}
    for e in range(len(en)):
        for f in itertools.combinations(range(nv), dim):
            sides.setdefault(tuple(sorted(en[e, list(f)])), []).append(e)
    shared = [(k, v) for k, v in sides.items() if len(v) == 2]
    assert len(shared) > 0

    def field(e, x):
        X = xyz[en[e, :nv]][:, :dim]
        J = (X[1:] - X[0]).T  # dx / duvw
        uvw = np.zeros((len(x), 3))
        uvw[:, :dim] = np.linalg.solve(J, (x - X[0]).T).T
        code = femg.basis_orientation(femg.FG_SPACE_HCURL, p, dim, en[e, :nv] + 1)
        val, _ = femg.basis_eval(femg.FG_SPACE_HCURL, p, dim, code, uvw)
        ref = np.einsum("qnc,n->qc", val[:, :, :dim], c[edof[e]])
        return np.linalg.solve(J.T, ref.T).T  # covariant map J^-T

    worst = 0.0
    for nodes, (ea, eb) in shared:
        V = xyz[list(nodes)][:, :dim]
        w = rng.dirichlet(np.ones(dim), size=3)
        x = w @ V
        ta = [V[k] - V[0] for k in range(1, dim)]  # tangents of the shared side
        fa, fb = field(ea, x), field(eb, x)
        for t in ta:
            worst = max(worst, np.abs((fa - fb) @ t).max() / max(1.0, np.abs(fa @ t).max()))
    assert worst <= 1e-11, worst


@pytest.mark.parametrize("dim,m,p", [(2, 3, 2), (2, 2, 5), (3, 2, 2), (3, 1, 3)])
def test_structure(femg, dim, m, p):
    prob = femg.Problem(maxwell(femg, dim, m, p))
    a = prob.arrays()
    assert a["form"] == femg.FG_FORM_1 and a["nb"] == nedelec_dim(dim, p)
    rd = prob.raw_dofs()
    per_elem = p * (p + 1) if dim == 2 else (p - 1) * p * (p + 1) // 2  # the element's own functions
    assert int((rd["assemble_type"] == femg.FG_AT_UNKNOWN_BUBBLE).sum()) == per_elem * prob.E


@pytest.mark.skipif(not reference.available(), reason="reference program not built (no reference tree)")
@pytest.mark.parametrize("dim,m,p,coef_mode", [(2, 3, 2, 1), (2, 2, 4, 0), (3, 2, 2, 1), (3, 1, 3, 0)])
def test_high_order_matches_reference(femg, oracle, dim, m, p, coef_mode):
    cfg = maxwell(femg, dim, m, p, coef_mode)
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
