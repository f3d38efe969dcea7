"""Pins of the oracle's element matrices against closed forms, and of the
reference-element data (quadrature, bases) against their defining
properties."""
import numpy as np
import pytest


def _p1_exact(X):
    """Exact P1 stiffness and mass of a simplex with vertex rows X (d+1, d)."""
    d = X.shape[1]
    T = np.hstack([np.ones((d + 1, 1)), X])
    grads = np.linalg.inv(T)[1:, :]  # column i = grad lambda_i
    vol = abs(np.linalg.det(T)) / (2.0 if d == 2 else 6.0)
    K = vol * grads.T @ grads
    M = vol / ((d + 1) * (d + 2)) * (np.ones((d + 1, d + 1)) + np.eye(d + 1))
    return K, M


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_p1_element_matrices_are_exact(femg, oracle, dim):
    k = 3.0
    if dim == 2:
        cfg = femg.config(dim=2, m=3, mesh_order=1, space=femg.FG_SPACE_LAGRANGE, gauss=2, jitter=0.2, k=k)
    else:
        cfg = femg.config_c2(m=2, order=1)
        cfg.k = k
    prob = femg.Problem(cfg)
    a = prob.arrays()
    t, nt = prob.terms()
    ke, _ = oracle.element_matrices(a, t, nt)
    xyz = a["xyz"]
    for e in range(a["E"]):
        X = xyz[a["enodes"][e, :dim + 1], :dim]
        K, M = _p1_exact(X)
        assert np.allclose(ke[e].real, K - k * k * M, rtol=0, atol=1e-13 * max(1, np.abs(K).max()))
        assert np.all(ke[e].imag == 0)


@pytest.mark.parametrize("gauss,dim", [(2, 2), (4, 2), (6, 2), (2, 3), (4, 3), (6, 3), (8, 3)])
def test_quadrature_exactness(femg, oracle, gauss, dim):
    """Gauss<N> integrates every monomial of degree <= N exactly on the
    reference simplex: int x^a y^b z^c = a! b! c! / (a+b+c+d)!"""
    from math import factorial
    cfg = femg.config(dim=dim, m=1, mesh_order=1, space=femg.FG_SPACE_LAGRANGE, gauss=gauss, jitter=0.0)
    prob = femg.Problem(cfg)
    r = prob.rule
    nq = r.nq
    w = np.ctypeslib.as_array(r.weights, shape=(nq,)).copy()
    # reference points from the geometric basis values: P1 values are the barycentrics
    gv = np.ctypeslib.as_array(r.geo_val, shape=(nq * (dim + 1),)).reshape(nq, dim + 1)
    pts = gv[:, 1:]
    for a_ in range(gauss + 1):
        for b_ in range(gauss + 1 - a_):
            for c_ in range(gauss + 1 - a_ - b_ if dim == 3 else 1):
                f = pts[:, 0] ** a_ * pts[:, 1] ** b_ * (pts[:, 2] ** c_ if dim == 3 else 1.0)
                exact = factorial(a_) * factorial(b_) * factorial(c_) / factorial(a_ + b_ + c_ + dim)
                assert abs(w @ f - exact) < 1e-14, (a_, b_, c_)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_hierarchical_vertex_functions_partition_unity(femg, order):
    prob = femg.Problem(femg.config_c2(m=1, order=order))
    a = prob.arrays()
    # vertex functions are the barycentrics: they sum to one; the others vanish at the vertices
    assert np.allclose(a["bval"][:, :, :4].sum(axis=2), 1.0, atol=1e-14)
    assert np.allclose(a["bgrad"][:, :, :4, :].sum(axis=2), 0.0, atol=1e-14)


def test_lagrange_partition_of_unity(femg):
    for cfg in (femg.config_c1(m=2), femg.config(dim=3, m=1, mesh_order=2, gauss=4)):
        a = femg.Problem(cfg).arrays()
        assert np.allclose(a["bval"].sum(axis=2), 1.0, atol=1e-14)
        assert np.allclose(a["bgrad"].sum(axis=2), 0.0, atol=1e-13)


@pytest.mark.parametrize("order", [2, 3, 4])
def test_conforming_energy_of_linear_function(femg, oracle, order):
    """u = x interpolated by vertex values only: u^T A u = int |grad x|^2 - k^2 int x^2
    = 1 - k^2/3 on the unit cube (needs conforming vertex functions and exact
    quadrature)."""
    k = 2.0
    cfg = femg.config_c2(m=2, order=order)
    cfg.k = k
    prob = femg.Problem(cfg)
    a = prob.arrays()
    t, nt = prob.terms()
    v, _ = oracle.assemble(a, t, nt)
    rd = prob.raw_dofs()
    u = np.zeros(int(a["n_rows"]))
    # vertex DOFs: type key 0, entity = node tag
    vert = (rd["num_type"] == 0) & ((rd["assemble_type"] == 2) | (rd["assemble_type"] == 3))
    u[(rd["num_dof"][vert] - 1).astype(np.int64)] = a["xyz"][(rd["entity"][vert] - 1).astype(np.int64), 0]
    ai, aj = a["ai"], a["aj"]
    rows = np.repeat(np.arange(int(a["n_rows"])), np.diff(ai.astype(np.int64)))
    uAu = np.sum(u[rows] * v.real * u[aj.astype(np.int64)])
    assert abs(uAu - (1.0 - k * k / 3.0)) < 1e-11
