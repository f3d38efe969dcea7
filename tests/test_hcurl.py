"""Lowest-order HCurl (edge elements) in the host mirror and the oracle,
pinned by exact identities of the discrete de Rham sequence rather than by
gmsh's basis tables (absent here):
- the edge values of a P1 nodal function (phi at the higher-tag end minus
  phi at the lower-tag end) lie in the kernel of the curl-curl matrix;
- a constant field is reproduced exactly: u^T A u = -k^2 |E|^2 |Omega|;
- the mass energy of a discrete gradient equals the P1 Laplace energy of
  the same nodal function on the same mesh (H1 and HCurl assembled apart)."""
import ctypes as C

import numpy as np
import pytest

EDGES = {2: [(0, 1), (1, 2), (2, 0)], 3: [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]}


def maxwell(femg, dim, m, coef_mode=0, k=3.0, seed=7):
    return femg.Problem(femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=dim, m=m, mesh_order=1, space=femg.FG_SPACE_HCURL,
                                    order=0, gauss=2, jitter=0.15, seed=seed, k=k, coef_mode=coef_mode))


def edge_values(a, phi_nodes):
    """DOF vector of the discrete gradient of nodal values phi_nodes."""
    dim = int(a["dim"])
    u = np.zeros(int(a["n_rows"]))
    en = a["enodes"].astype(np.int64)
    for k, (p, q) in enumerate(EDGES[dim]):
        na, nb = en[:, p], en[:, q]
        lo, hi = np.minimum(na, nb), np.maximum(na, nb)
        u[a["edof"][:, k].astype(np.int64)] = phi_nodes[hi] - phi_nodes[lo]
    return u


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


@pytest.mark.parametrize("dim,m", [(2, 4), (3, 3)])
def test_host_structure(femg, dim, m):
    prob = maxwell(femg, dim, m)
    a = prob.arrays()
    assert a["form"] == femg.FG_FORM_1
    assert a["nb"] == (3 if dim == 2 else 6)
    n_edges = 3 * m * m + 2 * m if dim == 2 else None
    if dim == 2:
        assert a["n_rows"] == n_edges
    assert a["bval"].shape[-1] == 3


@pytest.mark.parametrize("dim,m", [(2, 5), (3, 3)])
def test_discrete_gradients_in_curl_kernel(femg, oracle, dim, m):
    prob = maxwell(femg, dim, m)
    a = prob.arrays()
    rng = np.random.default_rng(3)
    u = edge_values(a, rng.standard_normal(len(a["xyz"])))
    t, nt = only(femg, prob, femg.FG_TERM_GRAD_GRAD)
    v, _ = oracle.assemble(a, t, nt)
    Ku = csr_apply(a, v, u)
    assert np.linalg.norm(Ku) <= 1e-12 * np.abs(v).max() * np.linalg.norm(u) * np.sqrt(len(u))


@pytest.mark.parametrize("dim,m", [(2, 5), (3, 3)])
def test_constant_field_energy(femg, oracle, dim, m):
    k = 3.0
    prob = maxwell(femg, dim, m, k=k)
    a = prob.arrays()
    E = np.array([1.0, -2.0, 0.5])[:dim] if dim == 3 else np.array([1.0, -2.0])
    u = edge_values(a, a["xyz"][:, :dim] @ E)
    t, nt = prob.terms()
    v, _ = oracle.assemble(a, t, nt)
    energy = np.dot(u, csr_apply(a, v, u).real)
    assert abs(energy - (-k * k * E @ E)) <= 1e-11 * k * k * (E @ E)


@pytest.mark.parametrize("dim,m", [(2, 5), (3, 3)])
def test_gradient_mass_equals_p1_laplace(femg, oracle, dim, m):
    k = 2.0
    prob = maxwell(femg, dim, m, k=k)
    a = prob.arrays()
    rng = np.random.default_rng(5)
    phi = rng.standard_normal(len(a["xyz"]))
    u = edge_values(a, phi)
    t, nt = only(femg, prob, femg.FG_TERM_MASS)
    v, _ = oracle.assemble(a, t, nt)
    e_hcurl = np.dot(u, csr_apply(a, v, u).real) / (-k * k)
    # the same mesh with P1 H1: vertex DOF of node x has entity x + 1
    h1 = femg.Problem(femg.config(dim=dim, m=m, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=1, gauss=2,
                                  jitter=0.15, seed=7, k=k))
    b = h1.arrays()
    assert np.array_equal(b["xyz"], a["xyz"])
    rd = h1.raw_dofs()
    w = np.zeros(int(b["n_rows"]))
    w[(rd["num_dof"] - 1).astype(np.int64)] = phi[(rd["entity"] - 1).astype(np.int64)]
    t1, n1 = only(femg, h1, femg.FG_TERM_GRAD_GRAD)
    v1, _ = oracle.assemble(b, t1, n1)
    e_h1 = np.dot(w, csr_apply(b, v1, w).real)
    assert abs(e_hcurl - e_h1) <= 1e-12 * abs(e_h1)
