"""The reference-element basis entry points of the host ABI
(fg_basis_eval, fg_basis_orientation in include/fem_g_gb300_host.h), for the
hierarchical H1 space: the vertex functions are the barycentric coordinates,
the gradients are those of the values (central differences), the function
count matches the space, and the orientation code reverses an edge when its
vertex tags are swapped; invalid arguments return -FG_ERR_ARG."""
import numpy as np
import pytest


def h1_count(dim, p):
    if dim == 2:
        return (p + 1) * (p + 2) // 2
    return (p + 1) * (p + 2) * (p + 3) // 6


@pytest.mark.parametrize("dim,p", [(2, 1), (2, 3), (2, 5), (3, 1), (3, 2), (3, 4)])
def test_h1_basis(femg, dim, p):
    rng = np.random.default_rng(dim * 10 + p)
    pts = rng.random((400, dim))
    pts = pts[pts.sum(1) < 1][:40]
    uvw = np.zeros((len(pts), 3))
    uvw[:, :dim] = pts
    val, grad = femg.basis_eval(femg.FG_SPACE_HIERARCHICAL_H1, p, dim, 0, uvw)
    assert val.shape == (len(pts), h1_count(dim, p))
    lam = np.concatenate([1.0 - pts.sum(1, keepdims=True), pts], axis=1)
    assert np.allclose(val[:, :dim + 1], lam, rtol=0, atol=1e-14)
    h = 1e-6
    for d in range(dim):
        e = np.zeros(3)
        e[d] = h
        vp, _ = femg.basis_eval(femg.FG_SPACE_HIERARCHICAL_H1, p, dim, 0, uvw + e)
        vm, _ = femg.basis_eval(femg.FG_SPACE_HIERARCHICAL_H1, p, dim, 0, uvw - e)
        assert np.abs((vp - vm) / (2 * h) - grad[:, :, d]).max() <= 1e-6 * max(1.0, np.abs(grad).max())


def test_orientation_codes(femg):
    # edge (0, 1) is the first edge: its bit flips when the two tags swap
    a = femg.basis_orientation(femg.FG_SPACE_HIERARCHICAL_H1, 3, 2, [1, 2, 3])
    b = femg.basis_orientation(femg.FG_SPACE_HIERARCHICAL_H1, 3, 2, [2, 1, 3])
    assert (a ^ b) & 1 == 1
    # order-0 HCurl codes carry the edge bits alone (no face digits)
    assert femg.basis_orientation(femg.FG_SPACE_HCURL, 0, 3, [4, 3, 2, 1]) < 64
    assert femg.basis_orientation(femg.FG_SPACE_HCURL, 1, 3, [4, 3, 2, 1]) >= 0


def test_invalid_arguments(femg):
    L = femg.lib()
    assert L.fg_basis_eval(femg.FG_SPACE_LAGRANGE, 1, 2, 0, 0, None, None, None) == -femg.FG_ERR_ARG
    assert L.fg_basis_eval(femg.FG_SPACE_HCURL, 1, 4, 0, 0, None, None, None) == -femg.FG_ERR_ARG
    assert L.fg_basis_orientation(femg.FG_SPACE_HCURL, 1, 3, None) == -femg.FG_ERR_ARG
