"""The tensor diffusion term integral(c * D * grad(dof(u)), grad(tf(u))) with
a symmetric 3x3 tensor of coefficient programs (the reference's
TensorFunction times grad, as its PML examples use) in the oracle, pinned
by identities that do not depend on the oracle's code:
- D = d I gives the scalar term with coefficient c d;
- for a linear u = v . x (exactly represented by P1 and P2 spaces) the
  energy u^T A u equals v^T D v |Omega| for any constant D, complex too."""
import ctypes as C

import numpy as np
import pytest

ORDER = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def const_expr(femg, ex, re, im=0.0):
    ex.n_code, ex.n_arrays = 1, 0
    ins = ex.code[0]
    ins.op, ins.arg, ins.re, ins.im = femg.FG_OP_CONST, 0, re, im


def tensor_terms(femg, prob, D, c=1.0, keep_mass=False, point_xx=False):
    """The problem's grad-grad term as a tensor term with constant D (3x3,
    complex allowed) and multiplier c (None: the problem's own coefficient);
    the mass term kept when asked; D_xx times (1 + x y) with point_xx."""
    t, nt = prob.terms()
    gg = [i for i in range(nt) if t[i].kind == femg.FG_TERM_GRAD_GRAD][0]
    mass = [i for i in range(nt) if t[i].kind == femg.FG_TERM_MASS]
    n = 1 + (1 if keep_mass and mass else 0)
    arr = (femg.TermDesc * n)()
    C.memmove(C.byref(arr[0]), C.byref(t[gg]), C.sizeof(femg.TermDesc))
    if n == 2:
        C.memmove(C.byref(arr[1]), C.byref(t[mass[0]]), C.sizeof(femg.TermDesc))
    arr[0].kind = femg.FG_TERM_GRAD_GRAD_TENSOR
    if c is not None:
        const_expr(femg, arr[0].coef, c)
    tens = (femg.Expr * 6)()
    for k, (a, b) in enumerate(ORDER):
        const_expr(femg, tens[k], float(np.real(D[a][b])), float(np.imag(D[a][b])))
    if point_xx:  # D_xx (1 + x y)
        code = [(femg.FG_OP_CONST, 0, 1.0, 0.0), (femg.FG_OP_X, 0, 0.0, 0.0), (femg.FG_OP_Y, 0, 0.0, 0.0),
                (femg.FG_OP_MUL, 0, 0.0, 0.0), (femg.FG_OP_ADD, 0, 0.0, 0.0), (femg.FG_OP_MUL, 0, 0.0, 0.0)]
        for i, (op, arg, re, im) in enumerate(code, start=1):
            ins = tens[0].code[i]
            ins.op, ins.arg, ins.re, ins.im = op, arg, re, im
        tens[0].n_code = 1 + len(code)
    arr[0].tensor = C.cast(tens, C.POINTER(femg.Expr))
    arr._tensor = tens  # keep the programs alive with the terms
    return arr, n


def scalar_terms(femg, prob, c):
    t, nt = prob.terms()
    gg = [i for i in range(nt) if t[i].kind == femg.FG_TERM_GRAD_GRAD][0]
    arr = (femg.TermDesc * 1)()
    C.memmove(C.byref(arr[0]), C.byref(t[gg]), C.sizeof(femg.TermDesc))
    const_expr(femg, arr[0].coef, c)
    return arr, 1


def linear_vector(prob, a, v):
    rd = prob.raw_dofs()
    u = np.zeros(int(a["n_rows"]))
    vert = (rd["num_type"] == 0) & ((rd["assemble_type"] == 2) | (rd["assemble_type"] == 3))
    u[(rd["num_dof"][vert] - 1).astype(np.int64)] = a["xyz"][(rd["entity"][vert] - 1).astype(np.int64)] @ v
    return u


def quad_form(a, vals, u):
    ai, aj = a["ai"].astype(np.int64), a["aj"].astype(np.int64)
    rows = np.repeat(np.arange(len(ai) - 1), np.diff(ai))
    return np.sum(u[rows] * vals * u[aj])


def problems(femg):
    return {
        "tet_p1": femg.Problem(femg.config(dim=3, m=3, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=1, gauss=2,
                                           jitter=0.15, seed=3)),
        "tet_p2": femg.Problem(femg.config(dim=3, m=2, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=2, gauss=4,
                                           jitter=0.15, seed=3)),
        "tri_p2": femg.Problem(femg.config(dim=2, m=4, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=3)),
    }


def test_isotropic_tensor_is_the_scalar_term(femg, oracle):
    prob = problems(femg)["tet_p2"]
    a = prob.arrays()
    t1, n1 = tensor_terms(femg, prob, 2.5 * np.eye(3), c=1.5)
    v1, _ = oracle.assemble(a, t1, n1, with_rhs=False)
    t2, n2 = scalar_terms(femg, prob, 1.5 * 2.5)
    v2, _ = oracle.assemble(a, t2, n2, with_rhs=False)
    assert np.abs(v1 - v2).max() <= 1e-13 * np.abs(v2).max()


@pytest.mark.parametrize("name", ["tet_p1", "tet_p2", "tri_p2"])
@pytest.mark.parametrize("cplx", [False, True])
def test_linear_field_energy(femg, oracle, name, cplx):
    prob = problems(femg)[name]
    a = prob.arrays()
    dim = int(a["dim"])
    rng = np.random.default_rng(11)
    M = rng.standard_normal((3, 3))
    D = M @ M.T + 3 * np.eye(3)
    if cplx:
        D = D + 1j * (0.5 * np.eye(3) + 0.1 * (M + M.T))
    if dim == 2:
        D[2, :] = D[:, 2] = 0.0
        D[2, 2] = 1.0
    t, n = tensor_terms(femg, prob, D)
    vals, _ = oracle.assemble(a, t, n, with_rhs=False)
    for _ in range(3):
        v = rng.standard_normal(3)
        if dim == 2:
            v[2] = 0.0
        u = linear_vector(prob, a, v)
        energy = quad_form(a, vals, u)
        expect = v @ D @ v  # |Omega| = 1
        assert abs(energy - expect) <= 1e-11 * abs(expect)
