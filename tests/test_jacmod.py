"""Jacobian modificators (transformation shells and the axisymmetric measure)
in the oracle, pinned against integrals computed independently of it.

A shell of the reference (src/domain/*Shell.cpp) is the change of variables
x' = c + (x - c) f(r) in its stretched directions, with
f(r) = (r_min (r_max - r_min) / (r (r_max - r)))^k; its jac and det formulas
are the derivative of that map. The pins take the map's derivative by central
differences and integrate on a tensor Gauss-Legendre grid over the unit
square or cube, so they check the jac/det formulas, their composition with
the element Jacobian and the assembly, without sharing code with the oracle:
  mass of u = 1:        |Omega'| = int det(Dx') (times r' when axisymmetric)
  stiffness of u = x_0: int |Dx'^-T e_0|^2 det(Dx') (times r')
The plain axisymmetric measure gives int_0^1 int_0^1 r dr dz = 1/2 for both."""
import ctypes as C

import numpy as np
import pytest

SQ = dict(r_min=1.5, r_max=4.0)


def jm_problem(femg, dim, m, gauss=8):
    return femg.Problem(femg.config(dim=dim, m=m, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=1, gauss=gauss,
                                    jitter=0.15, seed=4, k=2.0))


def with_jacmod(femg, prob, kind, term_kind, axis=0, exponent=1, center=(0.0, 0.0, 0.0), r_min=1.5, r_max=4.0):
    """The problem's term of term_kind alone, with the modificator."""
    t, nt = prob.terms()
    src = [i for i in range(nt) if t[i].kind == term_kind][0]
    arr = (femg.TermDesc * 1)()
    C.memmove(C.byref(arr[0]), C.byref(t[src]), C.sizeof(femg.TermDesc))
    arr[0].coef.n_code, arr[0].coef.n_arrays = 1, 0  # coefficient 1
    ins = arr[0].coef.code[0]
    ins.op, ins.arg, ins.re, ins.im = femg.FG_OP_CONST, 0, 1.0, 0.0
    j = arr[0].jacmod
    j.kind, j.axis, j.exponent, j.r_min, j.r_max = kind, axis, exponent, r_min, r_max
    for c in range(3):
        j.center[c] = center[c]
    return arr, 1


def vertex_vector(prob, a, fn):
    rd = prob.raw_dofs()
    u = np.zeros(int(a["n_rows"]))
    vert = (rd["num_type"] == 0) & ((rd["assemble_type"] == 2) | (rd["assemble_type"] == 3))
    u[(rd["num_dof"][vert] - 1).astype(np.int64)] = fn(a["xyz"][(rd["entity"][vert] - 1).astype(np.int64)])
    return u


def quad_form(a, v, u):
    ai, aj = a["ai"].astype(np.int64), a["aj"].astype(np.int64)
    rows = np.repeat(np.arange(len(ai) - 1), np.diff(ai))
    return float(np.sum(u[rows] * v.real * u[aj]))


def shell_map(x, kind, femg, center, axis, exponent, r_min, r_max):
    """x' for points x [N, 3] (the stretched map of the shell)."""
    c = np.asarray(center, float)
    d = x - c
    if kind == femg.FG_JACMOD_AXISYMMETRY_SHELL:
        d = x - np.array([0.0, c[1], 0.0])
        d[:, 2] = 0.0
    elif kind == femg.FG_JACMOD_POLAR_SHELL:
        d[:, 2] = 0.0
    elif kind == femg.FG_JACMOD_CYLINDRICAL_SHELL:
        d[:, axis] = 0.0
    r = np.linalg.norm(d, axis=1)
    f = ((r_min * (r_max - r_min)) / (r * (r_max - r))) ** exponent
    return x + d * (f - 1.0)[:, None]


def grid(dim, n=40):
    g, w = np.polynomial.legendre.leggauss(n)
    g, w = 0.5 * (g + 1.0), 0.5 * w
    if dim == 2:
        X, Y = np.meshgrid(g, g, indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
        return pts, np.outer(w, w).ravel()
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1), np.einsum("i,j,k->ijk", w, w, w).ravel()


def reference_integrals(femg, dim, kind, **p):
    """(int det Dx' [r'], int |Dx'^-T e0|^2 det Dx' [r']) over the unit square/cube."""
    pts, w = grid(dim)
    h = 1e-5
    D = np.zeros((len(pts), dim, dim))  # D[:, l, m] = dx'_l / dx_m
    for mm in range(dim):
        e = np.zeros(3)
        e[mm] = h
        D[:, :, mm] = ((shell_map(pts + e, kind, femg, **p) - shell_map(pts - e, kind, femg, **p)) / (2 * h))[:, :dim]
    det = np.linalg.det(D)
    g0 = np.linalg.solve(np.transpose(D, (0, 2, 1)), np.tile(np.eye(dim)[0], (len(pts), 1))[..., None])[..., 0]
    meas = det.copy()
    if kind == femg.FG_JACMOD_AXISYMMETRY_SHELL:
        meas *= shell_map(pts, kind, femg, **p)[:, 0]  # r' = x'_0
    return float(np.sum(w * meas)), float(np.sum(w * meas * np.sum(g0 * g0, axis=1)))


def fe_integrals(femg, oracle, prob, kind, **p):
    a = prob.arrays()
    one = vertex_vector(prob, a, lambda X: np.ones(len(X)))
    x0 = vertex_vector(prob, a, lambda X: X[:, 0])
    tm, nm = with_jacmod(femg, prob, kind, femg.FG_TERM_MASS, **p)
    vm, _ = oracle.assemble(a, tm, nm, with_rhs=False)
    tg, ng = with_jacmod(femg, prob, kind, femg.FG_TERM_GRAD_GRAD, **p)
    vg, _ = oracle.assemble(a, tg, ng, with_rhs=False)
    return quad_form(a, vm, one), quad_form(a, vg, x0), (a, vg, one)


def test_axisymmetry_measure(femg, oracle):
    prob = jm_problem(femg, 2, 16)
    mass, stiff, (a, vg, one) = fe_integrals(femg, oracle, prob, femg.FG_JACMOD_AXISYMMETRY)
    assert abs(mass - 0.5) < 1e-12 and abs(stiff - 0.5) < 1e-12
    assert abs(quad_form(a, vg, one)) < 1e-12


SHELLS = {
    "polar_k1": (2, "FG_JACMOD_POLAR_SHELL", dict(center=(-2.0, 0.5, 0.0), exponent=1)),
    "polar_k2": (2, "FG_JACMOD_POLAR_SHELL", dict(center=(-2.0, 0.5, 0.0), exponent=2)),
    "axisym_shell": (2, "FG_JACMOD_AXISYMMETRY_SHELL", dict(center=(0.0, -2.0, 0.0), exponent=1)),
    "spherical": (3, "FG_JACMOD_SPHERICAL_SHELL", dict(center=(-2.0, 0.5, 0.5), exponent=1)),
    "cylindrical_z": (3, "FG_JACMOD_CYLINDRICAL_SHELL", dict(center=(-2.0, 0.5, 0.0), axis=2, exponent=1)),
    "cylindrical_y": (3, "FG_JACMOD_CYLINDRICAL_SHELL", dict(center=(-2.0, 0.0, 0.5), axis=1, exponent=1)),
}


@pytest.mark.parametrize("case", list(SHELLS))
def test_shell_against_its_map(femg, oracle, case):
    dim, name, p = SHELLS[case]
    kind = getattr(femg, name)
    prob = jm_problem(femg, dim, 24 if dim == 2 else 6)
    p = dict(p, **SQ)
    mass, stiff, (a, vg, one) = fe_integrals(femg, oracle, prob, kind, **p)
    ref_mass, ref_stiff = reference_integrals(femg, dim, kind, axis=p.get("axis", 0), **{k: v for k, v in p.items() if k != "axis"})
    tol = 1e-8
    assert abs(mass - ref_mass) <= tol * abs(ref_mass), (mass, ref_mass)
    assert abs(stiff - ref_stiff) <= tol * abs(ref_stiff), (stiff, ref_stiff)
    # constants stay in the kernel of the stiffness whatever the geometry
    assert abs(quad_form(a, vg, one)) <= 1e-11 * np.abs(vg).sum()


def test_point_outside_shell_is_an_error(femg, oracle):
    prob = jm_problem(femg, 2, 4)
    t, nt = with_jacmod(femg, prob, femg.FG_JACMOD_POLAR_SHELL, femg.FG_TERM_GRAD_GRAD, center=(-2.0, 0.5, 0.0),
                        r_min=1.5, r_max=2.5)
    with pytest.raises(ValueError):
        oracle.assemble(prob.arrays(), t, nt, with_rhs=False)
