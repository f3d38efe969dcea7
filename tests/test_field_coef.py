"""Field-node coefficients (FG_OP_FIELD): a scalar field of the bucket's own
H1 space evaluated at the quadrature points, u(x_q) = sum_j phi_j(x_q) u_e[j],
as the reference's field nodes do (fieldOperations.h:160-170). The oracle is
pinned by an identity that does not use its field code: the field u = v . x
(in a hierarchical H1 space its coefficients are the vertex values, and zero
on the edge, face and volume functions) evaluated by the field node equals
the coefficient v . x written with the point ops X, Y, Z, in the mass and
grad-grad terms and in the source."""
import ctypes as C

import numpy as np
import pytest

from test_tensor_coef import const_expr


def set_code(femg, ex, code, arrays=()):
    ex.n_code = len(code)
    for i, (op, arg, re, im) in enumerate(code):
        ins = ex.code[i]
        ins.op, ins.arg, ins.re, ins.im = op, arg, re, im
    ex.n_arrays = len(arrays)
    for k, arr in enumerate(arrays):
        ex.elem_values[k] = arr.ctypes.data_as(C.POINTER(C.c_double))


def linear_code(femg, v):
    """v . x with the point ops"""
    O = femg
    return [(O.FG_OP_CONST, 0, v[0], 0.0), (O.FG_OP_X, 0, 0.0, 0.0), (O.FG_OP_MUL, 0, 0.0, 0.0),
            (O.FG_OP_CONST, 0, v[1], 0.0), (O.FG_OP_Y, 0, 0.0, 0.0), (O.FG_OP_MUL, 0, 0.0, 0.0), (O.FG_OP_ADD, 0, 0.0, 0.0),
            (O.FG_OP_CONST, 0, v[2], 0.0), (O.FG_OP_Z, 0, 0.0, 0.0), (O.FG_OP_MUL, 0, 0.0, 0.0), (O.FG_OP_ADD, 0, 0.0, 0.0)]


def element_values(prob, a, dof_value):
    """[E][nb][2] field values at the elements' local DOFs from a function of
    the global DOF (num_type, entity, num_dof, assemble_type)."""
    rd = prob.raw_dofs()
    edof = a["edof"].astype(np.int64)
    etype = a["etype"]
    E, n = edof.shape
    by_row, by_fixed = {}, {}
    for k in range(len(rd["num_dof"])):
        at = int(rd["assemble_type"][k])
        val = dof_value(int(rd["num_type"][k]), int(rd["entity"][k]))
        if at in (2, 3):
            by_row[int(rd["num_dof"][k]) - 1] = val
        elif at == 1:
            by_fixed[int(rd["num_dof"][k]) - 1] = val
    u = np.zeros((E, n, 2))
    for e in range(E):
        for j in range(n):
            t = int(etype[e, j])
            val = by_row.get(int(edof[e, j]), 0.0) if t in (2, 3) else by_fixed.get(int(edof[e, j]), 0.0) if t == 1 else 0.0
            u[e, j, 0] = np.real(val)
            u[e, j, 1] = np.imag(val)
    return np.ascontiguousarray(u)


def linear_field(prob, a, v):
    xyz = a["xyz"]
    return element_values(prob, a, lambda nt, ent: float(xyz[ent - 1] @ v) if nt == 0 else 0.0)


def problem(femg, order=2, m=2):
    return femg.Problem(femg.config(dim=3, m=m, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=order, gauss=2 * order + 2,
                                    jitter=0.15, seed=3))


def field_terms(femg, prob, code_of, arrays, source=True):
    """The problem's grad-grad and mass terms with coefficients code_of(kind)
    (and a source with code_of(SOURCE))."""
    t, nt = prob.terms()
    keep = [i for i in range(nt) if t[i].kind in (femg.FG_TERM_GRAD_GRAD, femg.FG_TERM_MASS)]
    n = len(keep) + (1 if source else 0)
    arr = (femg.TermDesc * n)()
    for k, i in enumerate(keep):
        C.memmove(C.byref(arr[k]), C.byref(t[i]), C.sizeof(femg.TermDesc))
        set_code(femg, arr[k].coef, code_of(int(t[i].kind)), arrays)
    if source:
        s = arr[n - 1]
        s.kind, s.dt = femg.FG_TERM_SOURCE, 0
        set_code(femg, s.coef, code_of(femg.FG_TERM_SOURCE), arrays)
    return arr, n


@pytest.mark.parametrize("order", [1, 2, 3])
def test_linear_field_equals_point_coefficient(femg, oracle, order):
    prob = problem(femg, order)
    a = prob.arrays()
    v = np.array([0.7, -1.3, 2.1])
    u = linear_field(prob, a, v)
    O = femg
    # mass and source: u; grad-grad: 1 + u^2
    fcode = {O.FG_TERM_MASS: [(O.FG_OP_FIELD, 0, 0.0, 0.0)],
             O.FG_TERM_SOURCE: [(O.FG_OP_FIELD, 0, 0.0, 0.0)],
             O.FG_TERM_GRAD_GRAD: [(O.FG_OP_CONST, 0, 1.0, 0.0), (O.FG_OP_FIELD, 0, 0.0, 0.0), (O.FG_OP_FIELD, 0, 0.0, 0.0),
                                   (O.FG_OP_MUL, 0, 0.0, 0.0), (O.FG_OP_ADD, 0, 0.0, 0.0)]}
    lin = linear_code(femg, v)
    pcode = {O.FG_TERM_MASS: lin, O.FG_TERM_SOURCE: lin,
             O.FG_TERM_GRAD_GRAD: [(O.FG_OP_CONST, 0, 1.0, 0.0)] + lin + lin + [(O.FG_OP_MUL, 0, 0.0, 0.0), (O.FG_OP_ADD, 0, 0.0, 0.0)]}
    t1, n1 = field_terms(femg, prob, lambda k: fcode[k], [u])
    t2, n2 = field_terms(femg, prob, lambda k: pcode[k], [])
    v1, b1 = oracle.assemble(a, t1, n1)
    v2, b2 = oracle.assemble(a, t2, n2)
    assert np.abs(v1 - v2).max() <= 1e-12 * np.abs(v2).max()
    assert np.abs(b1 - b2).max() <= 1e-12 * np.abs(b2).max()


def test_const_field_is_a_constant(femg, oracle):
    """u_e[j] = 1 on the vertex functions is the constant 1 (partition of unity)."""
    prob = problem(femg, 2)
    a = prob.arrays()
    u = element_values(prob, a, lambda nt, ent: 1.0 if nt == 0 else 0.0)
    O = femg
    t1, n1 = field_terms(femg, prob, lambda k: [(O.FG_OP_CONST, 0, 3.0, 0.5), (O.FG_OP_FIELD, 0, 0.0, 0.0),
                                                (O.FG_OP_MUL, 0, 0.0, 0.0)], [u])
    t2, n2 = field_terms(femg, prob, lambda k: [(O.FG_OP_CONST, 0, 3.0, 0.5)], [])
    v1, b1 = oracle.assemble(a, t1, n1)
    v2, b2 = oracle.assemble(a, t2, n2)
    assert np.abs(v1 - v2).max() <= 1e-12 * np.abs(v2).max()
    assert np.abs(b1 - b2).max() <= 1e-12 * np.abs(b2).max()
