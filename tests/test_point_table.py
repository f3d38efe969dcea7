"""Point tables (FG_OP_POINT): a coefficient given by its value at every
integration point of the bucket, element-major, as a caller fills it with the
reference's own evaluator (EquationEvaluator::initialize,
src/term/evaluator/EquationEvaluator.h:155-168) when it does not describe the
Function. The oracle's assembly with the table of a point-dependent program
equals its assembly with the program itself (mass and source terms, one and
two tables per term)."""
import ctypes as C

import numpy as np
import pytest

from coef_programs import argument, configs, set_expr


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def points(a):
    """physical integration points [E][nq][3] of an arrays() dict"""
    X = a["xyz"][a["enodes"].astype(np.int64)]  # [E][nn][3]
    return np.einsum("qk,ekc->eqc", a["geo_val"], X)


def argument_values(x):
    """a(x, y) = 0.4 + 0.3 x + 0.2 y + 0.1 i (x - y), as coef_programs.argument"""
    return 0.4 + 0.3 * x[..., 0] + 0.2 * x[..., 1] + 0.1j * (x[..., 0] - x[..., 1])


def tables_terms(F, a, split):
    """(program terms, table terms, keep-alive): mass m = a and source f = a / 2,
    each once as the program and once as point tables (split: the table in
    two halves added by the program)"""
    x = points(a)
    val = argument_values(x).reshape(-1)
    keep = []

    def table(v):
        t = np.ascontiguousarray(np.stack([v.real, v.imag], 1).reshape(-1))
        keep.append(t)
        return t

    prog = (F.TermDesc * 2)()
    tab = (F.TermDesc * 2)()
    for arr in (prog, tab):
        for t in arr:
            C.memset(C.byref(t), 0, C.sizeof(F.TermDesc))
        arr[0].kind, arr[1].kind = F.FG_TERM_MASS, F.FG_TERM_SOURCE
    code = argument(F)
    set_expr(prog[0].coef, code)
    set_expr(prog[1].coef, code + [(F.FG_OP_CONST, 0, 0.5, 0.0), (F.FG_OP_MUL, 0, 0, 0)])
    for k, scale in ((0, 1.0), (1, 0.5)):
        ex = tab[k].coef
        if split:
            set_expr(ex, [(F.FG_OP_POINT, 0, 0, 0), (F.FG_OP_POINT, 1, 0, 0), (F.FG_OP_ADD, 0, 0, 0)])
            ex.n_arrays = 2
            ex.elem_values[0] = table(0.25 * scale * val).ctypes.data_as(C.POINTER(C.c_double))
            ex.elem_values[1] = table(0.75 * scale * val).ctypes.data_as(C.POINTER(C.c_double))
        else:
            set_expr(ex, [(F.FG_OP_POINT, 0, 0, 0)])
            ex.n_arrays = 1
            ex.elem_values[0] = table(scale * val).ctypes.data_as(C.POINTER(C.c_double))
    return prog, tab, keep


@pytest.mark.parametrize("geom", ["tri_p2", "tet_h1_p2"])
@pytest.mark.parametrize("split", [False, True])
def test_point_table_equals_program(femg, oracle, geom, split):
    prob = femg.Problem(configs(femg)[geom])
    a = prob.arrays()
    prog, tab, keep = tables_terms(femg, a, split)
    vp, bp = oracle.assemble(a, prog, 2)
    vt, bt = oracle.assemble(a, tab, 2)
    assert rel(vt, vp) <= 1e-13 and rel(bt, bp) <= 1e-13
    assert np.abs(vp).max() > 0 and np.abs(bp).max() > 0
