"""The coefficient language's scalar operators on the GPU FP64 path against
the oracle (which test_coef_ops.py pins to the reference's own expression
trees): mass and source terms with the operator applied to a complex,
point-dependent argument, to 1e-12 relative Frobenius. And one element-
constant coefficient through an operator on the mixed paths (split and
fused), to the mixed tolerance."""
import ctypes as C

import numpy as np
import pytest

from coef_programs import OPS, configs, set_expr, terms

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("geom", ["tri_p2", "tet_h1_p2"])
@pytest.mark.parametrize("op", OPS)
def test_gpu_operator_matches_oracle(femg, oracle, cuda, geom, op):
    prob = femg.Problem(configs(femg)[geom])
    a = prob.arrays()
    t, nt, _ = terms(femg, op)
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64", terms=(t, nt))
    assert rel(v, ref_v) <= 1e-12, rel(v, ref_v)
    assert rel(b, ref_b) <= 1e-12, rel(b, ref_b)


@pytest.mark.parametrize("fused", [True, False])
def test_mixed_element_coefficient_through_operators(femg, oracle, cuda, fused):
    """c_e = -k^2 exp(0.1 sqrt(w_e)) with w_e > 0 per element: real, constant
    per element, so the tensor-core paths take it."""
    prob = femg.Problem(femg.config_c2(m=4))
    a = prob.arrays()
    E = int(a["E"])
    w = np.ascontiguousarray(np.stack([np.linspace(0.5, 2.0, E), np.zeros(E)], axis=1))
    t0, n0 = prob.terms()
    arr = (femg.TermDesc * n0)()
    for k in range(n0):
        C.memmove(C.byref(arr[k]), C.byref(t0[k]), C.sizeof(femg.TermDesc))
    mass = [k for k in range(n0) if arr[k].kind == femg.FG_TERM_MASS][0]
    set_expr(arr[mass].coef, [(femg.FG_OP_ELEM, 0, 0, 0), (femg.FG_OP_SQRT, 0, 0, 0), (femg.FG_OP_CONST, 0, 0.1, 0.0),
                              (femg.FG_OP_MUL, 0, 0, 0), (femg.FG_OP_EXP, 0, 0, 0), (femg.FG_OP_CONST, 0, -400.0, 0.0),
                              (femg.FG_OP_MUL, 0, 0, 0)])
    arr[mass].coef.n_arrays = 1
    arr[mass].coef.elem_values[0] = w.ctypes.data_as(C.POINTER(C.c_double))
    ref_v, _ = oracle.assemble(a, arr, n0)
    plan = prob.plan()
    plan.set_mixed_fused(fused)
    v, _ = plan.assemble("mixed", terms=(arr, n0))
    assert rel(v, ref_v) <= 1e-6
    v64, _ = plan.assemble("fp64", terms=(arr, n0))
    assert rel(v64, ref_v) <= 1e-12
