"""Jacobian modificators on the GPU FP64 path against the oracle (1e-12
relative Frobenius): every shell kind and the axisymmetric measure, terms
with and without a modificator in one assembly (two groups of integration
passes), a source term (the linear term uses the modified determinant),
HCurl and compound (elastic) fields, the shell-radius error, and the paths
that decline modificators."""
import ctypes as C

import numpy as np
import pytest

from test_jacmod import SHELLS, SQ, jm_problem

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def set_jm(femg, term, kind, axis=0, exponent=1, center=(0.0, 0.0, 0.0), r_min=1.5, r_max=4.0):
    j = term.jacmod
    j.kind, j.axis, j.exponent, j.r_min, j.r_max = kind, axis, exponent, r_min, r_max
    for c in range(3):
        j.center[c] = center[c]


def copy_terms(femg, prob, source=False):
    t, nt = prob.terms()
    extra = 1 if source else 0
    arr = (femg.TermDesc * (nt + extra))()
    for k in range(nt):
        C.memmove(C.byref(arr[k]), C.byref(t[k]), C.sizeof(femg.TermDesc))
    if source:  # f = 1 + x y
        s = arr[nt]
        s.kind, s.dt = femg.FG_TERM_SOURCE, 0
        code = [(femg.FG_OP_CONST, 0, 1.0, 0.0), (femg.FG_OP_X, 0, 0.0, 0.0), (femg.FG_OP_Y, 0, 0.0, 0.0),
                (femg.FG_OP_MUL, 0, 0.0, 0.0), (femg.FG_OP_ADD, 0, 0.0, 0.0)]
        for i, (op, arg, re, im) in enumerate(code):
            s.coef.code[i].op, s.coef.code[i].arg, s.coef.code[i].re, s.coef.code[i].im = op, arg, re, im
        s.coef.n_code = len(code)
    return arr, nt + extra


CASES = dict(SHELLS, axisymmetry=(2, "FG_JACMOD_AXISYMMETRY", {}))


@pytest.mark.parametrize("case", list(CASES))
def test_fp64_matches_oracle(femg, oracle, cuda, case):
    dim, name, p = CASES[case]
    kind = getattr(femg, name)
    prob = jm_problem(femg, dim, 10 if dim == 2 else 4, gauss=6)
    a = prob.arrays()
    t, nt = copy_terms(femg, prob, source=True)
    for k in range(nt):
        set_jm(femg, t[k], kind, **(dict(p, **SQ) if p else {}))
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64", terms=(t, nt))
    assert rel(v, ref_v) <= TOL and rel(b, ref_b) <= TOL
    # the factored FP64 method does not apply: it falls back to the quadrature loop
    plan.set_fp64_method(femg.FG_FP64_FACTORED)
    v2, _ = plan.assemble("fp64", terms=(t, nt))
    assert np.array_equal(v2.view(np.uint64), v.view(np.uint64))
    with pytest.raises(femg.FgError) as err:
        plan.assemble("mixed", terms=(t, nt))
    assert err.value.status == femg.FG_ERR_UNSUPPORTED


def test_terms_with_different_modificators(femg, oracle, cuda):
    """grad-grad on a spherical shell, the mass term plain, the source on the
    axisymmetric measure: three groups of integration passes."""
    prob = jm_problem(femg, 3, 4, gauss=6)
    a = prob.arrays()
    t, nt = copy_terms(femg, prob, source=True)
    for k in range(nt):
        if t[k].kind == femg.FG_TERM_GRAD_GRAD:
            set_jm(femg, t[k], femg.FG_JACMOD_SPHERICAL_SHELL, center=(-2.0, 0.5, 0.5))
        elif t[k].kind == femg.FG_TERM_SOURCE:
            set_jm(femg, t[k], femg.FG_JACMOD_AXISYMMETRY)
    ref_v, ref_b = oracle.assemble(a, t, nt)
    v, b = prob.plan().assemble("fp64", terms=(t, nt))
    assert rel(v, ref_v) <= TOL and rel(b, ref_b) <= TOL


def test_hcurl_and_elastic_on_a_shell(femg, oracle, cuda):
    mx = femg.Problem(femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=3, m=3, mesh_order=1, space=femg.FG_SPACE_HCURL, order=0,
                                  gauss=4, jitter=0.15, seed=7, k=3.0))
    nv = femg.Problem(femg.config_c5(m=2))
    for prob in (mx, nv):
        a = prob.arrays()
        t, nt = copy_terms(femg, prob)
        for k in range(nt):
            set_jm(femg, t[k], femg.FG_JACMOD_CYLINDRICAL_SHELL, axis=2, center=(-2.0, 0.5, 0.0))
        ref_v, _ = oracle.assemble(a, t, nt)
        v, _ = prob.plan().assemble("fp64", terms=(t, nt))
        assert rel(v, ref_v) <= TOL


def test_point_outside_the_shell(femg, oracle, cuda):
    prob = jm_problem(femg, 2, 6, gauss=4)
    t, nt = copy_terms(femg, prob)
    for k in range(nt):
        set_jm(femg, t[k], femg.FG_JACMOD_POLAR_SHELL, center=(-2.0, 0.5, 0.0), r_min=1.5, r_max=2.5)
    plan = prob.plan()
    with pytest.raises(femg.FgError) as err:
        plan.assemble("fp64", terms=(t, nt))
    assert err.value.status == femg.FG_ERR_ARG
    assert b"outside the shell" in femg.lib().fg_last_error()
    # the plan stays usable
    t2, nt2 = prob.terms()
    ref_v, _ = oracle.assemble(prob.arrays(), t2, nt2)
    v, _ = plan.assemble("fp64")
    assert rel(v, ref_v) <= TOL


def test_batches_decline_modificators(femg, cuda):
    prob = jm_problem(femg, 2, 4, gauss=4)
    t, nt = copy_terms(femg, prob)
    set_jm(femg, t[0], femg.FG_JACMOD_AXISYMMETRY)
    plan = prob.plan()
    L = femg.lib()
    plans = (C.c_void_p * 1)(plan.ptr)
    tl = (C.POINTER(femg.TermDesc) * 1)(C.cast(t, C.POINTER(femg.TermDesc)))
    nts = (C.c_int32 * 1)(nt)
    out = C.c_void_p()
    assert L.fg_batch_create(plans, tl, nts, 1, 0, C.byref(out)) == femg.FG_ERR_UNSUPPORTED


@pytest.mark.parametrize("bad", ["kind", "radii", "axis", "exponent"])
def test_invalid_modificator_arguments(femg, cuda, bad):
    prob = jm_problem(femg, 3, 2, gauss=4)
    t, nt = copy_terms(femg, prob)
    args = dict(center=(-2.0, 0.5, 0.5))
    if bad == "kind":
        set_jm(femg, t[0], 9, **args)
    elif bad == "radii":
        set_jm(femg, t[0], femg.FG_JACMOD_SPHERICAL_SHELL, r_min=3.0, r_max=2.0, **args)
    elif bad == "axis":
        set_jm(femg, t[0], femg.FG_JACMOD_CYLINDRICAL_SHELL, axis=3, **args)
    else:
        set_jm(femg, t[0], femg.FG_JACMOD_POLAR_SHELL, exponent=-1, **args)
    with pytest.raises(femg.FgError) as err:
        prob.plan().assemble("fp64", terms=(t, nt))
    assert err.value.status == femg.FG_ERR_ARG
