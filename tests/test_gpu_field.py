"""Field-node coefficients (FG_OP_FIELD) on the GPU against the oracle: the
FP64 path with complex field values in the grad-grad, mass, source, tensor
and elastic terms (1e-12 relative Frobenius), the tensor-core path (field
sources; bilinear field coefficients are refused), the argument checks, and
coefficient buffers reused across calls with arrays of different sizes."""
import ctypes as C

import numpy as np
import pytest

from test_field_coef import field_terms, problem
from test_tensor_coef import tensor_terms

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def random_field(a, seed=1, cplx=True):
    E, n = a["edof"].shape
    rng = np.random.default_rng(seed)
    u = np.zeros((E, n, 2))
    u[:, :, 0] = 1.0 + 0.5 * rng.random((E, n))
    if cplx:
        u[:, :, 1] = 0.3 * rng.standard_normal((E, n))
    return np.ascontiguousarray(u)


def times_field(femg, ex, u):
    """ex <- ex * field(u)"""
    k, n = ex.n_arrays, ex.n_code
    ex.code[n].op, ex.code[n].arg = femg.FG_OP_FIELD, k
    ex.code[n + 1].op = femg.FG_OP_MUL
    ex.n_code = n + 2
    ex.elem_values[k] = u.ctypes.data_as(C.POINTER(C.c_double))
    ex.n_arrays = k + 1


def copy_terms(femg, prob):
    t, nt = prob.terms()
    arr = (femg.TermDesc * nt)()
    for k in range(nt):
        C.memmove(C.byref(arr[k]), C.byref(t[k]), C.sizeof(femg.TermDesc))
    return arr, nt


@pytest.mark.parametrize("order", [1, 2, 3])
def test_fp64_field_coefficients(femg, oracle, cuda, order):
    prob = problem(femg, order)
    a = prob.arrays()
    u = random_field(a)
    O = femg
    code = {O.FG_TERM_MASS: [(O.FG_OP_FIELD, 0, 0.0, 0.0)],
            O.FG_TERM_SOURCE: [(O.FG_OP_CONST, 0, 2.0, 0.0), (O.FG_OP_FIELD, 0, 0.0, 0.0), (O.FG_OP_MUL, 0, 0.0, 0.0)],
            O.FG_TERM_GRAD_GRAD: [(O.FG_OP_FIELD, 0, 0.0, 0.0), (O.FG_OP_FIELD, 0, 0.0, 0.0), (O.FG_OP_MUL, 0, 0.0, 0.0)]}
    t, nt = field_terms(femg, prob, lambda k: code[k], [u])
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64", terms=(t, nt))
    assert rel(v, ref_v) <= FP64_TOL and rel(b, ref_b) <= FP64_TOL
    # bilinear field coefficients depend on the point: not on the tensor-core path
    with pytest.raises(femg.FgError) as err:
        plan.assemble("mixed", terms=(t, nt))
    assert err.value.status == femg.FG_ERR_UNSUPPORTED


def test_mixed_with_field_source(femg, oracle, cuda):
    """Constant bilinear coefficients, a field-valued source: the right-hand
    side is integrated in FP64 on the tensor-core path too."""
    prob = problem(femg, 2, m=3)
    a = prob.arrays()
    u = random_field(a, seed=2)
    O = femg
    code = {O.FG_TERM_MASS: [(O.FG_OP_CONST, 0, -4.0, 0.0)], O.FG_TERM_GRAD_GRAD: [(O.FG_OP_CONST, 0, 1.0, 0.0)],
            O.FG_TERM_SOURCE: [(O.FG_OP_FIELD, 0, 0.0, 0.0)]}
    t, nt = field_terms(femg, prob, lambda k: code[k], [u])
    ref_v, ref_b = oracle.assemble(a, t, nt)
    v, b = prob.plan().assemble("mixed", terms=(t, nt))
    lifted = a["n_fixed"] > 0 and np.any(a["dirichlet"] != 0)  # the lifting uses the mixed element matrices
    assert rel(v, ref_v) <= MIXED_TOL and rel(b, ref_b) <= (MIXED_TOL if lifted else FP64_TOL)


def test_tensor_and_elastic_terms(femg, oracle, cuda):
    prob = problem(femg, 2)
    a = prob.arrays()
    u = random_field(a, seed=3, cplx=False)
    D = np.array([[2.0, 0.3, 0.1], [0.3, 1.5, -0.2], [0.1, -0.2, 1.0]])
    t, nt = tensor_terms(femg, prob, D, c=None, keep_mass=True)
    tens = C.cast(t[0].tensor, C.POINTER(femg.Expr * 6)).contents
    times_field(femg, tens[0], u)  # D_xx u(x)
    times_field(femg, t[1].coef, u)  # mass c u(x)
    ref_v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    v, _ = prob.plan().assemble("fp64", terms=(t, nt), rhs=False)
    assert rel(v, ref_v) <= FP64_TOL
    # Navier (3 components): lambda, mu and the mass times a field of the scalar basis
    nav = femg.Problem(femg.config(kind=femg.FG_PROBLEM_NAVIER, dim=3, m=2, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1,
                                   order=1, gauss=4, jitter=0.15, seed=9, omega=2.0, lame_sigma=0.5))
    na = nav.arrays()
    E, n = na["edof"].shape
    un = np.ascontiguousarray(random_field(dict(edof=np.zeros((E, n // 3))), seed=4))
    tn, ntn = copy_terms(femg, nav)
    for k in range(ntn):
        times_field(femg, tn[k].coef, un)
        if tn[k].kind == femg.FG_TERM_ELASTIC:
            times_field(femg, tn[k].coef2, un)
    ref_v, _ = oracle.assemble(na, tn, ntn, with_rhs=False)
    v, _ = nav.plan().assemble("fp64", terms=(tn, ntn), rhs=False)
    assert rel(v, ref_v) <= FP64_TOL


def test_argument_checks(femg, cuda):
    prob = problem(femg, 1)
    a = prob.arrays()
    u = random_field(a)
    O = femg
    # one array both per element and as field values
    t, nt = field_terms(femg, prob, lambda k: [(O.FG_OP_FIELD, 0, 0.0, 0.0), (O.FG_OP_ELEM, 0, 0.0, 0.0),
                                               (O.FG_OP_MUL, 0, 0.0, 0.0)], [u], source=False)
    with pytest.raises(femg.FgError) as err:
        prob.plan().assemble("fp64", terms=(t, nt), rhs=False)
    assert err.value.status == femg.FG_ERR_ARG
    # an HCurl bucket has no scalar basis to evaluate a field with
    mx = femg.Problem(femg.config(kind=femg.FG_PROBLEM_MAXWELL, dim=3, m=2, mesh_order=1, space=femg.FG_SPACE_HCURL, order=0,
                                  gauss=2, jitter=0.1, seed=3))
    tm, ntm = copy_terms(femg, mx)
    ma = mx.arrays()
    um = random_field(ma)
    times_field(femg, tm[0].coef, um)
    with pytest.raises(femg.FgError) as err:
        mx.plan().assemble("fp64", terms=(tm, ntm), rhs=False)
    assert err.value.status == femg.FG_ERR_UNSUPPORTED


def test_buffers_reused_across_array_sizes(femg, oracle, cuda):
    """Per-element arrays ([E]) and field arrays ([E][nb]) in turn on one plan:
    each call's device copies fit their arrays."""
    prob = femg.Problem(femg.config_c3(m=3))
    a = prob.arrays()
    plan = prob.plan()
    own, nown = prob.terms()
    ref_own, _ = oracle.assemble(a, own, nown, with_rhs=False)
    u = random_field(a, seed=5)
    tf, ntf = copy_terms(femg, prob)
    for k in range(ntf):
        times_field(femg, tf[k].coef, u)
    ref_f, _ = oracle.assemble(a, tf, ntf, with_rhs=False)
    for terms, ref in [((own, nown), ref_own), ((tf, ntf), ref_f), ((own, nown), ref_own), ((tf, ntf), ref_f)]:
        v, _ = plan.assemble("fp64", terms=terms, rhs=False)
        assert rel(v, ref) <= FP64_TOL


def test_batch_and_multi_frequency(femg, oracle, cuda):
    """Field coefficients through fg_batch (FP64; the mixed batch refuses
    them) and fg_assemble_multi_freq (mass with a second time derivative)."""
    prob = problem(femg, 2)
    a = prob.arrays()
    u = random_field(a, seed=6)
    O = femg
    code = {O.FG_TERM_MASS: [(O.FG_OP_FIELD, 0, 0.0, 0.0)], O.FG_TERM_GRAD_GRAD: [(O.FG_OP_CONST, 0, 1.0, 0.0)],
            O.FG_TERM_SOURCE: [(O.FG_OP_FIELD, 0, 0.0, 0.0)]}
    t, nt = field_terms(femg, prob, lambda k: code[k], [u])
    plan = prob.plan()
    femg.check(femg.lib().fg_plan_bind_terms(plan.ptr, t, nt, 0.0))
    ref_v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    vals, _ = femg.Batch([plan], mixed=False, bound=True).run()
    assert rel(vals[0], ref_v) <= FP64_TOL
    with pytest.raises(femg.FgError) as err:
        femg.Batch([plan], mixed=True, bound=True)
    assert err.value.status == femg.FG_ERR_UNSUPPORTED
    mass = [k for k in range(nt) if t[k].kind == femg.FG_TERM_MASS][0]
    t[mass].dt = femg.FG_DT_2
    omegas = [1.0, 2.5]
    mv, mr = plan.assemble_multi_freq(omegas, terms=(t, nt))
    for f, om in enumerate(omegas):
        rv, rb = oracle.assemble(a, t, nt, freq=om)
        assert rel(mv[f], rv) <= FP64_TOL and rel(mr[f], rb) <= FP64_TOL
