"""The tensor diffusion term integral(c D grad(dof(u)), grad(tf(u))) on the
GPU against the oracle: the FP64 path (point-dependent tensors, complex
tensors, tets and second-order triangles; 1e-12 relative Frobenius), the
tensor-core path (per-element tensors; 1e-6), the separate K/M matrices, the batch, the
factored FP64 method's fallback and the argument checks."""
import ctypes as C

import numpy as np
import pytest

from test_tensor_coef import problems, tensor_terms

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def tensor(cplx, dim=3, seed=5):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((3, 3))
    D = M @ M.T + 2 * np.eye(3)
    if cplx:  # a PML-like stretching: complex diagonal plus a small coupling
        D = D + 1j * (np.diag([0.7, -0.4, 0.3]) + 0.05 * (M + M.T))
    if dim == 2:
        D[2, :] = D[:, 2] = 0.0
        D[2, 2] = 1.0
    return D


@pytest.mark.parametrize("name", ["tet_p1", "tet_p2", "tri_p2"])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("point", [False, True])
def test_fp64_matches_oracle(femg, oracle, cuda, name, cplx, point):
    prob = problems(femg)[name]
    a = prob.arrays()
    t, nt = tensor_terms(femg, prob, tensor(cplx, int(a["dim"])), c=None, keep_mass=True, point_xx=point)
    ref_v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    plan = prob.plan()
    v, _ = plan.assemble("fp64", terms=(t, nt), rhs=False)
    assert rel(v, ref_v) <= FP64_TOL
    # the factored FP64 method does not take tensors: same values as the quadrature loop
    plan.set_fp64_method(femg.FG_FP64_FACTORED)
    v2, _ = plan.assemble("fp64", terms=(t, nt), rhs=False)
    assert np.array_equal(v2.view(np.uint64), v.view(np.uint64))
    if point:
        # point-dependent tensors stay on the FP64 path
        with pytest.raises(femg.FgError) as err:
            plan.assemble("mixed", terms=(t, nt), rhs=False)
        assert err.value.status == femg.FG_ERR_UNSUPPORTED
    else:
        vm, _ = plan.assemble("mixed", terms=(t, nt), rhs=False)
        assert rel(vm, ref_v) <= MIXED_TOL


@pytest.mark.parametrize("name", ["tet_p1", "tet_p2"])
@pytest.mark.parametrize("cplx", [False, True])
def test_mixed_matches_oracle(femg, oracle, cuda, name, cplx):
    prob = problems(femg)[name]
    a = prob.arrays()
    t, nt = tensor_terms(femg, prob, tensor(cplx), c=None, keep_mass=True)
    ref_v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    v, _, rep = prob.plan().assemble("mixed", terms=(t, nt), rhs=False, report=True)
    assert rel(v, ref_v) <= MIXED_TOL
    assert rep["global_"] <= MIXED_TOL and rep["max_elem"] <= 10 * MIXED_TOL


def test_c3_sized_mixed_against_fp64(femg, cuda):
    """Order-3 tets with a per-element coefficient times an anisotropic tensor:
    the tensor-core path against the FP64 path on 24,000 elements."""
    prob = femg.Problem(femg.config_c3(m=20))
    t, nt = tensor_terms(femg, prob, tensor(True), c=None, keep_mass=True)
    plan = prob.plan()
    v64, _ = plan.assemble("fp64", terms=(t, nt), rhs=False)
    vm, _ = plan.assemble("mixed", terms=(t, nt), rhs=False)
    assert rel(vm, v64) <= MIXED_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_separate_matrices(femg, oracle, cuda, precision):
    """The tensor term in K (no time derivative), the mass term in M (second
    derivative): each matrix against the oracle of its own terms."""
    prob = problems(femg)["tet_p2"]
    a = prob.arrays()
    t, nt = tensor_terms(femg, prob, tensor(False), c=None, keep_mass=True)
    t[1].dt = femg.FG_DT_2
    K, Cm, M, _ = prob.plan().assemble_separate(precision, terms=(t, nt), with_rhs=False)
    assert Cm is None
    ref_k, _ = oracle.assemble(a, t, 1, with_rhs=False)
    tm = (femg.TermDesc * 1)()
    C.memmove(C.byref(tm[0]), C.byref(t[1]), C.sizeof(femg.TermDesc))
    tm[0].dt = femg.FG_DT_NONE
    ref_m, _ = oracle.assemble(a, tm, 1, with_rhs=False)
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    assert rel(K, ref_k) <= tol and rel(M, ref_m) <= tol


@pytest.mark.parametrize("mixed", [False, True])
def test_batch(femg, oracle, cuda, mixed):
    probs = problems(femg)
    names = ["tet_p1", "tet_p2"]
    plans, terms, refs = [], [], []
    for k, name in enumerate(names):
        prob = probs[name]
        t, nt = tensor_terms(femg, prob, tensor(k == 1, seed=7 + k), c=None, keep_mass=True)
        plan = prob.plan()
        femg.check(femg.lib().fg_plan_bind_terms(plan.ptr, t, nt, 0.0))
        refs.append(oracle.assemble(prob.arrays(), t, nt, with_rhs=False)[0])
        plans.append(plan)
        terms.append(t)
    batch = femg.Batch(plans, mixed=mixed, bound=True)
    vals, _ = batch.run()
    tol = MIXED_TOL if mixed else FP64_TOL
    for v, r in zip(vals, refs):
        assert rel(v, r) <= tol


def test_argument_checks(femg, cuda):
    prob = problems(femg)["tet_p1"]
    plan = prob.plan()
    t, nt = tensor_terms(femg, prob, np.eye(3))
    t[0].tensor = None
    with pytest.raises(femg.FgError) as err:
        plan.assemble("fp64", terms=(t, nt), rhs=False)
    assert err.value.status == femg.FG_ERR_ARG
    # two tensor terms in one assembly
    t2, _ = tensor_terms(femg, prob, np.eye(3))
    both = (femg.TermDesc * 2)()
    for k in range(2):
        C.memmove(C.byref(both[k]), C.byref(t2[0]), C.sizeof(femg.TermDesc))
    with pytest.raises(femg.FgError) as err:
        plan.assemble("fp64", terms=(both, 2), rhs=False)
    assert err.value.status == femg.FG_ERR_ARG
    # a compound (3-component) field does not take the tensor term
    nav = femg.Problem(femg.config(kind=femg.FG_PROBLEM_NAVIER, dim=3, m=2, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1,
                                   order=1, gauss=2, jitter=0.15, seed=9, omega=2.0, lame_sigma=0.5))
    nt_, nnt = nav.terms()
    tt = (femg.TermDesc * 1)()
    C.memmove(C.byref(tt[0]), C.byref(nt_[0]), C.sizeof(femg.TermDesc))
    tt[0].kind = femg.FG_TERM_GRAD_GRAD_TENSOR
    tt[0].tensor = t2[0].tensor
    with pytest.raises(femg.FgError) as err:
        nav.plan().assemble("fp64", terms=(tt, 1), rhs=False)
    assert err.value.status == femg.FG_ERR_UNSUPPORTED
