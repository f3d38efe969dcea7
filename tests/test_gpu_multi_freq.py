"""fg_assemble_multi_freq against the oracle assembled at each frequency
(AFrequency module: -omega^2 on dt2 terms, -i omega on dt terms) and against
the single-frequency GPU path. FP64: 1e-12 relative Frobenius; mixed: 1e-6."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6
OMEGAS = [1.5, 4.0, 7.25]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def with_dt(femg, prob, layout):
    """Copy of the problem's terms: layout = [(term index, dt), ...]."""
    t, nt = prob.terms()
    arr = (femg.TermDesc * len(layout))()
    for k, (src, dt) in enumerate(layout):
        C.memmove(C.byref(arr[k]), C.byref(t[src]), C.sizeof(femg.TermDesc))
        arr[k].dt = dt
    return arr, len(layout)


def problems(femg):
    navier = femg.Problem(femg.config_c5(m=2, omega=0.0))  # elastic (dt 0) + dt2 mass
    scalar = femg.Problem(femg.config_c3(m=3))             # grad-grad, per-element mass
    dirichlet = femg.Problem(femg.config_c1(m=8))          # + Dirichlet lifting and a source
    return {
        "navier_dt2": (navier, navier.terms()),
        "scalar_dt1_dt2": (scalar, with_dt(femg, scalar, [(0, 0), (1, 1), (1, 2)])),
        "dirichlet_source_dt2": (dirichlet, with_dt(femg, dirichlet, [(0, 0), (1, 2), (2, 0)])),
    }


@pytest.mark.parametrize("case", ["navier_dt2", "scalar_dt1_dt2", "dirichlet_source_dt2"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_freq_matches_oracle(femg, oracle, cuda, case, precision):
    prob, (t, nt) = problems(femg)[case]
    a = prob.arrays()
    plan = prob.plan()
    vals, rhs = plan.assemble_multi_freq(OMEGAS, precision=precision, terms=(t, nt))
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    lifted = a["n_fixed"] > 0 and np.any(a["dirichlet"] != 0)
    for f, w in enumerate(OMEGAS):
        ref_v, ref_b = oracle.assemble(a, t, nt, freq=w)
        assert rel(vals[f], ref_v) <= tol, (f, rel(vals[f], ref_v))
        if np.linalg.norm(ref_b) > 0:
            assert rel(rhs[f], ref_b) <= (tol if (precision == "fp64" or lifted) else FP64_TOL)
        if precision == "fp64":
            v1, b1 = plan.assemble("fp64", frequency=w, terms=(t, nt))
            assert rel(vals[f], v1) <= FP64_TOL
            assert rel(rhs[f], b1) <= FP64_TOL


def test_multi_freq_device_outputs_and_repeat(femg, cuda):
    torch = cuda
    prob = femg.Problem(femg.config_c5(m=2, omega=0.0))
    plan = prob.plan()
    F = len(OMEGAS)
    host_v, _ = plan.assemble_multi_freq(OMEGAS, precision="mixed")
    dv = torch.empty(F * 2 * prob.nnz, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        plan.assemble_multi_freq(OMEGAS, precision="mixed", values=dv.data_ptr(), rhs=False, stream=stream)
        torch.cuda.synchronize()
        v = dv.cpu().numpy().view(np.complex128).reshape(F, prob.nnz)
        assert np.array_equal(v.view(np.uint64), host_v.view(np.uint64))


def test_multi_freq_rejects(femg, cuda):
    prob = femg.Problem(femg.config_c3(m=2))
    plan = prob.plan()
    L = femg.lib()
    t, nt = prob.terms()
    om = np.array([1.0])
    v = np.zeros(prob.nnz, np.complex128)
    assert L.fg_assemble_multi_freq(plan.ptr, t, nt, om.ctypes.data, 0, 0, None, v.ctypes.data, None, None) == femg.FG_ERR_ARG
    bad, nb = with_dt(femg, prob, [(0, 0), (0, 1)])
    bad[1].kind = femg.FG_TERM_SOURCE
    assert L.fg_assemble_multi_freq(plan.ptr, bad, nb, om.ctypes.data, 1, 0, None, v.ctypes.data, None, None) == femg.FG_ERR_ARG
    assert b"time derivative" in L.fg_last_error()


@pytest.mark.parametrize("case", ["navier_dt2", "scalar_dt1_dt2", "dirichlet_source_dt2"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_separate_modules_match_oracle(femg, oracle, cuda, case, precision):
    """assemble(separate = true): K, C, M each from its own terms without the
    frequency factor; the right-hand side lifts with K alone."""
    prob, (t, nt) = problems(femg)[case]
    a = prob.arrays()
    plan = prob.plan()
    K, Cm, M, rhs = plan.assemble_separate(precision=precision, terms=(t, nt))
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    dts = [int(t[i].dt) for i in range(nt)]
    for d, got in zip((0, 1, 2), (K, Cm, M)):
        layout = [(i, 0) for i in range(nt) if dts[i] == d and t[i].kind != femg.FG_TERM_SOURCE]
        if not layout:
            assert got is None or np.all(got == 0)
            continue
        tt, nn = _copy_terms(femg, t, layout)
        ref_v, _ = oracle.assemble(a, tt, nn)
        assert rel(got, ref_v) <= tol, (d, rel(got, ref_v))
    # right-hand side: sources + lifting of K
    layout = [(i, 0) for i in range(nt) if dts[i] == 0]
    tt, nn = _copy_terms(femg, t, layout)
    _, ref_b = oracle.assemble(a, tt, nn)
    if np.linalg.norm(ref_b) > 0:
        lifted = a["n_fixed"] > 0 and np.any(a["dirichlet"] != 0)
        assert rel(rhs, ref_b) <= (tol if (precision == "fp64" or lifted) else FP64_TOL)


def _copy_terms(femg, t, layout):
    arr = (femg.TermDesc * len(layout))()
    for k, (src, dt) in enumerate(layout):
        C.memmove(C.byref(arr[k]), C.byref(t[src]), C.sizeof(femg.TermDesc))
        arr[k].dt = dt
    return arr, len(layout)
