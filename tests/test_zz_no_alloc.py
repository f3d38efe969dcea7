"""fg_assemble_fp64_static: the FP64 assembly for callers that may not
allocate device memory once set up (a solver that owns the device memory
pool, or one that overlaps this step's assembly with the previous step's
solve and cannot afford the device-wide synchronisation of cudaFree). Its
element scratch is a fixed device array inside the library.

Each case makes a fresh plan that is only bound (no assemble call before),
calls the static entry three times in a row, and checks
  * every result against the oracle and against fg_assemble_fp64 on a second
    plan of the same problem, at the FP64 tolerance;
  * that the device's free memory does not change across the second and
    third calls (the first call of a process may load the array itself);
with the quadrature method, the factored method and a Jacobian modificator.
Collected last so that it also runs after every other GPU test in the same
process."""
import ctypes as C

import numpy as np
import pytest

from test_jacmod import SHELLS, SQ, jm_problem

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
STATIC_BYTES = 64 << 20


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _outputs(femg, torch, prob, with_rhs=True):
    nnz, nrows = prob.nnz, int(prob.sys.n_rows)
    dv = torch.full((2 * nnz,), float("nan"), dtype=torch.float64, device="cuda")
    db = torch.full((2 * nrows,), float("nan"), dtype=torch.float64, device="cuda") if with_rhs else None
    dd = None
    if prob.sys.n_fixed:
        a = prob.arrays()
        dd = torch.from_numpy(np.ascontiguousarray(a["dirichlet"]).view(np.float64).copy()).cuda()
    torch.cuda.synchronize()
    return dv, db, dd


def _static_calls(femg, torch, plan, prob, with_rhs=True, calls=3):
    """`calls` static calls in a row into preallocated device outputs; returns
    the results of each call and the free device bytes after the first call
    and after the last. The first call of a process on a device may load the
    library's code module that holds the scratch array (64 MiB of device
    memory, kept until exit); the calls after it must change nothing."""
    dv, db, dd = _outputs(femg, torch, prob, with_rhs)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = []
    free0 = None
    for k in range(calls):
        if k == 1:
            free0 = torch.cuda.mem_get_info()[0]
        dv.fill_(float("nan"))
        if db is not None:
            db.fill_(float("nan"))
        st = femg.lib().fg_assemble_fp64_static(plan.ptr, dd.data_ptr() if dd is not None else None, dv.data_ptr(),
                                                db.data_ptr() if db is not None else None, stream)
        torch.cuda.synchronize()
        assert st == femg.FG_OK, femg.lib().fg_last_error()
        out.append((dv.cpu().numpy().view(np.complex128).copy(),
                    db.cpu().numpy().view(np.complex128).copy() if db is not None else None))
    free1 = torch.cuda.mem_get_info()[0]
    return out, free0, free1


def _check(v, b, ref_v, ref_b):
    assert rel(v, ref_v) <= FP64_TOL
    if b is None:
        return
    if np.linalg.norm(ref_b) > 0:
        assert rel(b, ref_b) <= FP64_TOL
    else:
        assert np.all(b == 0)


CASES = {"c3_m4": ("config_c3", dict(m=4)), "c1_m8": ("config_c1", dict(m=8)), "c5_m2": ("config_c5", dict(m=2))}


@pytest.mark.parametrize("method", ["quadrature", "factored"])
@pytest.mark.parametrize("case", list(CASES))
def test_static_matches_oracle_and_fp64_twice(femg, oracle, cuda, case, method):
    torch = cuda
    fn, kw = CASES[case]
    prob = femg.Problem(getattr(femg, fn)(**kw))
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(a, t, nt)
    other = prob.plan()  # fg_assemble_fp64 on a second plan
    v64, b64 = other.assemble("fp64")
    plan = prob.plan()  # fresh: bound, never assembled
    if method == "factored":
        plan.set_fp64_method(femg.FG_FP64_FACTORED)
    plan.bind_terms()
    out, free0, free1 = _static_calls(femg, torch, plan, prob)
    assert free0 == free1, "device memory changed across the static calls: %d -> %d" % (free0, free1)
    for v, b in out:
        _check(v, b, ref_v, ref_b)
        _check(v, b, v64, b64)
    plan.close()
    other.close()


def test_static_jacobian_modificator(femg, oracle, cuda):
    """A spherical shell on every term: the element kernel's shell-radius
    check reads a device word back, which allocates nothing either."""
    torch = cuda
    from test_gpu_jacmod import copy_terms, set_jm
    prob = jm_problem(femg, 3, 4, gauss=6)
    a = prob.arrays()
    t, nt = copy_terms(femg, prob, source=True)
    for k in range(nt):
        set_jm(femg, t[k], femg.FG_JACMOD_SPHERICAL_SHELL, **dict(SHELLS["spherical"][2], **SQ))
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    assert femg.lib().fg_plan_bind_terms(plan.ptr, t, nt, 0.0) == femg.FG_OK, femg.lib().fg_last_error()
    out, free0, free1 = _static_calls(femg, torch, plan, prob)
    assert free0 == free1
    for v, b in out:
        _check(v, b, ref_v, ref_b)
    plan.close()


def test_static_without_rhs(femg, oracle, cuda):
    torch = cuda
    prob = femg.Problem(femg.config_c3(m=3))
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(prob.arrays(), t, nt)
    plan = prob.plan()
    plan.bind_terms()
    out, free0, free1 = _static_calls(femg, torch, plan, prob, with_rhs=False)
    assert free0 == free1
    for v, _ in out:
        assert rel(v, ref_v) <= FP64_TOL


def test_static_rejects(femg, cuda):
    torch = cuda
    L = femg.lib()
    prob = femg.Problem(femg.config_c3(m=3))
    plan = prob.plan()
    dv = torch.zeros(2 * prob.nnz, dtype=torch.float64, device="cuda")
    # no bound terms
    assert L.fg_assemble_fp64_static(plan.ptr, None, dv.data_ptr(), None, None) == femg.FG_ERR_ARG
    assert b"fg_plan_bind_terms" in L.fg_last_error()
    plan.bind_terms()
    # host outputs
    hv = np.zeros(prob.nnz, np.complex128)
    assert L.fg_assemble_fp64_static(plan.ptr, None, hv.ctypes.data, None, None) == femg.FG_ERR_ARG
    assert b"device memory" in L.fg_last_error()
    # element scratch beyond the static array: 24,576 order-3 tets, 20 DOFs,
    # real element matrices: 24,576 * 400 * 8 bytes > 64 MiB
    big = femg.Problem(femg.config_c2(m=16))
    bplan = big.plan()
    bplan.bind_terms()
    need = int(bplan.info()["E"]) * 20 * 20 * 8
    assert need > STATIC_BYTES
    bv = torch.zeros(2 * big.nnz, dtype=torch.float64, device="cuda")
    assert L.fg_assemble_fp64_static(bplan.ptr, None, bv.data_ptr(), None, None) == femg.FG_ERR_UNSUPPORTED
    assert b"exceeds" in L.fg_last_error()
