"""fg_assemble_fp64_static (element scratch in a fixed device array, no
allocation in the call) against fg_assemble_fp64 on the same plan, two calls
in a row; its argument and size checks. Collected last so that it also runs
after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
STATIC_BYTES = 64 << 20


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _static_call(femg, torch, plan, prob, with_rhs=True):
    nnz, nrows = prob.nnz, int(prob.sys.n_rows)
    dv = torch.full((2 * nnz,), float("nan"), dtype=torch.float64, device="cuda")
    db = torch.full((2 * nrows,), float("nan"), dtype=torch.float64, device="cuda") if with_rhs else None
    dd = None
    if prob.sys.n_fixed:
        a = prob.arrays()
        dd = torch.from_numpy(np.ascontiguousarray(a["dirichlet"]).view(np.float64).copy()).cuda()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = femg.lib().fg_assemble_fp64_static(plan.ptr, dd.data_ptr() if dd is not None else None, dv.data_ptr(),
                                            db.data_ptr() if db is not None else None, stream)
    torch.cuda.synchronize()
    assert st == femg.FG_OK, femg.lib().fg_last_error()
    v = dv.cpu().numpy().view(np.complex128)
    b = db.cpu().numpy().view(np.complex128) if db is not None else None
    return v, b


@pytest.mark.parametrize("case", ["c3_m4", "c1_m8", "c5_m2"])
def test_static_matches_fp64_twice(femg, cuda, case):
    torch = cuda
    cfg = {"c3_m4": femg.config_c3(m=4), "c1_m8": femg.config_c1(m=8), "c5_m2": femg.config_c5(m=2)}[case]
    prob = femg.Problem(cfg)
    plan = prob.plan()
    v_ref, b_ref = plan.assemble("fp64")
    plan.bind_terms()
    for _ in range(2):
        v, b = _static_call(femg, torch, plan, prob)
        assert rel(v, v_ref) <= FP64_TOL
        if np.linalg.norm(b_ref) > 0:
            assert rel(b, b_ref) <= FP64_TOL
        else:
            assert np.all(b == 0)


def test_static_without_rhs(femg, cuda):
    torch = cuda
    prob = femg.Problem(femg.config_c3(m=3))
    plan = prob.plan()
    v_ref, _ = plan.assemble("fp64")
    plan.bind_terms()
    v, _ = _static_call(femg, torch, plan, prob, with_rhs=False)
    assert rel(v, v_ref) <= FP64_TOL


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
