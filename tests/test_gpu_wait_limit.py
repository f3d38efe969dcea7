"""The tensor-core contraction's bounded wait, run out on purpose without a
fault: fg_set_wait_limit(0) makes the wait for each MMA chain give up at
once. The kernel then records the timeout, waits again (with the fixed
bound) for the MMAs it issued, frees its TMEM and returns. The call reports
FG_ERR_TIMEOUT, and the next call, with the default bound, assembles
correctly on the same plan and device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def test_contraction_wait_runs_out_and_recovers(femg, oracle, cuda):
    L = femg.lib()
    prob = femg.Problem(femg.config_c3(m=4))
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(prob.arrays(), t, nt)
    plan = prob.plan()
    assert L.fg_set_wait_limit(-1.0) == femg.FG_ERR_ARG
    try:
        assert L.fg_set_wait_limit(0.0) == femg.FG_OK
        with pytest.raises(femg.FgError) as e:
            plan.assemble("mixed")  # host outputs: the call reports its own timeout
        assert e.value.status == femg.FG_ERR_TIMEOUT
    finally:
        assert L.fg_set_wait_limit(2.0) == femg.FG_OK
    cuda.cuda.synchronize()
    v, b = plan.assemble("mixed")
    assert rel(v, ref_v) <= 1e-6 and rel(b, ref_b) <= 1e-6
    # device outputs: a timeout is reported by the next call on the plan
    dv = cuda.zeros(2 * prob.nnz, dtype=cuda.float64, device="cuda")
    try:
        assert L.fg_set_wait_limit(0.0) == femg.FG_OK
        plan.assemble("mixed", values=dv.data_ptr(), rhs=False)
        cuda.cuda.synchronize()
    finally:
        assert L.fg_set_wait_limit(2.0) == femg.FG_OK
    with pytest.raises(femg.FgError) as e:
        plan.assemble("mixed", values=dv.data_ptr(), rhs=False)
    assert e.value.status == femg.FG_ERR_TIMEOUT
    plan.assemble("mixed", values=dv.data_ptr(), rhs=False)
    cuda.cuda.synchronize()
    assert rel(dv.cpu().numpy().view(np.complex128), ref_v) <= 1e-6
    plan.close()
