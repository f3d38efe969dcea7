"""The drop-in binding's C ABI calls on the GPU: the calls that
fem-g_gb300/binding/GpuFormulation.h (compiled against the reference's
headers) made for the cases of tests/dropin_cases.py, recorded in
tests/golden/dropin.npz, replayed through libfemg.so (fg_plan_create,
fg_assemble_fp64, fg_assemble_mixed) and set against the reference's own
Formulation::assemble on the same problems: FP64 to 1e-12, mixed to 1e-6
(point-dependent bilinear coefficients and the non-symmetric terms take the
FP64 path only, and the mixed call refuses them)."""
import os

import numpy as np
import pytest

from dropin_cases import ReplayPlan, Terms, from_fixture, separate_refs
from test_dropin import EXPECTED, FIXTURE, expected_calls

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("name", list(EXPECTED))
def test_dropin_calls_match_reference(femg, cuda, name):
    assert os.path.exists(FIXTURE)
    z = np.load(FIXTURE)
    calls, ref_v, ref_b = from_fixture(z, name + "/")
    sep = separate_refs(z, name + "/")
    if sep is not None:  # fg_assemble_separate: K, C, M apart
        t = Terms(femg, calls[0])
        plan = ReplayPlan(femg, calls[0])
        k, c, m, b = plan.assemble_separate(t)
        assert rel(k, ref_v) <= 1e-12 and rel(c, sep[0]) <= 1e-12 and rel(m, sep[1]) <= 1e-12 and rel(b, ref_b) <= 1e-12
        plan.close()
        return
    fp64_only = {"GRAD_GRAD_TENSOR_FULL", "ADVECTION", "VECTOR_GRAD_TEST", "SOURCE_GRAD"}
    v, b, vm, bm, mixed = 0.0, 0.0, 0.0, 0.0, True
    for call, want in zip(calls, expected_calls(name)):
        t = Terms(femg, call)
        plan = ReplayPlan(femg, call)
        vk, bk = plan.assemble("fp64", t)
        v2, _ = plan.assemble("fp64", t)
        assert np.array_equal(vk.view(np.uint64), v2.view(np.uint64))
        v, b = v + vk, b + bk
        # two-field plans take the FP64 path only; so do point-dependent
        # bilinear coefficients, the non-symmetric terms and large HCurl elements
        # the tensor-core path takes element matrices up to 24 x 24 for HCurl fields
        big_hcurl = call["form"] == femg.FG_FORM_1 and call["nb"] > 24
        if call["unknown"] is not None or big_hcurl or ("MASS", "POINT") in want or any(k in fp64_only for k, _ in want):
            with pytest.raises(femg.FgError) as err:
                plan.assemble("mixed", t)
            assert err.value.status == femg.FG_ERR_UNSUPPORTED
            mixed = False
        else:
            vmk, bmk = plan.assemble("mixed", t)
            vm, bm = vm + vmk, bm + bmk
        plan.close()
    assert rel(v, ref_v) <= 1e-12 and rel(b, ref_b) <= 1e-12
    if mixed:
        assert rel(vm, ref_v) <= 1e-6 and rel(bm, ref_b) <= 1e-6
