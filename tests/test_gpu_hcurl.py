"""Lowest-order HCurl (Maxwell curl-curl + mass) on the GPU: FP64 and the
tensor-core path against the oracle, the discrete de Rham identity on the
GPU's own matrix, and HCurl problems inside a batch with H1 problems."""
import numpy as np
import pytest

from test_hcurl import EDGES, csr_apply, edge_values, maxwell, only

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


CASES = {"tri_m8": (2, 8, 0), "tet_m4": (3, 4, 0), "tet_m4_percell": (3, 4, 1), "tet_m12": (3, 12, 0)}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("precision", ["fp64", "fp64_factored", "mixed"])
def test_maxwell_matches_oracle(femg, oracle, cuda, case, precision):
    dim, m, mode = CASES[case]
    prob = maxwell(femg, dim, m, coef_mode=mode)
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    if precision == "mixed":
        v, _, rep = plan.assemble("mixed", report=True)
        assert rep["global_"] <= 1e-6
    else:
        if precision == "fp64_factored":
            plan.set_fp64_method(femg.FG_FP64_FACTORED)
        v, _ = plan.assemble("fp64")
    assert rel(v, ref_v) <= (1e-6 if precision == "mixed" else 1e-12)


def test_gpu_curl_kernel(femg, cuda):
    prob = maxwell(femg, 3, 6)
    a = prob.arrays()
    t, nt = only(femg, prob, femg.FG_TERM_GRAD_GRAD)
    v, _ = prob.plan().assemble("fp64", terms=(t, nt))
    u = edge_values(a, np.random.default_rng(9).standard_normal(len(a["xyz"])))
    Ku = csr_apply(a, v, u)
    assert np.linalg.norm(Ku) <= 1e-12 * np.abs(v).max() * np.linalg.norm(u) * np.sqrt(len(u))


def test_batch_with_hcurl_and_h1(femg, oracle, cuda):
    probs = [maxwell(femg, 3, 4), femg.Problem(femg.config_c2(m=2, order=2)), maxwell(femg, 2, 6, coef_mode=1)]
    plans = [p.plan() for p in probs]
    for mixed, tol in ((False, 1e-12), (True, 1e-6)):
        batch = femg.Batch(plans, mixed=mixed)
        vals, _ = batch.run()
        for p, v in zip(probs, vals):
            t, nt = p.terms()
            ref, _ = oracle.assemble(p.arrays(), t, nt)
            assert rel(v, ref) <= tol
        batch.close()


# order 1 (HcurlLegendre1): 8 functions per triangle, 20 per tet
ORDER1 = {"tri_m6": (2, 6, 1), "tet_m3": (3, 3, 0), "tet_m8_percell": (3, 8, 1)}


@pytest.mark.parametrize("case", list(ORDER1))
@pytest.mark.parametrize("precision", ["fp64", "fp64_factored", "mixed"])
def test_maxwell_order1_matches_oracle(femg, oracle, cuda, case, precision):
    from test_hcurl_order1 import maxwell1
    dim, m, mode = ORDER1[case]
    prob = femg.Problem(maxwell1(femg, dim, m, coef_mode=mode))
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    if precision == "mixed":
        v, _, rep = plan.assemble("mixed", report=True)
        assert rep["global_"] <= 1e-6
    else:
        if precision == "fp64_factored":
            plan.set_fp64_method(femg.FG_FP64_FACTORED)
        v, _ = plan.assemble("fp64")
    assert rel(v, ref_v) <= (1e-6 if precision == "mixed" else 1e-12)


# higher orders (HcurlLegendre<p>): (p+1)(p+3) functions per triangle, (p+1)(p+3)(p+4)/2 per tet;
# the tensor-core path takes element matrices up to 24 x 24 (its B tile), FP64 up to 64 x 64
HIGH = {"tri_p2": (2, 6, 2, 1), "tri_p3": (2, 4, 3, 0), "tri_p5": (2, 3, 5, 1), "tet_p2": (3, 3, 2, 1),
        "tet_p2_m6": (3, 6, 2, 0)}


@pytest.mark.parametrize("case", list(HIGH))
@pytest.mark.parametrize("precision", ["fp64", "fp64_factored", "mixed"])
def test_maxwell_high_order_matches_oracle(femg, oracle, cuda, case, precision):
    from test_hcurl_high_order import maxwell as maxwell_p
    dim, m, p, mode = HIGH[case]
    prob = femg.Problem(maxwell_p(femg, dim, m, p, coef_mode=mode))
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    if precision == "mixed":
        if a["nb"] > 24:
            with pytest.raises(femg.FgError) as err:
                plan.assemble("mixed")
            assert err.value.status == femg.FG_ERR_UNSUPPORTED
            return
        v, _, rep = plan.assemble("mixed", report=True)
        assert rep["global_"] <= 1e-6
    else:
        if precision == "fp64_factored":
            plan.set_fp64_method(femg.FG_FP64_FACTORED)
        v, _ = plan.assemble("fp64")
        v2, _ = plan.assemble("fp64")
        assert np.array_equal(v.view(np.uint64), v2.view(np.uint64))
    assert rel(v, ref_v) <= (1e-6 if precision == "mixed" else 1e-12)
