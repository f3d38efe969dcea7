"""Tensor coefficients on HCurl fields (Maxwell PML form) on the GPU
against the oracle: FP64 (1e-12 relative Frobenius) and the tensor-core path
(1e-6), real and complex tensors, constant and per-element coefficients, 2D
and 3D; the factored FP64 method's fallback and the argument check."""
import numpy as np
import pytest

from test_hcurl import maxwell
from test_hcurl_tensor import hcurl_tensor_terms, spd
from test_tensor_coef import tensor_terms

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("dim,m", [(2, 6), (3, 3)])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("coef_mode", [0, 1])
@pytest.mark.parametrize("which", ["both", "curl", "mass"])
def test_matches_oracle(femg, oracle, cuda, dim, m, cplx, coef_mode, which):
    prob = maxwell(femg, dim, m, coef_mode=coef_mode)
    a = prob.arrays()
    Dc = spd(3, cplx, dim) if which in ("both", "curl") else None
    Dm = spd(4, cplx, dim) if which in ("both", "mass") else None
    t, nt = hcurl_tensor_terms(femg, prob, Dc, Dm)
    ref_v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    plan = prob.plan()
    v, _ = plan.assemble("fp64", terms=(t, nt), rhs=False)
    assert rel(v, ref_v) <= FP64_TOL
    plan.set_fp64_method(femg.FG_FP64_FACTORED)  # falls back to the quadrature loop
    v2, _ = plan.assemble("fp64", terms=(t, nt), rhs=False)
    assert np.array_equal(v2.view(np.uint64), v.view(np.uint64))
    vm, _, rep = plan.assemble("mixed", terms=(t, nt), rhs=False, report=True)
    assert rel(vm, ref_v) <= MIXED_TOL and rep["global_"] <= MIXED_TOL


def test_mass_tensor_needs_hcurl(femg, cuda):
    from test_tensor_coef import problems
    prob = problems(femg)["tet_p1"]
    t, nt = tensor_terms(femg, prob, np.eye(3))
    t[0].kind = femg.FG_TERM_MASS_TENSOR
    with pytest.raises(femg.FgError) as err:
        prob.plan().assemble("fp64", terms=(t, nt), rhs=False)
    assert err.value.status == femg.FG_ERR_UNSUPPORTED
