"""Non-symmetric element matrices on the GPU FP64 path (the full-matrix
element kernel) against the oracle, which test_nonsym.py pins to the
reference's own assembly: a general TensorFunction and the advection term,
with Dirichlet lifting through the transposed element entry, to 1e-12; the
factored method falls back to the quadrature loop for them, and the tensor-
core paths decline them."""
import numpy as np
import pytest

from coef_programs import nonsym_configs, nonsym_terms

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("what", ["full", "advect", "both", "vdof", "vsrc", "vector"])
@pytest.mark.parametrize("geom", ["tri_p2_dirichlet1", "tri_h1_p3", "tet_h1_p2"])
def test_gpu_nonsymmetric_matches_oracle(femg, oracle, cuda, geom, what):
    prob = femg.Problem(nonsym_configs(femg)[geom])
    a = prob.arrays()
    t, nt, _, keep = nonsym_terms(femg, what)
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64", terms=(t, nt))
    assert rel(v, ref_v) <= 1e-12, rel(v, ref_v)
    assert rel(b, ref_b) <= 1e-12, rel(b, ref_b)
    plan.set_fp64_method(femg.FG_FP64_FACTORED)  # not exact for these terms: the quadrature loop runs
    v2, b2 = plan.assemble("fp64", terms=(t, nt))
    assert rel(v2, ref_v) <= 1e-12 and rel(b2, ref_b) <= 1e-12


def test_gpu_nonsymmetric_declined_by_tensor_core_paths(femg, cuda):
    prob = femg.Problem(nonsym_configs(femg)["tet_h1_p2"])
    t, nt, _, keep = nonsym_terms(femg, "both")
    plan = prob.plan()
    with pytest.raises(femg.FgError) as err:
        plan.assemble("mixed", terms=(t, nt))
    assert err.value.status == femg.FG_ERR_UNSUPPORTED
