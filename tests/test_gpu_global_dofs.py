"""UnknownGlobal element DOFs on the GPU (the merged systems of
test_global_dofs.py: every boundary DOF lumped into one row): the plan's
rows and columns take them as Unknown DOFs, several local DOFs of an element
landing on one row and one slot. FP64 (1e-12) and mixed (1e-6) against the
oracle, and the GPU pattern against the oracle's, bit for bit."""
import numpy as np
import pytest

from test_global_dofs import CFGS, merged_system, pair_merged_system
from test_gpu_linked import LinkedPlan

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("name", list(CFGS))
def test_global_rows_match_oracle(femg, oracle, cuda, name):
    prob, _, b, _ = merged_system(femg, oracle, name)
    b = dict(b, linked_row=np.zeros(0, np.uint64), linked_value=np.zeros(0, np.complex128))
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(b, t, nt)
    plan = LinkedPlan(femg, prob, b)
    v, r = plan.assemble("fp64", (t, nt))
    assert rel(v, ref_v) <= 1e-12 and rel(r, ref_b) <= 1e-12
    vm, rm = plan.assemble("mixed", (t, nt))
    assert rel(vm, ref_v) <= 1e-6 and rel(rm, ref_b) <= 1e-6
    plan.close()


def test_global_pairs_on_the_vector_reduction(femg, oracle, cuda):
    """Order-3 tetrahedra with DOF pairs of one element on one row: two lanes
    of an element row add into one slot of the mixed path's vector-load
    reduction in the same step, which the plan then keeps on atomic adds."""
    prob, _, b, _ = pair_merged_system(femg, oracle)
    b = dict(b, linked_row=np.zeros(0, np.uint64), linked_value=np.zeros(0, np.complex128))
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(b, t, nt)
    plan = LinkedPlan(femg, prob, b)
    v, r = plan.assemble("fp64", (t, nt))
    assert rel(v, ref_v) <= 1e-12 and rel(r, ref_b) <= 1e-12
    femg.profile_enable(True)
    femg.profile_read()
    try:
        vm, rm = plan.assemble("mixed", (t, nt))
        kernels = femg.profile_read()
    finally:
        femg.profile_enable(False)
    assert "k_gather_v4" in kernels
    assert rel(vm, ref_v) <= 1e-6 and rel(rm, ref_b) <= 1e-6
    plan.close()


@pytest.mark.parametrize("name", list(CFGS))
def test_gpu_pattern_with_global_rows(femg, oracle, cuda, name):
    _, _, b, _ = merged_system(femg, oracle, name)
    ai, aj = femg.pattern_build(b["edof"], b["etype"], b["n_rows"])
    assert np.array_equal(ai, b["ai"]) and np.array_equal(aj, b["aj"])
