"""Linked bubble DOFs on the GPU: plans over the systems of
tests/test_linked_bubble.py (the interior DOFs of the elements right of
x = 0.5 linked to those of the element 0.5 to their left), FP64 (1e-12) and
mixed (1e-6) against the oracle, full and symmetric storage, and the GPU
pattern against the oracle's, bit for bit."""
import numpy as np
import pytest

from test_gpu_linked import LinkedPlan
from test_linked_bubble import CFGS, linked_bubble_system

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("name", list(CFGS))
@pytest.mark.parametrize("upper", [False, True])
def test_linked_bubble_assembly_matches_oracle(femg, oracle, cuda, name, upper):
    prob, b, _ = linked_bubble_system(femg, oracle, name, 0.7, upper=upper)
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(b, t, nt)
    plan = LinkedPlan(femg, prob, b, upper=int(upper))
    v, r = plan.assemble("fp64", (t, nt))
    assert rel(v, ref_v) <= 1e-12 and rel(r, ref_b) <= 1e-12
    vm, rm = plan.assemble("mixed", (t, nt))
    assert rel(vm, ref_v) <= 1e-6 and rel(rm, ref_b) <= 1e-6
    v2, _ = plan.assemble("fp64", (t, nt))
    assert np.array_equal(v2.view(np.uint64), v.view(np.uint64))
    plan.close()


@pytest.mark.parametrize("name", list(CFGS))
@pytest.mark.parametrize("upper", [False, True])
def test_gpu_linked_bubble_pattern(femg, oracle, cuda, name, upper):
    _, b, _ = linked_bubble_system(femg, oracle, name, 0.7, upper=upper)
    ai, aj = femg.pattern_build(b["edof"], b["etype"], b["n_rows"], upper=upper, linked_row=b["linked_row"])
    assert np.array_equal(ai, b["ai"]) and np.array_equal(aj, b["aj"])
