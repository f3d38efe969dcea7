"""Symmetric (upper-triangle) storage on the GPU: the plan skips the entries
below the diagonal, FP64 (1e-12) and mixed (1e-6) against the oracle, with
Dirichlet lifting and sources, complex element matrices, and the GPU pattern
build against the host's upper pattern, bit for bit."""
import ctypes as C

import numpy as np
import pytest

from test_upper import CFGS

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("name", list(CFGS))
def test_upper_assembly_matches_oracle(femg, oracle, cuda, name):
    prob = femg.Problem(femg.config(upper=1, **CFGS[name]))
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64")
    assert rel(v, ref_v) <= 1e-12
    vm, bm = plan.assemble("mixed")
    assert rel(vm, ref_v) <= 1e-6
    if np.linalg.norm(ref_b) > 0:
        assert rel(b, ref_b) <= 1e-12 and rel(bm, ref_b) <= 1e-6


def test_upper_complex_elements(femg, oracle, cuda):
    """Damping dt_dof(u) at omega = 2: complex element matrices (hermitian storage)."""
    prob = femg.Problem(femg.config(upper=1, **CFGS["tet_h1_p3"]))
    t, nt = prob.terms()
    arr = (femg.TermDesc * 3)()
    for k, (src, dt) in enumerate([(0, 0), (1, 0), (1, 1)]):
        C.memmove(C.byref(arr[k]), C.byref(t[src]), C.sizeof(femg.TermDesc))
        arr[k].dt = dt
    a = prob.arrays()
    ref_v, _ = oracle.assemble(a, arr, 3, freq=2.0)
    plan = prob.plan()
    for precision, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        v, _ = plan.assemble(precision, frequency=2.0, terms=(arr, 3))
        assert rel(v, ref_v) <= tol


@pytest.mark.parametrize("name", list(CFGS))
def test_gpu_upper_pattern(femg, cuda, name):
    prob = femg.Problem(femg.config(upper=1, **CFGS[name]))
    a = prob.arrays()
    ai, aj = femg.pattern_build(a["edof"], a["etype"], a["n_rows"], upper=True)
    assert np.array_equal(ai, a["ai"]) and np.array_equal(aj, a["aj"])
