"""Golden vectors (tests/golden/golden_small.npz, made by make_golden.py from
the reference's own Hilbert sort and robin_hood map and from the oracle):
the oracle and the host mirror against them on the CPU, the GPU paths
against them on a GPU. No access to the reference tree at test time."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")
CASES = {
    "c1_m8": ("config_c1", dict(m=8)),
    "c2_m2": ("config_c2", dict(m=2)),
    "c2_m1_p4": ("config_c2", dict(m=1, order=4)),
    "c3_m2": ("config_c3", dict(m=2)),
    "c5_m1": ("config_c5", dict(m=1)),
}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def problem(femg, name):
    cfg, kw = CASES[name]
    return femg.Problem(getattr(femg, cfg)(**kw))


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_hilbert_matches_reference_golden(oracle, golden, dim):
    pts = golden["hilbert_%dd_pts" % dim]
    mn = np.full(dim, -1e-6, np.float32)
    mx = np.full(dim, 1 + 1e-6, np.float32)
    assert np.array_equal(oracle.hilbert_order(dim, pts, mn, mx), golden["hilbert_%dd_perm" % dim])


@pytest.mark.parametrize("name", list(CASES))
def test_dictionary_order_matches_reference_golden(femg, golden, name):
    prob = problem(femg, name)
    cr = prob.created_dofs()
    rd = prob.raw_dofs()
    key = {(int(t), int(e)): i for i, (t, e) in enumerate(zip(cr["num_type"], cr["entity"]))}
    prod = np.array([key[(int(t), int(e))] for t, e in zip(rd["num_type"], rd["entity"])], np.uint32)
    assert np.array_equal(prod, golden["robin_%s" % name])


@pytest.mark.parametrize("name", list(CASES))
def test_pattern_and_oracle_values_match_golden(femg, oracle, golden, name):
    prob = problem(femg, name)
    a = prob.arrays()
    assert np.array_equal(a["ai"], golden["csr_%s_ai" % name])
    assert np.array_equal(a["aj"], golden["csr_%s_aj" % name])
    t, nt = prob.terms()
    v, b = oracle.assemble(a, t, nt)
    assert rel(v, golden["csr_%s_values" % name]) <= 1e-14
    gb = golden["csr_%s_rhs" % name]
    assert rel(b, gb) <= 1e-14 if np.linalg.norm(gb) > 0 else np.all(b == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_matches_golden(femg, cuda, golden, name):
    prob = problem(femg, name)
    plan = prob.plan()
    gv, gb = golden["csr_%s_values" % name], golden["csr_%s_rhs" % name]
    v, b = plan.assemble("fp64")
    assert rel(v, gv) <= 1e-12
    if np.linalg.norm(gb) > 0:
        assert rel(b, gb) <= 1e-12
    vm, bm = plan.assemble("mixed")
    assert rel(vm, gv) <= 1e-6
