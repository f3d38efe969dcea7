"""Golden vectors (tests/golden/golden_small.npz, made by make_golden.py from
the reference's own code: its Hilbert sort and robin_hood map, and its
Formulation::pre() and assemble() run through the gmsh stand-in): the
oracle and the host mirror against them on the CPU, the GPU paths against
them on a GPU. No access to the reference tree at test time."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import CASES, build_config  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def problem(femg, name):
    return femg.Problem(build_config(femg, name))


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
def test_pattern_numbering_and_oracle_values_match_reference_golden(femg, oracle, golden, name):
    """pattern and DOF dictionary bit for bit, the oracle's values to 1e-13
    (the reference sums with OpenMP atomics, in no fixed order)"""
    prob = problem(femg, name)
    a = prob.arrays()
    assert np.array_equal(a["ai"], golden["csr_%s_ai" % name])
    assert np.array_equal(a["aj"], golden["csr_%s_aj" % name])
    rd = prob.raw_dofs()
    for k in ("num_type", "entity", "num_dof", "assemble_type"):
        assert np.array_equal(rd[k], golden["dof_%s_%s" % (name, k)]), k
    t, nt = prob.terms()
    v, b = oracle.assemble(a, t, nt)
    assert rel(v, golden["csr_%s_values" % name]) <= 1e-13
    gb = golden["csr_%s_rhs" % name]
    assert rel(b, gb) <= 1e-13 if np.linalg.norm(gb) > 0 else np.all(b == 0)


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
