"""The drop-in binding, fem-g_gb300/binding/GpuFormulation.h: a subclass of
the reference's Formulation<T> compiled against the reference's own headers
(oracle/_ref/ref_dropin; build recipe in oracle/build.py), on the CPU:
  * with the reference tree here: the same GmshFEM program run with
    Formulation<T> (ref_assemble) and with GpuFormulation<T> (ref_dropin, its
    C ABI calls taken by a recording stand-in that assembles them with the
    oracle) gives the same pattern, CSR values and right-hand side, to 1e-13;
    the recorded terms carry the coefficients as the binding maps them
    (constants, per-element arrays, point tables);
  * everywhere: the calls recorded in tests/golden/dropin.npz, assembled by
    the oracle, give the reference's values stored beside them (1e-13)."""
import os

import numpy as np
import pytest

from dropin_cases import Terms, cases, from_fixture, oracle_assemble, oracle_separate, separate_refs
from oracle import reference

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dropin.npz")


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


# term kinds and coefficient ops the binding records for each case
EXPECTED = {
    "c1_m8": [("GRAD_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT")],
    "c3_m2": [("GRAD_GRAD", "CONST"), ("MASS", "ELEM"), ("SOURCE", "POINT")],
    "sqrt_p2": [("GRAD_GRAD", "CONST"), ("MASS", "POINT"), ("SOURCE", "POINT")],
    "maxwell_p1": [("GRAD_GRAD", "CONST"), ("MASS", "ELEM")],
    "maxwell_p2": [("GRAD_GRAD", "CONST"), ("MASS", "CONST")],
    "full_advect": [("GRAD_GRAD_TENSOR_FULL", "CONST"), ("ADVECTION", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT")],
    "vector_terms": [("VECTOR_GRAD_TEST", "CONST"), ("SOURCE_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT")],
    "c1_upper": [("GRAD_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT")],
    "sym_tensor": [("GRAD_GRAD_TENSOR", "CONST"), ("MASS", "CONST")],
    "maxwell_tensor": [("GRAD_GRAD_TENSOR", "CONST"), ("MASS_TENSOR", "CONST"), ("GRAD_GRAD", "CONST"), ("MASS", "CONST")],
    "navier_p2": [("ELASTIC", "ELEM"), ("MASS", "CONST")],
    "navier_p2_omega": [("ELASTIC", "ELEM"), ("MASS", "CONST")],
    "dt_terms": [("GRAD_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT"), ("MASS", "POINT"), ("MASS", "CONST")],
    "separate_mck": [("GRAD_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT"), ("MASS", "POINT"), ("MASS", "CONST")],
    # one call per (test field, unknown field) block: u-u, u-v, v-u, v-v
    "coupled_p2": [[("GRAD_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", None)], [("GRAD_GRAD", "CONST")],
                   [("MASS", "POINT"), ("ADVECTION", "CONST")], [("GRAD_GRAD", "CONST"), ("MASS", "CONST"), ("SOURCE", "POINT")]],
}


def expected_calls(name):
    e = EXPECTED[name]
    return e if isinstance(e[0], list) else [e]


@pytest.mark.skipif(not reference.dropin_available(), reason="drop-in program not built (no reference tree)")
@pytest.mark.parametrize("name", list(EXPECTED))
def test_dropin_matches_reference_assemble(femg, name):
    cfg, progs = cases(femg)[name]
    ref = reference.run(cfg, threads=2, programs=progs)
    drop = reference.run(cfg, threads=2, programs=progs, dropin=True)
    assert np.array_equal(ref["ai"], drop["ai"]) and np.array_equal(ref["aj"], drop["aj"])
    for k in ("num_type", "entity", "num_dof", "assemble_type"):
        assert np.array_equal(ref["dof_" + k], drop["dof_" + k]), k
    assert rel(drop["values"], ref["values"]) <= 1e-13, rel(drop["values"], ref["values"])
    assert rel(drop["rhs"], ref["rhs"]) <= 1e-13, rel(drop["rhs"], ref["rhs"])
    assert ("C" in drop) == ("C" in ref) == (name == "separate_mck")
    if "C" in ref:  # separate matrices: values are K, and C, M apart
        assert rel(drop["C"], ref["C"]) <= 1e-13 and rel(drop["M"], ref["M"]) <= 1e-13
        assert np.abs(ref["C"]).max() > 0 and np.abs(ref["M"]).max() > 0
    calls = drop["record"]
    want = expected_calls(name)
    assert len(calls) == len(want)
    for call, w in zip(calls, want):
        got = [(kind, code[0][0] if op is not None else None) for (kind, _, code, _, _, _), (_, op) in zip(call["terms"], w)]
        assert got == [(getattr(femg, "FG_TERM_" + k), getattr(femg, "FG_OP_" + op) if op else None) for k, op in w]
        assert call["upper"] == (1 if name == "c1_upper" else 0)
    assert sum(c.get("unknown") is not None for c in calls) == (2 if name == "coupled_p2" else 0)
    if name in ("dt_terms", "separate_mck"):  # damping dt, inertia dt2
        assert [t[1] for t in calls[0]["terms"]] == [0, 0, 0, femg.FG_DT_1, femg.FG_DT_2]
        assert calls[0]["entry"] == (1 if name == "separate_mck" else 0)
        if name == "dt_terms":  # at the formulation's frequency
            assert calls[0]["frequency"] == cfg.omega


@pytest.mark.skipif(not reference.dropin_available(), reason="drop-in program not built (no reference tree)")
def test_dropin_refuses_what_it_does_not_map(femg):
    """A coefficient on the test function's side (integral(dof(u), m tf(u)))
    is not mapped by the binding: assemble() sends the error to msg::error
    (silent at the program's verbosity 0) and leaves A and b zero, as the
    reference does when its assembly throws; no C ABI call is made."""
    cfg = femg.config(dim=2, m=3, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=3)
    progs = {"grad": [(femg.FG_OP_CONST, 0, 1.0, 0.0)], "mass_tf": [(femg.FG_OP_CONST, 0, 2.0, 0.5)]}
    ref = reference.run(cfg, threads=2, programs=progs)
    assert np.abs(ref["values"]).max() > 0
    drop = reference.run(cfg, threads=2, programs=progs, dropin=True)
    assert np.all(drop["values"] == 0) and np.all(drop["rhs"] == 0)
    assert drop["record"] == []


@pytest.mark.parametrize("name", list(EXPECTED))
def test_recorded_calls_assemble_to_reference(femg, oracle, name):
    z = np.load(FIXTURE)
    calls, ref_v, ref_b = from_fixture(z, name + "/")
    sep = separate_refs(z, name + "/")
    if sep is not None:
        assert len(calls) == 1 and calls[0]["entry"] == 1
        k, c, m, b = oracle_separate(femg, oracle, calls[0])
        assert rel(k, ref_v) <= 1e-13 and rel(c, sep[0]) <= 1e-13 and rel(m, sep[1]) <= 1e-13 and rel(b, ref_b) <= 1e-13
        return
    v, b = 0.0, 0.0
    for call in calls:
        vk, bk = oracle_assemble(oracle, call, Terms(femg, call))
        v, b = v + vk, b + bk
    assert rel(v, ref_v) <= 1e-13 and rel(b, ref_b) <= 1e-13
