"""Linked DOFs on the GPU: plans over the periodic / Bloch systems of
tests/test_linked.py (DOFs on one line linked to another with e^(i phi)),
FP64 (1e-12) and mixed (1e-6) against the oracle's linked assembly, the GPU
pattern against the oracle's linked pattern, and the paths that decline
linked DOFs (batches, several frequencies)."""
import ctypes as C

import numpy as np
import pytest

from test_linked import CFGS, linked_pattern

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


class LinkedPlan:
    def __init__(self, femg, prob, b, upper=0):
        self.keep = []

        def arr(x, dt):
            x = np.ascontiguousarray(x, dt)
            self.keep.append(x)
            return x

        ai, aj = arr(b["ai"], np.uint64), arr(b["aj"], np.uint64)
        ed, et = arr(b["edof"], np.uint64), arr(b["etype"], np.int32)
        lr, lv = arr(b["linked_row"], np.uint64), arr(b["linked_value"], np.complex128)
        U64, I32, F64 = C.POINTER(C.c_uint64), C.POINTER(C.c_int32), C.POINTER(C.c_double)
        self.sys = femg.SystemDesc(int(b["n_rows"]), ai.ctypes.data_as(U64), aj.ctypes.data_as(U64), ed.ctypes.data_as(U64),
                                   et.ctypes.data_as(I32), prob.sys.n_fixed, upper, len(lr), lr.ctypes.data_as(U64),
                                   lv.ctypes.data_as(F64))
        self.ptr = C.c_void_p()
        self.L = femg.lib()
        self.femg = femg
        self.prob = prob
        self.nnz, self.n_rows = len(aj), int(b["n_rows"])
        femg.check(self.L.fg_plan_create(C.byref(prob.mesh), C.byref(prob.rule), C.byref(prob.space), C.byref(self.sys),
                                         C.byref(self.ptr)))

    def assemble(self, precision, terms, frequency=0.0):
        v = np.zeros(self.nnz, np.complex128)
        r = np.zeros(self.n_rows, np.complex128)
        t, nt = terms
        d = C.cast(self.prob.dir_ptr, C.c_void_p) if self.prob.sys.n_fixed else None
        if precision == "fp64":
            self.femg.check(self.L.fg_assemble_fp64(self.ptr, t, nt, frequency, d, v.ctypes.data, r.ctypes.data, None))
        else:
            self.femg.check(self.L.fg_assemble_mixed(self.ptr, t, nt, frequency, d, v.ctypes.data, r.ctypes.data, None, None))
        return v, r

    def close(self):
        self.L.fg_plan_destroy(self.ptr)


@pytest.mark.parametrize("name", list(CFGS))
@pytest.mark.parametrize("phi", [0.0, 0.7])
def test_linked_assembly_matches_oracle(femg, oracle, cuda, name, phi):
    prob, b, _ = linked_pattern(femg, oracle, name, phi)
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(b, t, nt)
    plan = LinkedPlan(femg, prob, b)
    v, r = plan.assemble("fp64", (t, nt))
    assert rel(v, ref_v) <= 1e-12 and rel(r, ref_b) <= 1e-12
    vm, rm = plan.assemble("mixed", (t, nt))
    assert rel(vm, ref_v) <= 1e-6 and rel(rm, ref_b) <= 1e-6
    # FP64 runs are bit-identical
    v2, _ = plan.assemble("fp64", (t, nt))
    assert np.array_equal(v2.view(np.uint64), v.view(np.uint64))
    plan.close()


@pytest.mark.parametrize("name", list(CFGS))
def test_gpu_linked_pattern(femg, oracle, cuda, name):
    _, b, _ = linked_pattern(femg, oracle, name, 0.7)
    ai, aj = femg.pattern_build(b["edof"], b["etype"], b["n_rows"], linked_row=b["linked_row"])
    assert np.array_equal(ai, b["ai"]) and np.array_equal(aj, b["aj"])


def test_linked_plans_are_declined_where_unsupported(femg, oracle, cuda):
    prob, b, _ = linked_pattern(femg, oracle, "tri_p1", 0.7)
    plan = LinkedPlan(femg, prob, b)
    L = femg.lib()
    t, nt = prob.terms()
    om = np.array([1.0, 2.0])
    v = np.zeros(2 * plan.nnz, np.complex128)
    assert L.fg_assemble_multi_freq(plan.ptr, t, nt, om.ctypes.data, 2, 0, None, v.ctypes.data, None, None) == \
        femg.FG_ERR_UNSUPPORTED
    plans = (C.c_void_p * 1)(plan.ptr)
    out = C.c_void_p()
    assert L.fg_batch_create(plans, None, None, 1, 0, C.byref(out)) == femg.FG_ERR_UNSUPPORTED
    plan.close()


def test_linked_with_upper_storage(femg, oracle, cuda):
    prob, b, _ = linked_pattern(femg, oracle, "tri_p2_dirichlet", 0.7)
    bu = dict(b, upper=1)
    ai, aj = oracle.pattern(bu["edof"], bu["etype"], bu["n_rows"], upper=True, linked_row=bu["linked_row"])
    bu.update(ai=ai, aj=aj)
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(bu, t, nt)
    plan = LinkedPlan(femg, prob, bu, upper=1)
    v, r = plan.assemble("fp64", (t, nt))
    assert rel(v, ref_v) <= 1e-12 and rel(r, ref_b) <= 1e-12
    gai, gaj = femg.pattern_build(bu["edof"], bu["etype"], bu["n_rows"], upper=True, linked_row=bu["linked_row"])
    assert np.array_equal(gai, ai) and np.array_equal(gaj, aj)
    plan.close()
