"""Point tables (FG_OP_POINT) on the GPU: FP64 with the tables of
tests/test_point_table.py against the oracle's assembly of the program form
(1e-12); the mixed path takes a point-table source (the right-hand side is
FP64) and refuses a point-table bilinear coefficient."""
import ctypes as C

import numpy as np
import pytest

from coef_programs import configs
from test_point_table import tables_terms

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("geom", ["tri_p2", "tet_h1_p2"])
@pytest.mark.parametrize("split", [False, True])
def test_point_table_fp64(femg, oracle, cuda, geom, split):
    prob = femg.Problem(configs(femg)[geom])
    a = prob.arrays()
    prog, tab, keep = tables_terms(femg, a, split)
    ref_v, ref_b = oracle.assemble(a, prog, 2)
    plan = prob.plan()
    v, b = plan.assemble("fp64", terms=(tab, 2))
    assert rel(v, ref_v) <= 1e-12 and rel(b, ref_b) <= 1e-12


def test_point_table_mixed(femg, oracle, cuda):
    prob = femg.Problem(configs(femg)["tri_p2"])
    a = prob.arrays()
    prog, tab, keep = tables_terms(femg, a, False)
    plan = prob.plan()
    with pytest.raises(femg.FgError) as err:
        plan.assemble("mixed", terms=(tab, 2))
    assert err.value.status == femg.FG_ERR_UNSUPPORTED
    # the source alone as a table, with a constant grad-grad term
    both = (femg.TermDesc * 2)()
    for t in both:
        C.memset(C.byref(t), 0, C.sizeof(femg.TermDesc))
    both[0].kind = femg.FG_TERM_GRAD_GRAD
    both[0].coef.n_code = 1
    both[0].coef.code[0].op, both[0].coef.code[0].re = femg.FG_OP_CONST, 1.0
    C.memmove(C.byref(both[1]), C.byref(tab[1]), C.sizeof(femg.TermDesc))
    ref = (femg.TermDesc * 2)()
    C.memmove(C.byref(ref[0]), C.byref(both[0]), C.sizeof(femg.TermDesc))
    C.memmove(C.byref(ref[1]), C.byref(prog[1]), C.sizeof(femg.TermDesc))
    ref_v, ref_b = oracle.assemble(a, ref, 2)
    v, b = plan.assemble("mixed", terms=(both, 2))
    assert rel(v, ref_v) <= 1e-6 and rel(b, ref_b) <= 1e-12
