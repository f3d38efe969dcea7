"""fg_pattern_build (GPU symbolic assembly of the CSR pattern) against the
host pre()'s pattern, which the tests of test_numbering.py and
test_golden.py pin to the oracle and the reference: equal bit for bit,
including bubble-row aliasing (order-4 triangles: three bubbles each) and
the full 384,000-tet workload."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def configs(femg):
    H = femg.FG_SPACE_HIERARCHICAL_H1
    return {
        "c1_m8": femg.config_c1(m=8),
        "c1_m16_p1mesh": femg.config(dim=2, m=16, mesh_order=1, gauss=2, dirichlet=1, source=1),
        "tri_h4_aliased_bubbles": femg.config(dim=2, m=5, mesh_order=1, space=H, order=4, gauss=8),
        "tri_h3": femg.config(dim=2, m=4, mesh_order=1, space=H, order=3, gauss=6),
        "c2_m3": femg.config_c2(m=3),
        "c2_m2_p4": femg.config_c2(m=2, order=4),
        "c2_m3_p2": femg.config_c2(m=3, order=2),
        "tet_lagrange_p2": femg.config(dim=3, m=2, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4),
        "c5_m2": femg.config_c5(m=2),
    }


@pytest.mark.parametrize("case", ["c1_m8", "c1_m16_p1mesh", "tri_h4_aliased_bubbles", "tri_h3", "c2_m3", "c2_m2_p4",
                                  "c2_m3_p2", "tet_lagrange_p2", "c5_m2"])
def test_gpu_pattern_equals_pre(femg, cuda, case):
    prob = femg.Problem(configs(femg)[case])
    a = prob.arrays()
    ai, aj = femg.pattern_build(a["edof"], a["etype"], a["n_rows"])
    assert np.array_equal(ai, a["ai"])
    assert np.array_equal(aj, a["aj"])


def test_gpu_pattern_full_size(femg, cuda):
    prob = femg.Problem(femg.config_c3())
    a = prob.arrays()
    femg.pattern_build(a["edof"][:64], a["etype"][:64], a["n_rows"])  # warm-up (module load)
    t0 = time.perf_counter()
    ai, aj = femg.pattern_build(a["edof"], a["etype"], a["n_rows"])
    dt = time.perf_counter() - t0
    assert ai[-1] == 84640201
    assert np.array_equal(ai, a["ai"])
    assert np.array_equal(aj, a["aj"])
    print("GPU pattern build of 84,640,201 nonzeros: %.3f s (host pre() total %.3f s)" % (dt, prob.pre_seconds()))
