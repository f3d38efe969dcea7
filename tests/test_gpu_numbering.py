"""GPU DOF numbering (fg_hilbert_numbering / fg_hilbert_order) against the
host pre()'s numbering, which test_numbering.py and test_golden.py pin to the
reference's Hilbert sort; the GPU order also against the golden vectors of
the reference itself. Bit-exact, including ties (stable order) and bubbles."""
import os
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")


def configs(femg):
    H = femg.FG_SPACE_HIERARCHICAL_H1
    return {
        "c1_m8": femg.config_c1(m=8),
        "tri_h4_bubbles": femg.config(dim=2, m=5, mesh_order=1, space=H, order=4, gauss=8),
        "c2_m3": femg.config_c2(m=3),
        "c2_m2_p4": femg.config_c2(m=2, order=4),
        "tet_lagrange_p2": femg.config(dim=3, m=2, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4),
        "c5_m2": femg.config_c5(m=2),
    }


@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_hilbert_order_matches_reference_golden(femg, dim):
    g = np.load(GOLDEN)
    pts = g["hilbert_%dd_pts" % dim]
    mn = np.full(dim, -1e-6, np.float32)
    mx = np.full(dim, 1 + 1e-6, np.float32)
    assert np.array_equal(femg.hilbert_order(dim, pts, mn, mx), g["hilbert_%dd_perm" % dim])


@pytest.mark.parametrize("case", ["c1_m8", "tri_h4_bubbles", "c2_m3", "c2_m2_p4", "tet_lagrange_p2", "c5_m2"])
def test_gpu_numbering_equals_pre(femg, cuda, case):
    prob = femg.Problem(configs(femg)[case])
    rd = prob.raw_dofs()
    dim = int(prob.arrays()["dim"])
    start = rd["num_dof"].copy()
    unknown = (rd["assemble_type"] == 2) | (rd["assemble_type"] == 3)
    start[unknown] = 0
    got = femg.hilbert_numbering(dim, prob.bbox(), rd["xyz"], rd["assemble_type"], start)
    assert np.array_equal(got, rd["num_dof"])


def test_gpu_numbering_full_size(femg, cuda):
    prob = femg.Problem(femg.config_c3())
    rd = prob.raw_dofs()
    start = rd["num_dof"].copy()
    start[(rd["assemble_type"] == 2) | (rd["assemble_type"] == 3)] = 0
    femg.hilbert_numbering(3, prob.bbox(), rd["xyz"][:10], rd["assemble_type"][:10], start[:10])  # module load
    t0 = time.perf_counter()
    got = femg.hilbert_numbering(3, prob.bbox(), rd["xyz"], rd["assemble_type"], start)
    dt = time.perf_counter() - t0
    assert np.array_equal(got, rd["num_dof"])
    print("GPU numbering of %d DOFs: %.3f s" % (len(got), dt))
