"""The fused mixed path (tensor-core contraction and CSR reduction in one
kernel, no element matrix in device memory) against the oracle at the mixed
tolerance, against the split mixed path, and run to run: bit-identical. Also
where it declines (order-4 face functions, complex coefficients, Dirichlet
columns): the split path runs and the result is unchanged."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def cases(femg):
    return {
        "c3_m6": femg.config_c3(m=6),
        "c2_p1_m8": femg.config_c2(m=8, order=1),
        "c2_p2_m6": femg.config_c2(m=6, order=2),
        "c3_m10_tall": femg.config_c3(m=10),
        "tri_h1_p3_source": femg.config(dim=2, m=12, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=3, gauss=6,
                                        k=5.0, source=1, coef_mode=1),
        "tri_p2_lagrange": femg.config(dim=2, m=10, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4, k=7.0),
        "upper_c3_m4": femg.config_c3(m=4),
    }


@pytest.mark.parametrize("name", ["c3_m6", "c2_p1_m8", "c2_p2_m6", "c3_m10_tall", "tri_h1_p3_source", "tri_p2_lagrange",
                                  "upper_c3_m4"])
def test_fused_matches_oracle_split_and_itself(femg, oracle, cuda, name):
    cfg = cases(femg)[name]
    if name.startswith("upper"):
        cfg.upper = 1
    prob = femg.Problem(cfg)
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    info = plan.fused_info()
    assert info["applies"], info["why"]
    assert info["contractions_per_element"] >= 1.0
    plan.set_mixed_fused(True)
    v1, b1 = plan.assemble("mixed")
    v2, b2 = plan.assemble("mixed")
    assert np.array_equal(v1, v2) and np.array_equal(b1, b2)  # deterministic
    assert rel(v1, ref_v) <= MIXED_TOL
    if np.linalg.norm(ref_b) > 0:
        assert rel(b1, ref_b) <= 1e-12  # the right-hand side stays FP64
    plan.set_mixed_fused(False)
    vs, bs = plan.assemble("mixed")
    assert rel(v1, vs) <= MIXED_TOL
    assert np.array_equal(b1, bs)


def test_fused_device_outputs_and_accumulate(femg, oracle, cuda):
    torch = cuda
    prob = femg.Problem(femg.config_c3(m=5))
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    assert plan.fused_info()["applies"]
    plan.set_mixed_fused(True)
    dv = torch.zeros(2 * prob.nnz, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    plan.assemble("mixed", values=dv.data_ptr(), rhs=False, stream=stream)
    torch.cuda.synchronize()
    v = dv.cpu().numpy().view(np.complex128).copy()
    assert rel(v, ref_v) <= MIXED_TOL
    # accumulating plan: a second call adds the same system again
    plan.set_accumulate(True)
    plan.assemble("mixed", values=dv.data_ptr(), rhs=False, stream=stream)
    torch.cuda.synchronize()
    v2 = dv.cpu().numpy().view(np.complex128)
    assert rel(v2, 2 * ref_v) <= MIXED_TOL


@pytest.mark.parametrize("what", ["order4", "dirichlet"])
def test_fused_declines_and_split_path_runs(femg, oracle, cuda, what):
    cfg = femg.config_c2(m=3, order=4) if what == "order4" else femg.config_c1(m=8)
    if what == "order4":
        cfg.gauss = 8
    prob = femg.Problem(cfg)
    plan = prob.plan()
    info = plan.fused_info()
    assert not info["applies"]
    assert info["why"]
    plan.set_mixed_fused(True)
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    v, _ = plan.assemble("mixed")
    assert rel(v, ref_v) <= MIXED_TOL


def test_fused_full_size_c3(femg, oracle, cuda):
    """384,000 order-3 tets with per-tet coefficients: fused against the oracle
    entry by entry, and against the split path."""
    prob = femg.Problem(femg.config_c3())
    plan = prob.plan()
    info = plan.fused_info()
    assert info["applies"], info["why"]
    plan.set_mixed_fused(True)
    v, _ = plan.assemble("mixed")
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    assert rel(v, ref_v) <= MIXED_TOL
    plan.set_mixed_fused(False)
    vs, _ = plan.assemble("mixed")
    assert rel(v, vs) <= MIXED_TOL
