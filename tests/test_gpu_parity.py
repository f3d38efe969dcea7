"""GPU assembly through the C ABI against the oracle (FP64: 1e-12 relative
Frobenius; mixed: 1e-6), determinism, output residency and error codes."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def cases(femg):
    return {
        "c1_m8": femg.config_c1(m=8),
        "c1_full": femg.config_c1(),
        "c1_p1mesh_dirichlet1": femg.config(dim=2, m=12, mesh_order=1, gauss=2, dirichlet=1, dirichlet_value=1.5, source=1),
        "c2_m3": femg.config_c2(m=3),
        "c2_m4_p1": femg.config_c2(m=4, order=1),
        "c2_m3_p2": femg.config_c2(m=3, order=2),
        "c2_m2_p4": femg.config_c2(m=2, order=4),
        "c3_m4": femg.config_c3(m=4),
        "tet_lagrange_p2": femg.config(dim=3, m=3, mesh_order=2, space=femg.FG_SPACE_LAGRANGE, gauss=4),
        "c5_m2": femg.config_c5(m=2),
        "c5_m3_p1": femg.config(kind=femg.FG_PROBLEM_NAVIER, dim=3, m=3, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1,
                                order=1, gauss=2, jitter=0.15, seed=9, omega=2.0, lame_sigma=0.5),
    }


CASES = ["c1_m8", "c1_full", "c1_p1mesh_dirichlet1", "c2_m3", "c2_m4_p1", "c2_m3_p2", "c2_m2_p4", "c3_m4", "tet_lagrange_p2",
         "c5_m2", "c5_m3_p1"]


@pytest.mark.parametrize("case", CASES)
def test_fp64_matches_oracle(femg, oracle, cuda, case):
    prob = femg.Problem(cases(femg)[case])
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64")
    assert rel(v, ref_v) <= FP64_TOL
    if np.linalg.norm(ref_b) > 0:
        assert rel(b, ref_b) <= FP64_TOL
    else:
        assert np.all(b == 0)


@pytest.mark.parametrize("case", ["c2_m3", "c1_m8"])
def test_fp64_deterministic(femg, cuda, case):
    prob = femg.Problem(cases(femg)[case])
    plan = prob.plan()
    v1, b1 = plan.assemble("fp64")
    v2, b2 = plan.assemble("fp64")
    assert np.array_equal(v1.view(np.uint64), v2.view(np.uint64))
    assert np.array_equal(b1.view(np.uint64), b2.view(np.uint64))


def test_device_outputs_and_bound_terms(femg, cuda):
    torch = cuda
    prob = femg.Problem(femg.config_c3(m=3))
    plan = prob.plan()
    v_host, b_host = plan.assemble("fp64")
    plan.bind_terms()
    dv = torch.empty(2 * prob.nnz, dtype=torch.float64, device="cuda")
    db = torch.empty(2 * int(prob.sys.n_rows), dtype=torch.float64, device="cuda")
    plan.assemble("fp64", values=dv.data_ptr(), rhs=db.data_ptr(), bound=True,
                  stream=C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    v_dev = dv.cpu().numpy().view(np.complex128)
    assert np.array_equal(v_dev.view(np.uint64), v_host.view(np.uint64))


def test_pattern_mismatch_is_an_index_error(femg, cuda):
    prob = femg.Problem(femg.config_c2(m=2))
    ai = np.ctypeslib.as_array(prob.sys.ai, shape=(int(prob.sys.n_rows) + 1,)).copy()
    aj = np.ctypeslib.as_array(prob.sys.aj, shape=(int(ai[-1]),)).copy()
    aj_bad = aj.copy()
    aj_bad[ai[5]] = aj_bad[ai[5] + 1]  # drop a column from row 5 (duplicate its neighbour)
    sysd = femg.SystemDesc(prob.sys.n_rows, prob.sys.ai, aj_bad.ctypes.data_as(C.POINTER(C.c_uint64)),
                           prob.sys.elem_dof_idx, prob.sys.elem_dof_type, prob.sys.n_fixed)
    ptr = C.c_void_p()
    st = femg.lib().fg_plan_create(C.byref(prob.mesh), C.byref(prob.rule), C.byref(prob.space), C.byref(sysd), C.byref(ptr))
    assert st == femg.FG_ERR_INDEX
    assert b"pattern" in femg.lib().fg_last_error()


def test_bad_descriptor_is_an_argument_error(femg, cuda):
    prob = femg.Problem(femg.config_c2(m=2))
    mesh = femg.MeshDesc(prob.mesh.dim, 11, prob.mesh.n_nodes, prob.mesh.node_xyz, prob.mesh.n_elements, prob.mesh.elem_nodes)
    ptr = C.c_void_p()
    st = femg.lib().fg_plan_create(C.byref(mesh), C.byref(prob.rule), C.byref(prob.space), C.byref(prob.sys), C.byref(ptr))
    assert st == femg.FG_ERR_ARG


def _vertex_vector(prob, a, fn):
    rd = prob.raw_dofs()
    u = np.zeros(int(a["n_rows"]))
    vert = (rd["num_type"] == 0) & ((rd["assemble_type"] == 2) | (rd["assemble_type"] == 3))
    u[(rd["num_dof"][vert] - 1).astype(np.int64)] = fn(a["xyz"][(rd["entity"][vert] - 1).astype(np.int64)])
    return u


def _quad(a, v, u, w):
    ai, aj = a["ai"].astype(np.int64), a["aj"].astype(np.int64)
    rows = np.repeat(np.arange(len(ai) - 1), np.diff(ai))
    return np.sum(u[rows] * v * w[aj])


def test_full_size_c2_properties(femg, cuda):
    """384,000 tets, order 3: symmetry and exact energies of 1 and x, beside
    the entry-wise comparison with the oracle in test_gpu_full_size.py."""
    k = 20.0
    prob = femg.Problem(femg.config_c2())
    a = prob.arrays()
    assert a["E"] == 384000 and a["n_rows"] == 121 ** 3
    v, _ = prob.plan().assemble("fp64")
    assert np.all(v.imag == 0)
    one = _vertex_vector(prob, a, lambda X: np.ones(len(X)))
    x = _vertex_vector(prob, a, lambda X: X[:, 0])
    assert abs(_quad(a, v.real, one, one) - (-k * k)) < 1e-9 * k * k
    assert abs(_quad(a, v.real, x, x) - (1.0 - k * k / 3.0)) < 1e-9 * k * k
    # symmetry: A[i, j] == A[j, i]
    ai, aj = a["ai"].astype(np.int64), a["aj"].astype(np.int64)
    rows = np.repeat(np.arange(len(ai) - 1), np.diff(ai))
    key = rows * int(a["n_rows"]) + aj
    keyT = aj * int(a["n_rows"]) + rows
    order = np.argsort(key)
    pos = np.searchsorted(key[order], keyT)
    assert np.allclose(v.real, v.real[order[pos]], rtol=0, atol=1e-12 * np.abs(v.real).max())


MIXED_CASES = ["c2_m3", "c2_m4_p1", "c2_m3_p2", "c2_m2_p4", "c3_m4", "c1_m8", "c1_full", "c1_p1mesh_dirichlet1", "c5_m2", "c5_m3_p1"]


@pytest.mark.parametrize("case", MIXED_CASES)
def test_mixed_matches_oracle(femg, oracle, cuda, case):
    """3xTF32 tensor-core contraction: global relative Frobenius error <= 1e-6
    against the FP64 oracle, per-element report against the device FP64 path."""
    prob = femg.Problem(cases(femg)[case])
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b, rep = plan.assemble("mixed", report=True)
    assert rel(v, ref_v) <= MIXED_TOL
    assert rep["global_"] <= MIXED_TOL
    assert rep["max_elem"] <= 10 * MIXED_TOL
    if np.linalg.norm(ref_b) > 0:
        # source terms stay FP64; the Dirichlet lifting reads the FP32 element matrices
        lifted = a["n_fixed"] > 0 and np.any(a["dirichlet"] != 0)
        assert rel(b, ref_b) <= (MIXED_TOL if lifted else FP64_TOL)


def test_mixed_deterministic_and_complex(femg, cuda):
    prob = femg.Problem(femg.config_c3(m=3))
    plan = prob.plan()
    v1, _ = plan.assemble("mixed")
    v2, _ = plan.assemble("mixed")
    assert np.array_equal(v1.view(np.uint64), v2.view(np.uint64))
    v64, _ = plan.assemble("fp64")
    assert rel(v1, v64) <= MIXED_TOL


@pytest.mark.parametrize("case", ["scalar_m32", "elastic_m16"])
def test_mixed_many_tiles_per_cta(femg, oracle, cuda, case):
    """Sizes at which every persistent contraction CTA walks several tiles,
    across orientation changes; the elastic rows (9 per element) put tile
    boundaries inside elements. Two runs are bit-identical."""
    c = {"scalar_m32": femg.config_c3(m=32), "elastic_m16": femg.config_c5(m=16)}[case]
    prob = femg.Problem(c)
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v1, _ = plan.assemble("mixed")
    v2, _ = plan.assemble("mixed")
    assert np.array_equal(v1.view(np.uint64), v2.view(np.uint64))
    assert rel(v1, ref_v) <= MIXED_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_host_outputs_equal_device_outputs(femg, cuda, precision):
    """Host outputs go through the reduction range by range, each range copied
    out while the next reduces; the values are those of device outputs, bit
    for bit (24,576 P3 tets: 117,649 rows, eight ranges)."""
    torch = cuda
    prob = femg.Problem(femg.config_c3(m=16))
    plan = prob.plan()
    hv, hb = plan.assemble(precision)
    dv = torch.zeros(2 * prob.nnz, dtype=torch.float64, device="cuda")
    db = torch.zeros(2 * int(prob.sys.n_rows), dtype=torch.float64, device="cuda")
    plan.assemble(precision, values=dv.data_ptr(), rhs=db.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(hv.view(np.float64), dv.cpu().numpy())
    assert np.array_equal(hb.view(np.float64), db.cpu().numpy())


@pytest.mark.parametrize("case", ["c3_m4", "c1_m8", "c2_m2_p4", "tet_lagrange_p2"])
def test_fp64_methods_agree(femg, oracle, cuda, case):
    """FG_FP64_QUADRATURE (the plain quadrature loop) and FG_FP64_FACTORED
    (exact factorization on affine elements, FP64) both give the oracle's
    CSR; an unknown method is an argument error."""
    prob = femg.Problem(cases(femg)[case])
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v_quad, _ = plan.assemble("fp64")
    plan.set_fp64_method(femg.FG_FP64_FACTORED)
    v_auto, _ = plan.assemble("fp64")
    assert rel(v_auto, ref_v) <= FP64_TOL and rel(v_quad, ref_v) <= FP64_TOL
    assert rel(v_auto, v_quad) <= FP64_TOL
    assert femg.lib().fg_plan_set_fp64_method(plan.ptr, 7) == femg.FG_ERR_ARG
