"""Edge cases of the assembly path on the GPU: a bucket without elements, a
system whose DOFs are all fixed (no rows), one or two elements, complex
element matrices on the tensor-core path (damping term at a frequency), and
rows longer than 254 entries (16-bit slots)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def test_bucket_without_elements_writes_zeros(femg, cuda):
    prob = femg.Problem(femg.config_c2(m=2))
    mesh = femg.MeshDesc(prob.mesh.dim, prob.mesh.nodes_per_element, prob.mesh.n_nodes, prob.mesh.node_xyz, 0,
                         prob.mesh.elem_nodes)
    ptr = C.c_void_p()
    L = femg.lib()
    assert L.fg_plan_create(C.byref(mesh), C.byref(prob.rule), C.byref(prob.space), C.byref(prob.sys), C.byref(ptr)) == femg.FG_OK
    t, nt = prob.terms()
    v = np.full(prob.nnz, 7.0 + 1j)
    b = np.full(int(prob.sys.n_rows), 3.0 + 0j)
    for fn, extra in ((L.fg_assemble_fp64, ()), (L.fg_assemble_mixed, (None,))):
        assert fn(ptr, t, nt, 0.0, None, v.ctypes.data, b.ctypes.data, None, *extra) == femg.FG_OK
        assert np.all(v == 0) and np.all(b == 0)
        v[:] = 7.0
    L.fg_plan_destroy(ptr)


def test_all_dofs_fixed(femg, oracle, cuda):
    """One square, two triangles, every DOF on the Dirichlet boundary: no rows."""
    prob = femg.Problem(femg.config(dim=2, m=1, mesh_order=1, gauss=2, dirichlet=1, dirichlet_value=2.0, source=1))
    a = prob.arrays()
    assert a["n_rows"] == 0 and prob.nnz == 0
    plan = prob.plan()
    v, b = plan.assemble("fp64", values=np.zeros(1, np.complex128), rhs=np.zeros(1, np.complex128))
    v, b = plan.assemble("mixed", values=np.zeros(1, np.complex128), rhs=np.zeros(1, np.complex128))


@pytest.mark.parametrize("cfg", ["tri_two", "tet_p4_six"])
def test_few_elements(femg, oracle, cuda, cfg):
    c = {"tri_two": femg.config(dim=2, m=1, mesh_order=1, gauss=2, source=1),
         "tet_p4_six": femg.config_c2(m=1, order=4)}[cfg]
    prob = femg.Problem(c)
    a = prob.arrays()
    t, nt = prob.terms()
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    v, b = plan.assemble("fp64")
    assert rel(v, ref_v) <= FP64_TOL
    vm, bm = plan.assemble("mixed")
    assert rel(vm, ref_v) <= MIXED_TOL
    if np.linalg.norm(ref_b) > 0:
        assert rel(b, ref_b) <= FP64_TOL and rel(bm, ref_b) <= FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_complex_element_matrices(femg, oracle, cuda, precision):
    """A damping term dt_dof(u) at omega = 3: -i omega c M makes every element
    matrix complex (two TF32 rows per element on the tensor-core path)."""
    prob = femg.Problem(femg.config_c3(m=3))
    t, nt = prob.terms()
    arr = (femg.TermDesc * 3)()
    for k, (src, dt) in enumerate([(0, 0), (1, 0), (1, 1)]):
        C.memmove(C.byref(arr[k]), C.byref(t[src]), C.sizeof(femg.TermDesc))
        arr[k].dt = dt
    a = prob.arrays()
    ref_v, _ = oracle.assemble(a, arr, 3, freq=3.0)
    assert np.linalg.norm(ref_v.imag) > 0.1 * np.linalg.norm(ref_v.real)
    plan = prob.plan()
    v, _ = plan.assemble(precision, frequency=3.0, terms=(arr, 3))
    assert rel(v, ref_v) <= (FP64_TOL if precision == "fp64" else MIXED_TOL)


def test_long_rows_use_16bit_slots(femg, oracle, cuda):
    """Order 4 on 2^3 x 6 tets: rows of up to 369 entries (slots above 253)."""
    prob = femg.Problem(femg.config_c2(m=2, order=4))
    a = prob.arrays()
    assert int(np.diff(a["ai"].astype(np.int64)).max()) > 254
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt)
    plan = prob.plan()
    for precision, tol in (("fp64", FP64_TOL), ("mixed", MIXED_TOL)):
        v, _ = plan.assemble(precision)
        assert rel(v, ref_v) <= tol


def _point_coefficient_terms(femg, prob):
    """The problem's terms with the mass coefficient multiplied by (1 + x):
    a coefficient that varies inside the elements."""
    t, nt = prob.terms()
    arr = (femg.TermDesc * nt)()
    for k in range(nt):
        C.memmove(C.byref(arr[k]), C.byref(t[k]), C.sizeof(femg.TermDesc))
    mass = [k for k in range(nt) if arr[k].kind == femg.FG_TERM_MASS][0]
    ex = arr[mass].coef
    n = ex.n_code
    extra = [(femg.FG_OP_X, 0, 0.0, 0.0), (femg.FG_OP_CONST, 0, 1.0, 0.0), (femg.FG_OP_ADD, 0, 0.0, 0.0), (femg.FG_OP_MUL, 0, 0.0, 0.0)]
    for i, (op, arg, re, im) in enumerate(extra):
        ex.code[n + i].op, ex.code[n + i].arg, ex.code[n + i].re, ex.code[n + i].im = op, arg, re, im
    ex.n_code = n + len(extra)
    return arr, nt


@pytest.mark.parametrize("cfg", ["tet_p3", "tri_p2_curvedfree"])
def test_point_dependent_coefficient_uses_quadrature(femg, oracle, cuda, cfg):
    c = {"tet_p3": femg.config_c2(m=3), "tri_p2_curvedfree": femg.config_c1(m=6)}[cfg]
    prob = femg.Problem(c)
    a = prob.arrays()
    t, nt = _point_coefficient_terms(femg, prob)
    ref_v, ref_b = oracle.assemble(a, t, nt)
    plan = prob.plan()
    plan.set_fp64_method(femg.FG_FP64_FACTORED)  # not exact here: falls back to the quadrature loop
    v, b = plan.assemble("fp64", terms=(t, nt))
    assert rel(v, ref_v) <= FP64_TOL
    if np.linalg.norm(ref_b) > 0:
        assert rel(b, ref_b) <= FP64_TOL
    with pytest.raises(femg.FgError) as err:
        plan.assemble("mixed", terms=(t, nt))
    assert err.value.status == femg.FG_ERR_UNSUPPORTED
