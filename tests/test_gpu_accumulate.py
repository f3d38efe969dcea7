"""Buckets that share rows add into one system (fg_plan_set_accumulate), as
the reference's _assembleDim adds every (element type, entity) bucket into
one module: a problem's elements split into two plans, each accumulating
into the same device CSR values and right-hand side, give the one-plan
system (FP64: 1e-12; mixed: 1e-6), with Dirichlet lifting and a source.
Also the refusals: host outputs, batches, the mixed error report and the
multi-frequency calls."""
import ctypes as C

import numpy as np
import pytest

from test_tensor_coef import const_expr

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def offset(ptr, ctype, count):
    return C.cast(C.addressof(ptr.contents) + count * C.sizeof(ctype), C.POINTER(ctype))


def sliced_plan(femg, prob, e0, e1):
    """A plan over elements [e0, e1) of the problem (same pattern and numbering)."""
    mesh, space, sys_ = femg.MeshDesc(), femg.SpaceDesc(), femg.SystemDesc()
    C.memmove(C.byref(mesh), C.byref(prob.mesh), C.sizeof(mesh))
    C.memmove(C.byref(space), C.byref(prob.space), C.sizeof(space))
    C.memmove(C.byref(sys_), C.byref(prob.sys), C.sizeof(sys_))
    n = space.n_basis * space.multiplicity
    mesh.n_elements = e1 - e0
    mesh.elem_nodes = offset(prob.mesh.elem_nodes, C.c_int64, e0 * mesh.nodes_per_element)
    if space.elem_orientation:
        space.elem_orientation = offset(prob.space.elem_orientation, C.c_int32, e0)
    sys_.elem_dof_idx = offset(prob.sys.elem_dof_idx, C.c_uint64, e0 * n)
    sys_.elem_dof_type = offset(prob.sys.elem_dof_type, C.c_int32, e0 * n)
    ptr = C.c_void_p()
    femg.check(femg.lib().fg_plan_create(C.byref(mesh), C.byref(prob.rule), C.byref(space), C.byref(sys_), C.byref(ptr)))
    return ptr


def constant_terms(femg, prob):
    """The problem's bilinear terms with constant coefficients, and a constant source."""
    t, nt = prob.terms()
    bil = [i for i in range(nt) if t[i].kind != femg.FG_TERM_SOURCE]
    arr = (femg.TermDesc * (len(bil) + 1))()
    for k, i in enumerate(bil):
        C.memmove(C.byref(arr[k]), C.byref(t[i]), C.sizeof(femg.TermDesc))
        const_expr(femg, arr[k].coef, 1.0 + 0.5 * k, 0.25 * k)
    s = arr[len(bil)]
    s.kind, s.dt = femg.FG_TERM_SOURCE, 0
    const_expr(femg, s.coef, 2.0, -1.0)
    return arr, len(bil) + 1


CASES = {
    "c1_dirichlet": lambda f: f.config(dim=2, m=8, mesh_order=2, space=f.FG_SPACE_LAGRANGE, gauss=4, dirichlet=1, dirichlet_value=0.5),
    "tet_p3": lambda f: f.config(dim=3, m=3, mesh_order=1, space=f.FG_SPACE_HIERARCHICAL_H1, order=3, gauss=6, jitter=0.15, seed=2),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_buckets_add_up(femg, cuda, case, precision):
    torch = cuda
    prob = femg.Problem(CASES[case](femg))
    t, nt = constant_terms(femg, prob)
    ref_v, ref_b = prob.plan().assemble("fp64", terms=(t, nt))
    E = prob.E
    L = femg.lib()
    dv = torch.zeros(2 * prob.nnz, dtype=torch.float64, device="cuda")
    db = torch.zeros(2 * int(prob.sys.n_rows), dtype=torch.float64, device="cuda")
    dptr = C.cast(prob.dir_ptr, C.c_void_p) if prob.sys.n_fixed else None
    plans = [sliced_plan(femg, prob, 0, E // 3), sliced_plan(femg, prob, E // 3, E)]
    try:
        for pl in plans:
            femg.check(L.fg_plan_set_accumulate(pl, 1))
            if precision == "fp64":
                st = L.fg_assemble_fp64(pl, t, nt, 0.0, dptr, dv.data_ptr(), db.data_ptr(), None)
            else:
                st = L.fg_assemble_mixed(pl, t, nt, 0.0, dptr, dv.data_ptr(), db.data_ptr(), None, None)
            femg.check(st)
        torch.cuda.synchronize()
        v = dv.cpu().numpy().view(np.complex128)
        b = db.cpu().numpy().view(np.complex128)
        tol = 1e-12 if precision == "fp64" else 1e-6
        assert rel(v, ref_v) <= tol and rel(b, ref_b) <= tol
        # refusals: host outputs, the mixed error report, batches, several frequencies
        hv = np.zeros(prob.nnz, np.complex128)
        assert L.fg_assemble_fp64(plans[0], t, nt, 0.0, dptr, hv.ctypes.data, None, None) == femg.FG_ERR_ARG
        rep = femg.ErrReport()
        assert L.fg_assemble_mixed(plans[0], t, nt, 0.0, dptr, dv.data_ptr(), None, None, C.byref(rep)) == femg.FG_ERR_ARG
        bp = C.c_void_p()
        ptrs = (C.c_void_p * 1)(plans[0].value)
        tl = (C.c_void_p * 1)(C.cast(t, C.c_void_p).value)
        nl = (C.c_int32 * 1)(nt)
        assert L.fg_batch_create(ptrs, tl, nl, 1, 0, C.byref(bp)) == femg.FG_ERR_UNSUPPORTED
        om = np.array([1.0])
        assert L.fg_assemble_multi_freq(plans[0], t, nt, om.ctypes.data, 1, 0, dptr, dv.data_ptr(), None, None) == \
            femg.FG_ERR_UNSUPPORTED
        # back to overwriting: each bucket's own rows only
        femg.check(L.fg_plan_set_accumulate(plans[0], 0))
        assert L.fg_plan_set_accumulate(plans[0], 2) == femg.FG_ERR_ARG
    finally:
        for pl in plans:
            L.fg_plan_destroy(pl)
