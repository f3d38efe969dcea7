"""Python access to libfemg.so through its C ABI (ctypes only).

The library is the product: CUDA kernels for sm_103a plus the host-side
mirror of GmshFEM's Formulation interface. This module only binds the C
entry points declared in include/fem_g_gb300.h and include/fem_g_gb300_host.h
and converts arrays; it computes nothing itself. Loading fails loudly when
the library is missing or was not built.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfemg.so")
HOST_LIB_PATH = os.path.join(HERE, "_build", "libfemg_host.so")

FG_OK, FG_ERR_ARG, FG_ERR_OOM, FG_ERR_CUDA, FG_ERR_INDEX, FG_ERR_TIMEOUT, FG_ERR_UNSUPPORTED, FG_ERR_NO_DEVICE = range(8)
(FG_TERM_GRAD_GRAD, FG_TERM_MASS, FG_TERM_ELASTIC, FG_TERM_SOURCE, FG_TERM_GRAD_GRAD_TENSOR, FG_TERM_MASS_TENSOR,
 FG_TERM_GRAD_GRAD_TENSOR_FULL, FG_TERM_ADVECTION, FG_TERM_VECTOR_GRAD_TEST, FG_TERM_SOURCE_GRAD) = range(10)
FG_PROBLEM_HELMHOLTZ, FG_PROBLEM_NAVIER, FG_PROBLEM_MAXWELL, FG_PROBLEM_COUPLED = range(4)
FG_SPACE_LAGRANGE, FG_SPACE_HIERARCHICAL_H1, FG_SPACE_HCURL = range(3)
FG_FORM_0, FG_FORM_1 = range(2)
(FG_AT_UNDEFINED, FG_AT_FIXED, FG_AT_UNKNOWN, FG_AT_UNKNOWN_BUBBLE, FG_AT_UNKNOWN_GLOBAL, FG_AT_LINKED,
 FG_AT_LINKED_BUBBLE) = range(7)
FG_DT_NONE, FG_DT_1, FG_DT_2 = range(3)
FG_JACMOD_NONE, FG_JACMOD_AXISYMMETRY, FG_JACMOD_AXISYMMETRY_SHELL, FG_JACMOD_POLAR_SHELL, FG_JACMOD_CYLINDRICAL_SHELL, \
    FG_JACMOD_SPHERICAL_SHELL = range(6)
FG_FP64_QUADRATURE, FG_FP64_FACTORED = range(2)
(FG_OP_CONST, FG_OP_X, FG_OP_Y, FG_OP_Z, FG_OP_ELEM, FG_OP_ADD, FG_OP_SUB, FG_OP_MUL, FG_OP_DIV, FG_OP_NEG,
 FG_OP_HEAVISIDE, FG_OP_FIELD, FG_OP_SQRT, FG_OP_EXP, FG_OP_LN, FG_OP_LOG10, FG_OP_POW, FG_OP_SIN, FG_OP_COS, FG_OP_TAN,
 FG_OP_SINH, FG_OP_COSH, FG_OP_TANH, FG_OP_ASIN, FG_OP_ACOS, FG_OP_ATAN, FG_OP_ASINH, FG_OP_ACOSH, FG_OP_ATANH, FG_OP_ABS,
 FG_OP_CONJ, FG_OP_REAL, FG_OP_IMAG, FG_OP_CBRT, FG_OP_ATAN2, FG_OP_POINT) = range(36)
FG_EXPR_MAX_CODE = 32
FG_EXPR_MAX_ARRAYS = 4


class FgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("status %d: %s" % (status, msg))
        self.status = status


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nodes_per_element", C.c_int32), ("n_nodes", C.c_int64),
                ("node_xyz", C.POINTER(C.c_double)), ("n_elements", C.c_int64), ("elem_nodes", C.POINTER(C.c_int64))]


class RuleDesc(C.Structure):
    _fields_ = [("nq", C.c_int32), ("weights", C.POINTER(C.c_double)), ("geo_val", C.POINTER(C.c_double)),
                ("geo_grad", C.POINTER(C.c_double))]


class SpaceDesc(C.Structure):
    _fields_ = [("n_basis", C.c_int32), ("multiplicity", C.c_int32), ("n_orientations", C.c_int32),
                ("basis_val", C.POINTER(C.c_double)), ("basis_grad", C.POINTER(C.c_double)),
                ("elem_orientation", C.POINTER(C.c_int32)), ("form", C.c_int32)]


class SystemDesc(C.Structure):
    _fields_ = [("n_rows", C.c_uint64), ("ai", C.POINTER(C.c_uint64)), ("aj", C.POINTER(C.c_uint64)),
                ("elem_dof_idx", C.POINTER(C.c_uint64)), ("elem_dof_type", C.POINTER(C.c_int32)), ("n_fixed", C.c_uint64),
                ("upper", C.c_int32), ("n_linked", C.c_uint64), ("linked_row", C.POINTER(C.c_uint64)),
                ("linked_value", C.POINTER(C.c_double))]


class Instr(C.Structure):
    _fields_ = [("op", C.c_int32), ("arg", C.c_int32), ("re", C.c_double), ("im", C.c_double)]


class Expr(C.Structure):
    _fields_ = [("n_code", C.c_int32), ("code", Instr * FG_EXPR_MAX_CODE), ("n_arrays", C.c_int32),
                ("elem_values", C.POINTER(C.c_double) * FG_EXPR_MAX_ARRAYS)]


class JacMod(C.Structure):
    _fields_ = [("kind", C.c_int32), ("axis", C.c_int32), ("exponent", C.c_int32), ("pad_", C.c_int32),
                ("r_min", C.c_double), ("r_max", C.c_double), ("center", C.c_double * 3)]


class TermDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("dt", C.c_int32), ("coef", Expr), ("coef2", Expr), ("jacmod", JacMod),
                ("tensor", C.POINTER(Expr))]


class ErrReport(C.Structure):
    _fields_ = [("max_elem_rel_fro", C.c_double), ("mean_elem_rel_fro", C.c_double), ("global_rel_fro", C.c_double)]


class ProblemConfig(C.Structure):
    _fields_ = [("kind", C.c_int32), ("dim", C.c_int32), ("m", C.c_int32), ("mesh_order", C.c_int32),
                ("space", C.c_int32), ("order", C.c_int32), ("gauss", C.c_int32), ("jitter", C.c_double),
                ("seed", C.c_uint64), ("k", C.c_double), ("coef_mode", C.c_int32), ("dirichlet", C.c_int32),
                ("dirichlet_value", C.c_double), ("source", C.c_int32), ("omega", C.c_double),
                ("lame_sigma", C.c_double), ("upper", C.c_int32), ("order2", C.c_int32)]


_lib = None
_host_lib = None


def lib():
    """Load libfemg.so (build it first with build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libfemg.so is not built: run __graft_entry__.build()")
    _lib = _bind(C.CDLL(LIB_PATH))
    return _lib


def host_lib():
    """Load libfemg_host.so: the host mirror alone (problem set-up and pre(),
    no GPU code), for processes that must not map the GPU library."""
    global _host_lib
    if _host_lib is not None:
        return _host_lib
    if not os.path.exists(HOST_LIB_PATH):
        raise RuntimeError("libfemg_host.so is not built: run __graft_entry__.build()")
    _host_lib = _bind(C.CDLL(HOST_LIB_PATH))
    return _host_lib


def _bind(L):
    P = C.c_void_p
    sig = {
        "fg_plan_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(RuleDesc), C.POINTER(SpaceDesc), C.POINTER(SystemDesc), C.POINTER(P)]),
        "fg_plan_create_coupled": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(RuleDesc), C.POINTER(SpaceDesc), C.POINTER(SystemDesc),
                                             C.POINTER(SpaceDesc), P, P, C.POINTER(P)]),
        "fg_plan_destroy": (None, [P]),
        "fg_plan_info": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "fg_plan_bind_terms": (C.c_int, [P, C.POINTER(TermDesc), C.c_int32, C.c_double]),
        "fg_assemble_fp64": (C.c_int, [P, C.POINTER(TermDesc), C.c_int32, C.c_double, P, P, P, P]),
        "fg_assemble_mixed": (C.c_int, [P, C.POINTER(TermDesc), C.c_int32, C.c_double, P, P, P, P, C.POINTER(ErrReport)]),
        "fg_assemble_fp64_static": (C.c_int, [P, P, P, P, P]),
        "fg_assemble_multi_freq": (C.c_int, [P, C.POINTER(TermDesc), C.c_int32, P, C.c_int32, C.c_int32, P, P, P, P]),
        "fg_assemble_separate": (C.c_int, [P, C.POINTER(TermDesc), C.c_int32, C.c_int32, P, P, P, P, P, P]),
        "fg_batch_create": (C.c_int, [P, P, P, C.c_int32, C.c_int32, C.POINTER(P)]),
        "fg_batch_run": (C.c_int, [P, P, P, P]),
        "fg_batch_destroy": (None, [P]),
        "fg_batch_tuning": (C.c_char_p, [P]),
        "fg_pattern_build": (C.c_int, [P, P, C.c_int64, C.c_int32, C.c_uint64, P, C.POINTER(P), C.c_int32, P, C.c_uint64]),
        "fg_plan_set_fp64_method": (C.c_int, [P, C.c_int32]),
        "fg_plan_set_accumulate": (C.c_int, [P, C.c_int32]),
        "fg_plan_set_mixed_fused": (C.c_int, [P, C.c_int32]),
        "fg_set_wait_limit": (C.c_int, [C.c_double]),
        "fg_plan_fused_info": (C.c_int, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "fg_hilbert_order": (C.c_int, [C.c_int32, C.c_uint64, P, P, P, P]),
        "fg_hilbert_numbering": (C.c_int, [C.c_int32, P, C.c_uint64, P, P, P]),
        "fg_profile_enable": (C.c_int, [C.c_int]),
        "fg_profile_read": (C.c_int, [C.c_char_p, C.c_int32, P, P, C.c_int32]),
        "fg_last_error": (C.c_char_p, []),
        "fg_launch_count": (C.c_int64, []),
        "fg_host_alloc": (C.c_int, [C.POINTER(P), C.c_size_t]),
        "fg_host_free": (None, [P]),
        "fg_problem_create": (C.c_int, [C.POINTER(ProblemConfig), C.POINTER(P)]),
        "fg_problem_destroy": (None, [P]),
        "fg_problem_descs": (C.c_int, [P, C.POINTER(MeshDesc), C.POINTER(RuleDesc), C.POINTER(SpaceDesc), C.POINTER(SystemDesc),
                                       C.POINTER(C.POINTER(TermDesc)), C.POINTER(C.c_int32), C.POINTER(C.POINTER(C.c_double))]),
        "fg_problem_n_dofs": (C.c_int64, [P]),
        "fg_problem_raw_dofs": (C.c_int, [P, P, P, P, P, P]),
        "fg_problem_created_dofs": (C.c_int, [P, P, P, P, P]),
        "fg_problem_bbox": (C.c_int, [P, P]),
        "fg_problem_reserve_log": (C.c_int64, [P, P, P, C.c_int64]),
        "fg_problem_pre_seconds": (C.c_double, [P]),
        "fg_problem_n_fields": (C.c_int32, [P]),
        "fg_problem_field": (C.c_int, [P, C.c_int32, C.POINTER(SpaceDesc), C.POINTER(C.POINTER(C.c_uint64)),
                                       C.POINTER(C.POINTER(C.c_int32))]),
        "fg_problem_n_blocks": (C.c_int32, [P]),
        "fg_problem_block": (C.c_int, [P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.POINTER(TermDesc)),
                                       C.POINTER(C.c_int32)]),
        "fg_problem_assemble": (C.c_int, [P, C.c_int32, P, P, P]),
        "fg_basis_eval": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64, P, P, P]),
        "fg_basis_orientation": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, P]),
    }
    for name, (res, args) in sig.items():
        if not hasattr(L, name):  # the host-only library has the fg_problem_* calls alone
            continue
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def exported_symbols():
    """Names bound above (the C ABI of both headers)."""
    return [
        "fg_plan_create", "fg_plan_create_coupled", "fg_plan_destroy", "fg_plan_info", "fg_plan_bind_terms", "fg_plan_set_fp64_method", "fg_plan_set_accumulate", "fg_plan_set_mixed_fused", "fg_plan_fused_info", "fg_set_wait_limit", "fg_assemble_fp64", "fg_assemble_mixed",
        "fg_assemble_fp64_static", "fg_assemble_multi_freq", "fg_assemble_separate", "fg_batch_create", "fg_batch_run", "fg_batch_destroy", "fg_batch_tuning", "fg_pattern_build", "fg_hilbert_order", "fg_hilbert_numbering", "fg_profile_enable",
        "fg_profile_read", "fg_last_error", "fg_launch_count",
        "fg_host_alloc", "fg_host_free", "fg_problem_create", "fg_problem_destroy", "fg_problem_descs", "fg_problem_n_dofs",
        "fg_problem_raw_dofs", "fg_problem_created_dofs", "fg_problem_reserve_log", "fg_problem_bbox", "fg_problem_pre_seconds", "fg_problem_assemble",
        "fg_problem_n_fields", "fg_problem_field", "fg_problem_n_blocks", "fg_problem_block", "fg_basis_eval",
        "fg_basis_orientation",
    ]


def basis_eval(space, order, dim, code, uvw):
    """fg_basis_eval at points uvw [npts][3]: (values, derivatives) with
    values [npts][n] (H1) or [npts][n][3] (HCurl) and derivatives [npts][n][3]
    (gradients or curls)."""
    uvw = np.ascontiguousarray(uvw, np.float64).reshape(-1, 3)
    L = lib()
    n = L.fg_basis_eval(space, order, dim, code, 0, None, None, None)
    if n < 0:
        check(-n)
    shape = (len(uvw), n, 3) if space == FG_SPACE_HCURL else (len(uvw), n)
    val, der = np.zeros(shape), np.zeros((len(uvw), n, 3))
    r = L.fg_basis_eval(space, order, dim, code, len(uvw), uvw.ctypes.data, val.ctypes.data, der.ctypes.data)
    if r < 0:
        check(-r)
    return val, der


def basis_orientation(space, order, dim, vertex_tags):
    """fg_basis_orientation for the global tags of an element's vertices."""
    tags = np.ascontiguousarray(vertex_tags, np.int64)
    r = lib().fg_basis_orientation(space, order, dim, tags.ctypes.data)
    if r < 0:
        check(-r)
    return r


def profile_enable(on=True):
    lib().fg_profile_enable(1 if on else 0)


def profile_read():
    """{kernel name: (launches, total device ms)} since the last read."""
    buf = C.create_string_buffer(4096)
    cnt = np.zeros(64, np.int64)
    ms = np.zeros(64, np.float64)
    k = lib().fg_profile_read(buf, 4096, cnt.ctypes.data, ms.ctypes.data, 64)
    names = buf.value.decode().split("\n")[:k]
    return {n: (int(cnt[i]), float(ms[i])) for i, n in enumerate(names)}


def check(status, L=None):
    if status != FG_OK:
        raise FgError(status, (L or lib()).fg_last_error().decode())


def _arr(ptr, count, dtype):
    if count == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype, copy=True)


def config(kind=FG_PROBLEM_HELMHOLTZ, dim=2, m=4, mesh_order=2, space=FG_SPACE_LAGRANGE, order=1, gauss=4, jitter=0.2,
           seed=1, k=10.0, coef_mode=0, dirichlet=0, dirichlet_value=0.0, source=0, omega=1.0, lame_sigma=0.5, upper=0,
           order2=0):
    return ProblemConfig(kind, dim, m, mesh_order, space, order, gauss, jitter, seed, k, coef_mode, dirichlet,
                         dirichlet_value, source, omega, lame_sigma, upper, order2)


# The benchmark workloads (seeded synthetic inputs with the shapes of the
# reference's configurations)
def config_c1(m=64, seed=1):
    """2D Helmholtz, P2 triangles, Gauss4, k=10, Dirichlet u=0, disk source."""
    return config(dim=2, m=m, mesh_order=2, space=FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=seed, k=10.0,
                  dirichlet=1, source=1)


def config_c2(m=40, seed=2, order=3):
    """3D Helmholtz, Kuhn tets, hierarchical H1 order 3, Gauss6, k=20."""
    return config(dim=3, m=m, mesh_order=1, space=FG_SPACE_HIERARCHICAL_H1, order=order, gauss=6, jitter=0.15, seed=seed,
                  k=20.0)


def config_c3(m=40, seed=2, order=3):
    """c2 mesh with per-tet coefficient -k^2 (1 + 0.3 xi), xi ~ N(0,1)."""
    c = config_c2(m=m, seed=seed, order=order)
    c.coef_mode = 1
    return c


def config_c5(m=60, seed=5, omega=5.0):
    """3D Navier, 3-component hierarchical H1 order 2, Gauss4, lognormal Lame."""
    return config(kind=FG_PROBLEM_NAVIER, dim=3, m=m, mesh_order=1, space=FG_SPACE_HIERARCHICAL_H1, order=2, gauss=4,
                  jitter=0.15, seed=seed, omega=omega, lame_sigma=0.5)


def config_c4(n=64, seed=4, m_lo=8, m_hi=48, orders=(1, 2, 3, 4), k_lo=5.0, k_hi=40.0):
    """Batch of 3D Helmholtz problems: cube resolutions m ~ U{m_lo..m_hi}
    (x 6 tets), hierarchical H1 orders ~ U(orders), k ~ U[k_lo, k_hi],
    jitter 0.15 h, rule Gauss(2p); all drawn from one seed."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        m = int(rng.integers(m_lo, m_hi + 1))
        p = int(rng.choice(orders))
        k = float(rng.uniform(k_lo, k_hi))
        out.append(config(dim=3, m=m, mesh_order=1, space=FG_SPACE_HIERARCHICAL_H1, order=p, gauss=2 * p, jitter=0.15,
                          seed=seed * 1000 + q, k=k))
    return out


class Problem:
    """A problem built by the host mirror (mesh, field, terms, pre()).
    host_only: through libfemg_host.so, without loading the GPU library."""

    def __init__(self, cfg, host_only=False):
        L = host_lib() if host_only else lib()
        self._L = L
        self.ptr = C.c_void_p()
        check(L.fg_problem_create(C.byref(cfg), C.byref(self.ptr)), L)
        self.cfg = cfg
        self.mesh, self.rule, self.space, self.sys = MeshDesc(), RuleDesc(), SpaceDesc(), SystemDesc()
        self.terms_ptr = C.POINTER(TermDesc)()
        self.n_terms = C.c_int32()
        self.dir_ptr = C.POINTER(C.c_double)()
        check(L.fg_problem_descs(self.ptr, C.byref(self.mesh), C.byref(self.rule), C.byref(self.space), C.byref(self.sys),
                                 C.byref(self.terms_ptr), C.byref(self.n_terms), C.byref(self.dir_ptr)), L)

    def close(self):
        if self.ptr:
            self._L.fg_problem_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- arrays (copies)
    @property
    def E(self):
        return self.mesh.n_elements

    @property
    def n(self):
        return self.space.n_basis * self.space.multiplicity

    @property
    def nnz(self):
        return int(self.sys.ai[self.sys.n_rows])  # one element, no copy

    def arrays(self):
        m, r, s, y = self.mesh, self.rule, self.space, self.sys
        nq, nn, nb, no = r.nq, m.nodes_per_element, s.n_basis, s.n_orientations
        out = dict(
            dim=m.dim, nn=nn, nq=nq, nb=nb, mult=s.multiplicity, n_orient=no, E=m.n_elements,
            xyz=_arr(m.node_xyz, 3 * m.n_nodes, np.float64).reshape(-1, 3),
            enodes=_arr(m.elem_nodes, nn * m.n_elements, np.int64).reshape(-1, nn),
            w=_arr(r.weights, nq, np.float64),
            geo_val=_arr(r.geo_val, nq * nn, np.float64).reshape(nq, nn),
            geo_grad=_arr(r.geo_grad, nq * nn * 3, np.float64).reshape(nq, nn, 3),
            form=s.form,
            upper=y.upper,
            bval=(_arr(s.basis_val, no * nq * nb * 3, np.float64).reshape(no, nq, nb, 3) if s.form == FG_FORM_1
                  else _arr(s.basis_val, no * nq * nb, np.float64).reshape(no, nq, nb)),
            bgrad=_arr(s.basis_grad, no * nq * nb * 3, np.float64).reshape(no, nq, nb, 3),
            orient=(_arr(s.elem_orientation, m.n_elements, np.int32) if no > 1 else np.zeros(m.n_elements, np.int32)),
            n_rows=y.n_rows, ai=self.ai, aj=_arr(y.aj, int(self.ai[-1]), np.uint64),
            edof=_arr(y.elem_dof_idx, self.n * m.n_elements, np.uint64).reshape(m.n_elements, self.n),
            etype=_arr(y.elem_dof_type, self.n * m.n_elements, np.int32).reshape(m.n_elements, self.n),
            n_fixed=y.n_fixed,
            dirichlet=(_arr(self.dir_ptr, 2 * y.n_fixed, np.float64).view(np.complex128) if y.n_fixed else np.zeros(0, np.complex128)),
        )
        return out

    @property
    def ai(self):
        return _arr(self.sys.ai, self.sys.n_rows + 1, np.uint64)

    def terms(self):
        return self.terms_ptr, self.n_terms.value

    def raw_dofs(self):
        L = self._L
        n = L.fg_problem_n_dofs(self.ptr)
        nt = np.zeros(n, np.uint64)
        ent = np.zeros(n, np.uint64)
        nd = np.zeros(n, np.uint64)
        at = np.zeros(n, np.int32)
        xyz = np.zeros((n, 3), np.float32)
        check(L.fg_problem_raw_dofs(self.ptr, nt.ctypes.data, ent.ctypes.data, nd.ctypes.data, at.ctypes.data, xyz.ctypes.data))
        return dict(num_type=nt, entity=ent, num_dof=nd, assemble_type=at, xyz=xyz)

    def created_dofs(self):
        L = self._L
        n = L.fg_problem_n_dofs(self.ptr)
        nt = np.zeros(n, np.uint64)
        ent = np.zeros(n, np.uint64)
        at = np.zeros(n, np.int32)
        xyz = np.zeros((n, 3), np.float32)
        check(L.fg_problem_created_dofs(self.ptr, nt.ctypes.data, ent.ctypes.data, at.ctypes.data, xyz.ctypes.data))
        return dict(num_type=nt, entity=ent, assemble_type=at, xyz=xyz)

    def reserve_log(self):
        L = self._L
        n = L.fg_problem_reserve_log(self.ptr, None, None, 0)
        at = np.zeros(n, np.uint64)
        arg = np.zeros(n, np.uint64)
        L.fg_problem_reserve_log(self.ptr, at.ctypes.data, arg.ctypes.data, n)
        return at, arg

    def bbox(self):
        b = np.zeros(6)
        check(self._L.fg_problem_bbox(self.ptr, b.ctypes.data), self._L)
        return b

    def pre_seconds(self):
        return self._L.fg_problem_pre_seconds(self.ptr)

    def plan(self):
        return Plan(self)

    # --- several fields (FG_PROBLEM_COUPLED)
    def n_fields(self):
        return self._L.fg_problem_n_fields(self.ptr)

    def field(self, k):
        """(SpaceDesc, element DOF index [E][n], element DOF type [E][n]) of field k"""
        sp = SpaceDesc()
        ip, tp = C.POINTER(C.c_uint64)(), C.POINTER(C.c_int32)()
        check(self._L.fg_problem_field(self.ptr, k, C.byref(sp), C.byref(ip), C.byref(tp)), self._L)
        n = sp.n_basis * sp.multiplicity
        E = self.mesh.n_elements
        return sp, _arr(ip, n * E, np.uint64).reshape(E, n), _arr(tp, n * E, np.int32).reshape(E, n)

    def field_arrays(self, k):
        """arrays() with the space and element DOF map of field k"""
        a = self.arrays()
        sp, idx, typ = self.field(k)
        nq, no, nb, E = self.rule.nq, sp.n_orientations, sp.n_basis, self.mesh.n_elements
        a.update(nb=nb, mult=sp.multiplicity, n_orient=no, form=sp.form,
                 bval=_arr(sp.basis_val, no * nq * nb, np.float64).reshape(no, nq, nb),
                 bgrad=_arr(sp.basis_grad, no * nq * nb * 3, np.float64).reshape(no, nq, nb, 3),
                 orient=(_arr(sp.elem_orientation, E, np.int32) if no > 1 else np.zeros(E, np.int32)),
                 edof=idx, etype=typ)
        return a

    def blocks(self):
        """[(test field, unknown field, terms pointer, term count)]"""
        out = []
        for b in range(self._L.fg_problem_n_blocks(self.ptr)):
            t, u = C.c_int32(), C.c_int32()
            tp, nt = C.POINTER(TermDesc)(), C.c_int32()
            check(self._L.fg_problem_block(self.ptr, b, C.byref(t), C.byref(u), C.byref(tp), C.byref(nt)), self._L)
            out.append((t.value, u.value, tp, nt.value))
        return out

    def block_plan(self, test, unknown):
        """A plan for the block (test field, unknown field): fg_plan_create
        for test == unknown, fg_plan_create_coupled otherwise; accumulating
        when the problem has several blocks."""
        return Plan(self, test=test, unknown=unknown)


class Plan:
    """fg_plan over a Problem's descriptors (through the C ABI). test,
    unknown: the fields of a block of a multi-field problem (None: the
    problem's first block)."""

    def __init__(self, prob, test=None, unknown=None):
        L = lib()
        self.prob = prob
        self.ptr = C.c_void_p()
        if test is None:
            check(L.fg_plan_create(C.byref(prob.mesh), C.byref(prob.rule), C.byref(prob.space), C.byref(prob.sys),
                                   C.byref(self.ptr)))
            return
        spT, idxT, typT = prob.field(test)
        sys = SystemDesc()
        C.memmove(C.byref(sys), C.byref(prob.sys), C.sizeof(SystemDesc))
        self._keep = (spT, idxT, typT)
        sys.elem_dof_idx = idxT.ctypes.data_as(C.POINTER(C.c_uint64))
        sys.elem_dof_type = typT.ctypes.data_as(C.POINTER(C.c_int32))
        self.sys = sys
        if test == unknown:
            check(L.fg_plan_create(C.byref(prob.mesh), C.byref(prob.rule), C.byref(spT), C.byref(sys), C.byref(self.ptr)))
        else:
            spU, idxU, typU = prob.field(unknown)
            self._keep = self._keep + (spU, idxU, typU)
            check(L.fg_plan_create_coupled(C.byref(prob.mesh), C.byref(prob.rule), C.byref(spT), C.byref(sys), C.byref(spU),
                                           idxU.ctypes.data, typU.ctypes.data, C.byref(self.ptr)))
        if len(prob.blocks()) > 1:
            self.set_accumulate(True)

    def close(self):
        if self.ptr:
            lib().fg_plan_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        nnz, E = C.c_int64(), C.c_int64()
        n, nq, no = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().fg_plan_info(self.ptr, C.byref(nnz), C.byref(E), C.byref(n), C.byref(nq), C.byref(no)))
        return dict(nnz=nnz.value, E=E.value, n=n.value, nq=nq.value, n_orient=no.value)

    def set_fp64_method(self, method):
        check(lib().fg_plan_set_fp64_method(self.ptr, method))

    def set_accumulate(self, on=True):
        check(lib().fg_plan_set_accumulate(self.ptr, 1 if on else 0))

    def set_mixed_fused(self, on=True):
        check(lib().fg_plan_set_mixed_fused(self.ptr, 1 if on else 0))

    def fused_info(self):
        """(applies, blocks, elements per block, contractions per element,
        reason when it does not apply)"""
        a, nb = C.c_int32(), C.c_int32()
        epb, cpe = C.c_double(), C.c_double()
        check(lib().fg_plan_fused_info(self.ptr, C.byref(a), C.byref(nb), C.byref(epb), C.byref(cpe)))
        why = "" if a.value else lib().fg_last_error().decode()
        return dict(applies=bool(a.value), blocks=nb.value, elems_per_block=epb.value, contractions_per_element=cpe.value,
                    why=why)

    def bind_terms(self, frequency=0.0):
        t, nt = self.prob.terms()
        check(lib().fg_plan_bind_terms(self.ptr, t, nt, frequency))

    def assemble_separate(self, precision="fp64", terms=None, with_rhs=True, stream=None):
        """fg_assemble_separate: (K, C, M, rhs) numpy arrays (None for a
        matrix the formulation does not have)."""
        p = self.prob
        t, nt = terms if terms is not None else p.terms()
        have = set(int(t[i].dt) for i in range(nt) if t[i].kind != FG_TERM_SOURCE)
        has_source = any(t[i].kind == FG_TERM_SOURCE for i in range(nt))
        out = [np.zeros(p.nnz, np.complex128) if (d in have or (d == 0 and has_source)) else None for d in range(3)]
        rhs = np.zeros(int(p.sys.n_rows), np.complex128) if with_rhs else None
        ptr = lambda a: a.ctypes.data if a is not None else None
        dptr = C.cast(p.dir_ptr, C.c_void_p) if p.sys.n_fixed else None
        check(lib().fg_assemble_separate(self.ptr, t, nt, 1 if precision == "mixed" else 0, dptr, ptr(out[0]), ptr(out[1]),
                                         ptr(out[2]), ptr(rhs), stream))
        return out[0], out[1], out[2], rhs

    def assemble_multi_freq(self, omegas, precision="fp64", terms=None, values=None, rhs=None, stream=None):
        """fg_assemble_multi_freq: (values [F][nnz], rhs [F][n_rows]) for the
        angular frequencies omegas (numpy outputs unless device pointers)."""
        p = self.prob
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        F = len(om)
        if values is None:
            values = np.zeros((F, p.nnz), np.complex128)
        if rhs is None:
            rhs = np.zeros((F, int(p.sys.n_rows)), np.complex128)
        vptr = values if isinstance(values, int) else values.ctypes.data
        rptr = rhs if isinstance(rhs, int) else (rhs.ctypes.data if rhs is not False else None)
        t, nt = terms if terms is not None else p.terms()
        dptr = C.cast(p.dir_ptr, C.c_void_p) if p.sys.n_fixed else None
        check(lib().fg_assemble_multi_freq(self.ptr, t, nt, om.ctypes.data, F, 1 if precision == "mixed" else 0, dptr,
                                           vptr, rptr, stream))
        return values, rhs

    def assemble(self, precision="fp64", values=None, rhs=None, bound=False, frequency=0.0, stream=None, report=False,
                 terms=None):
        """Assemble into numpy arrays (host outputs) or raw device pointers
        (ints); returns (values, rhs[, report])."""
        L = lib()
        p = self.prob
        nnz = p.nnz
        nrows = p.sys.n_rows
        if values is None:
            values = np.zeros(nnz, np.complex128)
        if rhs is None:
            rhs = np.zeros(nrows, np.complex128)
        vptr = values if isinstance(values, int) else values.ctypes.data
        rptr = rhs if isinstance(rhs, int) else (rhs.ctypes.data if rhs is not False else None)
        t, nt = (None, 0) if bound else (terms if terms is not None else p.terms())
        dptr = C.cast(p.dir_ptr, C.c_void_p) if p.sys.n_fixed else None
        if precision == "fp64":
            check(L.fg_assemble_fp64(self.ptr, t, nt, frequency, dptr, vptr, rptr, stream))
            return values, rhs
        rep = ErrReport()
        check(L.fg_assemble_mixed(self.ptr, t, nt, frequency, dptr, vptr, rptr, stream, C.byref(rep) if report else None))
        if report:
            return values, rhs, dict(max_elem=rep.max_elem_rel_fro, mean_elem=rep.mean_elem_rel_fro, global_=rep.global_rel_fro)
        return values, rhs


class Batch:
    """fg_batch over plans (their problems' terms unless bound=True)."""

    def __init__(self, plans, mixed=False, bound=False):
        L = lib()
        self.plans = list(plans)
        n = len(self.plans)
        self.ptr = C.c_void_p()
        ptrs = (C.c_void_p * n)(*[p.ptr.value for p in self.plans])
        if bound:
            tl = None
            nl = None
        else:
            tl = (C.c_void_p * n)(*[C.cast(p.prob.terms()[0], C.c_void_p).value for p in self.plans])
            nl = (C.c_int32 * n)(*[p.prob.terms()[1] for p in self.plans])
        check(L.fg_batch_create(ptrs, tl, nl, n, 1 if mixed else 0, C.byref(self.ptr)))

    def run(self, values=None, rhs=None, stream=None):
        """values / rhs: lists of numpy arrays or device pointers (ints);
        None allocates numpy outputs (rhs None: no right-hand sides)."""
        n = len(self.plans)
        if values is None:
            values = [np.zeros(p.prob.nnz, np.complex128) for p in self.plans]
        vp = (C.c_void_p * n)(*[v if isinstance(v, int) else v.ctypes.data for v in values])
        rp = None
        if rhs is not None:
            rp = (C.c_void_p * n)(*[r if isinstance(r, int) else r.ctypes.data for r in rhs])
        check(lib().fg_batch_run(self.ptr, vp, rp, stream))
        return values, rhs

    def tuning(self):
        return lib().fg_batch_tuning(self.ptr).decode()

    def close(self):
        if self.ptr:
            lib().fg_batch_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pattern_build(edof, etype, n_rows, upper=False, linked_row=None):
    """fg_pattern_build on an element DOF map ([E][n] indices and types):
    (ai, aj) as numpy uint64 arrays."""
    L = lib()
    edof = np.ascontiguousarray(edof, np.uint64)
    etype = np.ascontiguousarray(etype, np.int32)
    E, n = edof.shape
    ai = np.zeros(int(n_rows) + 1, np.uint64)
    ajp = C.c_void_p()
    lrow = None if linked_row is None else np.ascontiguousarray(linked_row, np.uint64)
    check(L.fg_pattern_build(edof.ctypes.data, etype.ctypes.data, E, n, int(n_rows), ai.ctypes.data, C.byref(ajp),
                             1 if upper else 0, lrow.ctypes.data if lrow is not None and lrow.size else None,
                             0 if lrow is None else len(lrow)))
    nnz = int(ai[-1])
    aj = np.ctypeslib.as_array(C.cast(ajp, C.POINTER(C.c_uint64)), shape=(max(nnz, 1),))[:nnz].copy()
    L.fg_host_free(ajp)
    return ai, aj


def hilbert_order(dim, pts, mn, mx):
    """fg_hilbert_order: the stable Hilbert order of float points [n][dim]."""
    pts = np.ascontiguousarray(pts, np.float32)
    mn = np.ascontiguousarray(mn, np.float32)
    mx = np.ascontiguousarray(mx, np.float32)
    perm = np.zeros(len(pts), np.uint32)
    check(lib().fg_hilbert_order(dim, len(pts), pts.ctypes.data, mn.ctypes.data, mx.ctypes.data, perm.ctypes.data))
    return perm


def hilbert_numbering(dim, bbox, xyz, assemble_type, num_dof):
    """fg_hilbert_numbering on DOFs in dictionary order; returns the new num_dof."""
    bbox = np.ascontiguousarray(bbox, np.float64)
    xyz = np.ascontiguousarray(xyz, np.float32)
    at = np.ascontiguousarray(assemble_type, np.int32)
    out = np.ascontiguousarray(num_dof, np.uint64).copy()
    check(lib().fg_hilbert_numbering(dim, bbox.ctypes.data, len(at), xyz.ctypes.data, at.ctypes.data, out.ctypes.data))
    return out
