"""The drop-in binding's cases (fem-g_gb300/binding/GpuFormulation.h compiled
against the reference's headers into oracle/_ref/ref_dropin) and the replay
of its recorded C ABI calls, shared by the CPU and GPU tests and by
tests/golden/make_dropin.py."""
import ctypes as C

import numpy as np

from coef_programs import nonsym_terms
from coef_programs import terms as program_terms


def dt_programs(F):
    """grad-grad, mass and source, plus a point-dependent damping term
    c dt_dof(u) and an inertia term 2 dt2_dof(u)"""
    from coef_programs import argument
    one = [(F.FG_OP_CONST, 0, 1.0, 0.0)]
    src = [(F.FG_OP_CONST, 0, 1.0, 0.0), (F.FG_OP_X, 0, 0, 0), (F.FG_OP_Y, 0, 0, 0), (F.FG_OP_MUL, 0, 0, 0),
           (F.FG_OP_ADD, 0, 0, 0)]
    return {"grad": one, "mass": [(F.FG_OP_CONST, 0, -1.5, 0.0)], "source": src, "damping": argument(F),
            "inertia": [(F.FG_OP_CONST, 0, 2.0, 0.0)]}


def tensor_programs(F, name, rows):
    """programs name_0 .. name_8 of the constant 3 x 3 tensor `rows` (complex entries)"""
    return {"%s_%d" % (name, 3 * i + j): [(F.FG_OP_CONST, 0, complex(rows[i][j]).real, complex(rows[i][j]).imag)]
            for i in range(3) for j in range(3)}


def cases(F):
    """name -> (fg_problem_config, coefficient programs or None)"""
    _, _, progs = program_terms(F, "SQRT")
    return {
        # the same terms as separate matrices K, C, M (assemble(separate = true), the MCK module)
        "separate_mck": (F.config(dim=2, m=4, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=9, omega=1.7),
                         dict(dt_programs(F), separate=[(F.FG_OP_CONST, 0, 1.0, 0.0)])),
        # time derivatives of the unknown at an angular frequency (the AFrequency module)
        "dt_terms": (F.config(dim=2, m=5, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=8, omega=1.7),
                     dt_programs(F)),
        # the 2D P2 workload's terms: grad-grad, -k^2 mass, Dirichlet lifting, disk source
        "c1_m8": (F.config(dim=2, m=8, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=3, k=4.0, source=1,
                           dirichlet=1, dirichlet_value=1.0), None),
        # 3D hierarchical P3 with a per-element mass coefficient (a user nullary operation in the reference)
        "c3_m2": (F.config(dim=3, m=2, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=3, gauss=6, jitter=0.15, seed=5,
                           k=3.0, coef_mode=1, source=1), None),
        # point-dependent complex coefficients: mass sqrt(a(x, y)), source sqrt(a) / 2
        "sqrt_p2": (F.config(dim=2, m=6, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=3), progs),
        # HCurl order 1 (curl-curl and a per-element permittivity) on tets
        "maxwell_p1": (F.config(kind=F.FG_PROBLEM_MAXWELL, dim=3, m=1, mesh_order=1, space=F.FG_SPACE_HCURL, order=1, gauss=4,
                                jitter=0.15, seed=7, k=3.0, coef_mode=1), None),
        # a general tensor diffusion and an advection (point-dependent, partly complex)
        "full_advect": (F.config(dim=2, m=5, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=6),
                        nonsym_terms(F, "both")[2]),
        # b dof(u) tested by grad(v) and a vector source tested by grad(v)
        "vector_terms": (F.config(dim=2, m=5, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=7),
                         nonsym_terms(F, "vector")[2]),
        # two scalar fields coupled both ways (four blocks, two of them two-field plans), Dirichlet on u
        "coupled_p2": (F.config(kind=F.FG_PROBLEM_COUPLED, dim=2, m=5, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4,
                                jitter=0.2, seed=3, k=2.0, source=1, dirichlet=1, dirichlet_value=0.5), None),
        # HCurl order 2 on tets: 45 functions per element (the FP64 path)
        "maxwell_p2": (F.config(kind=F.FG_PROBLEM_MAXWELL, dim=3, m=1, mesh_order=1, space=F.FG_SPACE_HCURL, order=2, gauss=6,
                                jitter=0.15, seed=9, k=2.0, coef_mode=0), None),
        # a three-component field: isotropic elasticity with per-element Lame parameters and an inertia term
        "navier_p2": (F.config(kind=F.FG_PROBLEM_NAVIER, dim=3, m=2, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=2,
                               gauss=4, jitter=0.1, seed=2, omega=0.0, lame_sigma=0.3), None),
        # the same with the frequency in the mass coefficient (-omega^2 rho dof(u))
        "navier_p2_omega": (F.config(kind=F.FG_PROBLEM_NAVIER, dim=3, m=1, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1,
                                     order=2, gauss=4, jitter=0.1, seed=3, omega=2.5, lame_sigma=0.3), None),
        # a symmetric tensor diffusion: the six-entry kind, which the tensor-core path takes too
        "sym_tensor": (F.config(dim=2, m=5, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=10),
                       dict(tensor_programs(F, "dfull", [[1.2, 0.3, 0.1], [0.3, 0.9, -0.2], [0.1, -0.2, 1.1]]),
                            mass=[(F.FG_OP_CONST, 0, -2.0, 0.0)])),
        # anisotropic HCurl media (the PML form): complex symmetric tensors on the curls and the values
        "maxwell_tensor": (F.config(kind=F.FG_PROBLEM_MAXWELL, dim=3, m=1, mesh_order=1, space=F.FG_SPACE_HCURL, order=1,
                                    gauss=4, jitter=0.15, seed=11, k=2.0, coef_mode=0),
                           dict(tensor_programs(F, "dcurl", [[1 + 0.2j, 0.1, 0], [0.1, 0.9 - 0.1j, 0], [0, 0, 1.1]]),
                                **tensor_programs(F, "dmass", [[-1.5 + 0.3j, 0, 0.2], [0, -1.2, 0], [0.2, 0, -1.8 - 0.4j]]))),
        # symmetric storage
        "c1_upper": (F.config(dim=2, m=6, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=4, k=3.0, source=1,
                              dirichlet=1, dirichlet_value=0.5, upper=1), None),
    }


def oracle_arrays(call):
    """oracle.assemble's bucket dictionary of a recorded call"""
    a = dict(call)
    a["n_orient"] = call["n_orient"]
    a["dirichlet"] = call["dirichlet"]
    return a


def oracle_unknown_arrays(call):
    """the unknown field's bucket dictionary of a two-field call"""
    a = oracle_arrays(call)
    a.update(call["unknown"])
    return a


def oracle_assemble(oracle, call, terms):
    """the oracle's assembly of one recorded call"""
    if call.get("unknown") is not None:
        return oracle.assemble_coupled(oracle_arrays(call), oracle_unknown_arrays(call), terms.arr, terms.n, call["frequency"])
    return oracle.assemble(oracle_arrays(call), terms.arr, terms.n, call["frequency"])


def oracle_separate(F, oracle, call):
    """K, C, M and the right-hand side (with K) of a recorded
    fg_assemble_separate call: each group of terms by its time derivative,
    without the frequency factor"""
    out = []
    for dt in range(3):
        sub = dict(call, terms=[(k, 0) + tuple(t[2:]) for t in call["terms"] for k in [t[0]] if t[1] == dt])
        t = Terms(F, sub)
        out.append(oracle.assemble(oracle_arrays(sub), t.arr, t.n, 0.0))
    return out[0][0], out[1][0], out[2][0], out[0][1]


class Terms:
    """fg_term_desc array of a recorded call (keeps its arrays alive)"""

    def __init__(self, F, call):
        self.keep = []
        self.n = len(call["terms"])
        self.arr = (F.TermDesc * max(self.n, 1))()

        def fill(ex, code, arrays):
            ex.n_code = len(code)
            for i, (op, arg, re, im) in enumerate(code):
                ex.code[i].op, ex.code[i].arg, ex.code[i].re, ex.code[i].im = op, arg, re, im
            ex.n_arrays = len(arrays)
            for i, v in enumerate(arrays):
                v = np.ascontiguousarray(v, np.float64)
                self.keep.append(v)
                ex.elem_values[i] = v.ctypes.data_as(C.POINTER(C.c_double))

        for t, (kind, dt, code, arrays, tensor, (code2, arrays2)) in enumerate(call["terms"]):
            d = self.arr[t]
            C.memset(C.byref(d), 0, C.sizeof(F.TermDesc))
            d.kind, d.dt = kind, dt
            fill(d.coef, code, arrays)
            fill(d.coef2, code2, arrays2)
            if tensor:
                ex = (F.Expr * len(tensor))()
                for k, (c, a) in enumerate(tensor):
                    fill(ex[k], c, a)
                self.keep.append(ex)
                d.tensor = C.cast(ex, C.POINTER(F.Expr))


class ReplayPlan:
    """fg_plan_create from a recorded call's descriptors"""

    def __init__(self, F, call):
        self.F, self.L = F, F.lib()
        self.keep = []

        def arr(x, dt):
            x = np.ascontiguousarray(x, dt)
            self.keep.append(x)
            return x

        D, I64, I32, U64 = C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_uint64)
        xyz, en = arr(call["xyz"], np.float64), arr(call["enodes"], np.int64)
        self.mesh = F.MeshDesc(call["dim"], call["nn"], len(xyz), xyz.ctypes.data_as(D), call["E"], en.ctypes.data_as(I64))
        w, gv, gg = arr(call["w"], np.float64), arr(call["geo_val"], np.float64), arr(call["geo_grad"], np.float64)
        self.rule = F.RuleDesc(call["nq"], w.ctypes.data_as(D), gv.ctypes.data_as(D), gg.ctypes.data_as(D))
        bv, bg, orient = arr(call["bval"], np.float64), arr(call["bgrad"], np.float64), arr(call["orient"], np.int32)
        self.space = F.SpaceDesc(call["nb"], call["mult"], call["n_orient"], bv.ctypes.data_as(D), bg.ctypes.data_as(D),
                                 orient.ctypes.data_as(I32) if call["n_orient"] > 1 else None, call["form"])
        ai, aj = arr(call["ai"], np.uint64), arr(call["aj"], np.uint64)
        ed, et = arr(call["edof"], np.uint64), arr(call["etype"], np.int32)
        self.sys = F.SystemDesc(call["n_rows"], ai.ctypes.data_as(U64), aj.ctypes.data_as(U64), ed.ctypes.data_as(U64),
                                et.ctypes.data_as(I32), call["n_fixed"], call["upper"], 0, None, None)
        self.dir = arr(call["dirichlet"], np.complex128)
        self.freq = call["frequency"]
        self.nnz, self.n_rows = len(aj), int(call["n_rows"])
        self.ptr = C.c_void_p()
        u = call.get("unknown")
        if u is None:
            F.check(self.L.fg_plan_create(C.byref(self.mesh), C.byref(self.rule), C.byref(self.space), C.byref(self.sys),
                                          C.byref(self.ptr)))
            return
        ubv, ubg, uor = arr(u["bval"], np.float64), arr(u["bgrad"], np.float64), arr(u["orient"], np.int32)
        self.uspace = F.SpaceDesc(u["nb"], 1, u["n_orient"], ubv.ctypes.data_as(D), ubg.ctypes.data_as(D),
                                  uor.ctypes.data_as(I32) if u["n_orient"] > 1 else None, u["form"])
        ued, uet = arr(u["edof"], np.uint64), arr(u["etype"], np.int32)
        F.check(self.L.fg_plan_create_coupled(C.byref(self.mesh), C.byref(self.rule), C.byref(self.space), C.byref(self.sys),
                                              C.byref(self.uspace), ued.ctypes.data, uet.ctypes.data, C.byref(self.ptr)))

    def assemble(self, precision, terms):
        v = np.zeros(self.nnz, np.complex128)
        r = np.zeros(self.n_rows, np.complex128)
        d = self.dir.ctypes.data if self.dir.size else None
        if precision == "fp64":
            self.F.check(self.L.fg_assemble_fp64(self.ptr, terms.arr, terms.n, self.freq, d, v.ctypes.data, r.ctypes.data, None))
        else:
            self.F.check(self.L.fg_assemble_mixed(self.ptr, terms.arr, terms.n, self.freq, d, v.ctypes.data, r.ctypes.data, None,
                                                  None))
        return v, r

    def assemble_separate(self, terms):
        """fg_assemble_separate: K, C, M, rhs"""
        k, c, m = (np.zeros(self.nnz, np.complex128) for _ in range(3))
        r = np.zeros(self.n_rows, np.complex128)
        d = self.dir.ctypes.data if self.dir.size else None
        self.F.check(self.L.fg_assemble_separate(self.ptr, terms.arr, terms.n, 0, d, k.ctypes.data, c.ctypes.data, m.ctypes.data,
                                                 r.ctypes.data, None))
        return k, c, m, r

    def close(self):
        self.L.fg_plan_destroy(self.ptr)


FIXTURE_KEYS = ["dim", "nn", "E", "xyz", "enodes", "nq", "w", "geo_val", "geo_grad", "nb", "mult", "n_orient", "form", "bval",
                "bgrad", "orient", "n_rows", "ai", "aj", "edof", "etype", "n_fixed", "upper", "frequency", "dirichlet"]


UNKNOWN_KEYS = ["nb", "n_orient", "form", "bval", "bgrad", "orient", "edof", "etype"]


def to_fixture(prefix, calls, ref):
    """flat npz entries of a case's recorded calls and the reference's result"""
    out = {prefix + "n_calls": np.asarray(len(calls)), prefix + "ref_values": ref["values"], prefix + "ref_rhs": ref["rhs"]}
    if "C" in ref:  # separate matrices: values are K
        out[prefix + "ref_C"], out[prefix + "ref_M"] = ref["C"], ref["M"]
    for k, call in enumerate(calls):
        out.update(_call_to_fixture("%s%d/" % (prefix, k), call))
    return out


def _call_to_fixture(prefix, call):
    out = {prefix + k: np.asarray(call[k]) for k in FIXTURE_KEYS}
    out[prefix + "entry"] = np.asarray(call.get("entry", 0))
    u = call.get("unknown")
    out[prefix + "coupled"] = np.asarray(0 if u is None else 1)
    if u is not None:
        for k in UNKNOWN_KEYS:
            out[prefix + "u_" + k] = np.asarray(u[k])
    out[prefix + "n_terms"] = np.asarray(len(call["terms"]))

    def put(key, code, arrays):
        out[key + "_code"] = np.asarray(code, np.float64).reshape(-1, 4)
        for i, v in enumerate(arrays):
            out["%s_array%d" % (key, i)] = np.asarray(v)
        out[key + "_n_arrays"] = np.asarray(len(arrays))

    for t, (kind, dt, code, arrays, tensor, (code2, arrays2)) in enumerate(call["terms"]):
        key = "%sterm%d" % (prefix, t)
        out[key + "_kind"] = np.asarray([kind, dt, len(tensor)])
        put(key, code, arrays)
        put(key + "_coef2", code2, arrays2)
        for k, (c, a) in enumerate(tensor):
            put("%s_tensor%d" % (key, k), c, a)
    return out


def from_fixture(z, prefix):
    """(recorded calls, reference values, reference rhs) of a case from the npz;
    for separate matrices the values are K"""
    calls = [_call_from_fixture(z, "%s%d/" % (prefix, k)) for k in range(int(z[prefix + "n_calls"]))]
    return calls, z[prefix + "ref_values"], z[prefix + "ref_rhs"]


def separate_refs(z, prefix):
    """the reference's C and M of a separate-matrices case, or None"""
    return (z[prefix + "ref_C"], z[prefix + "ref_M"]) if prefix + "ref_C" in z.files else None


def _call_from_fixture(z, prefix):
    call = {}
    for k in FIXTURE_KEYS:
        v = z[prefix + k]
        call[k] = v.item() if v.ndim == 0 else v
    def get(key):
        code = [(int(c[0]), int(c[1]), float(c[2]), float(c[3])) for c in z[key + "_code"]]
        return code, [z["%s_array%d" % (key, i)] for i in range(int(z[key + "_n_arrays"]))]

    terms = []
    for t in range(int(z[prefix + "n_terms"])):
        key = "%sterm%d" % (prefix, t)
        kind, dt, nt = (int(x) for x in z[key + "_kind"])
        code, arrays = get(key)
        terms.append((kind, dt, code, arrays, [get("%s_tensor%d" % (key, k)) for k in range(nt)], get(key + "_coef2")))
    call["terms"] = terms
    call["entry"] = int(z[prefix + "entry"])
    call["unknown"] = None
    if int(z[prefix + "coupled"]):
        call["unknown"] = {k: (z[prefix + "u_" + k].item() if z[prefix + "u_" + k].ndim == 0 else z[prefix + "u_" + k])
                           for k in UNKNOWN_KEYS}
    return call
