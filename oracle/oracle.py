"""ctypes access to the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module, as the checker. ``ref()`` returns the reference's own numbering
code (oracle/_ref/libref.so) when it was built from the reference tree in
this container; it is absent on machines without that tree.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None


class Bucket(C.Structure):
    _fields_ = [("dim", C.c_int), ("nn", C.c_int), ("nq", C.c_int), ("nb", C.c_int), ("mult", C.c_int), ("E", C.c_int64),
                ("xyz", C.c_void_p), ("enodes", C.c_void_p), ("w", C.c_void_p), ("geo_val", C.c_void_p),
                ("geo_grad", C.c_void_p), ("bval", C.c_void_p), ("bgrad", C.c_void_p), ("orient", C.c_void_p),
                ("form", C.c_int32), ("upper", C.c_int32), ("linked_row", C.c_void_p), ("linked_value", C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        P = C.c_void_p
        L.or_element_matrices.argtypes = [C.POINTER(Bucket), P, C.c_int, C.c_double, P, P]
        L.or_assemble.argtypes = [C.POINTER(Bucket), P, C.c_int, C.c_double, P, P, P, P, P, P, P]
        L.or_assemble_coupled.argtypes = [C.POINTER(Bucket), C.POINTER(Bucket), P, C.c_int, C.c_double, P, P, P, P, P, P, P,
                                          P, P]
        L.or_pattern.argtypes = [C.c_int64, C.c_int, P, P, C.c_uint64, P, C.POINTER(P), C.c_int, P]
        L.or_free.argtypes = [P]
        L.or_hilbert_keys.argtypes = [C.c_int, C.c_int64, P, P, P, P]
        L.or_hilbert_sort.argtypes = [C.c_int64, P, P]
        L.or_reorder_hilbert.argtypes = [C.c_int, P, C.c_int64, P, P, C.c_uint64, C.c_uint64, P]
        L.or_robin_order.argtypes = [C.c_int64, P, P, P, P, P]
        L.or_robin_order.restype = C.c_int64
        L.or_num_threads.restype = C.c_int
        _lib = L
    return _lib


def ref():
    """The reference's robin_hood.h + Hilbert.cpp driver, or None."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_ref()
            except RuntimeError:
                path = None
        if not path or not os.path.exists(path):
            return None
        R = C.CDLL(path)
        P = C.c_void_p
        R.ref_robin_order.argtypes = [C.c_int64, P, P, P, P, P]
        R.ref_robin_order.restype = C.c_int64
        R.ref_hilbert_order.argtypes = [C.c_int, C.c_int64, P, P, P, P]
        _ref = R
    return _ref


def num_threads():
    return lib().or_num_threads()


class _Keep:
    """Holds numpy arrays alive while a Bucket points into them."""


def bucket(a):
    """Bucket over the arrays of femg.Problem.arrays()."""
    k = _Keep()
    k.xyz = np.ascontiguousarray(a["xyz"], np.float64)
    k.enodes = np.ascontiguousarray(a["enodes"], np.int64)
    k.w = np.ascontiguousarray(a["w"], np.float64)
    k.gv = np.ascontiguousarray(a["geo_val"], np.float64)
    k.gg = np.ascontiguousarray(a["geo_grad"], np.float64)
    k.bv = np.ascontiguousarray(a["bval"], np.float64)
    k.bg = np.ascontiguousarray(a["bgrad"], np.float64)
    k.orient = np.ascontiguousarray(a["orient"], np.int32)
    k.lrow = np.ascontiguousarray(a.get("linked_row", np.zeros(0)), np.uint64)
    k.lval = np.ascontiguousarray(a.get("linked_value", np.zeros(0)), np.complex128)
    b = Bucket(a["dim"], a["nn"], a["nq"], a["nb"], a["mult"], a["E"], k.xyz.ctypes.data, k.enodes.ctypes.data, k.w.ctypes.data,
               k.gv.ctypes.data, k.gg.ctypes.data, k.bv.ctypes.data, k.bg.ctypes.data,
               k.orient.ctypes.data if a["n_orient"] > 1 else None, int(a.get("form", 0)), int(a.get("upper", 0)),
               k.lrow.ctypes.data if k.lrow.size else None, k.lval.ctypes.data if k.lval.size else None)
    b._keep = k
    return b


def element_matrices(a, terms_ptr, n_terms, freq=0.0):
    """Ke [E][n][n] complex (row: test, column: unknown) and be [E][n]."""
    b = bucket(a)
    n = a["nb"] * a["mult"]
    ke = np.zeros((a["E"], n, n), np.complex128)
    be = np.zeros((a["E"], n), np.complex128)
    lib().or_element_matrices(C.byref(b), C.cast(terms_ptr, C.c_void_p), n_terms, freq, ke.ctypes.data, be.ctypes.data)
    return ke, be


def assemble(a, terms_ptr, n_terms, freq=0.0, with_rhs=True):
    """CSR values [nnz] and rhs [n_rows] as the reference's assemble builds them."""
    b = bucket(a)
    ai = np.ascontiguousarray(a["ai"], np.uint64)
    aj = np.ascontiguousarray(a["aj"], np.uint64)
    edof = np.ascontiguousarray(a["edof"], np.uint64)
    etype = np.ascontiguousarray(a["etype"], np.int32)
    dirichlet = np.ascontiguousarray(a["dirichlet"], np.complex128)
    values = np.zeros(int(ai[-1]), np.complex128)
    rhs = np.zeros(int(a["n_rows"]), np.complex128) if with_rhs else None
    err = lib().or_assemble(C.byref(b), C.cast(terms_ptr, C.c_void_p), n_terms, freq, ai.ctypes.data, aj.ctypes.data,
                            edof.ctypes.data, etype.ctypes.data, dirichlet.ctypes.data if dirichlet.size else None,
                            values.ctypes.data, rhs.ctypes.data if with_rhs else None)
    if err == 2:
        raise ValueError("oracle: an integration point lies outside a Jacobian modificator's shell")
    if err:
        raise RuntimeError("oracle: an element DOF pair is missing from the pattern")
    return values, rhs


def assemble_coupled(at, au, terms_ptr, n_terms, freq=0.0, with_rhs=True, values=None, rhs=None):
    """Adds the block of two-field terms (test field: arrays at, the rows;
    unknown field: au, the columns; femg.Problem.field_arrays) into CSR
    values [nnz] and rhs [n_rows] (zeros when not given), as the reference's
    assemble does; returns them."""
    bt, bu = bucket(at), bucket(au)
    ai = np.ascontiguousarray(at["ai"], np.uint64)
    aj = np.ascontiguousarray(at["aj"], np.uint64)
    et = np.ascontiguousarray(at["edof"], np.uint64)
    tt = np.ascontiguousarray(at["etype"], np.int32)
    eu = np.ascontiguousarray(au["edof"], np.uint64)
    tu = np.ascontiguousarray(au["etype"], np.int32)
    dirichlet = np.ascontiguousarray(at["dirichlet"], np.complex128)
    if values is None:
        values = np.zeros(int(ai[-1]), np.complex128)
    if rhs is None and with_rhs:
        rhs = np.zeros(int(at["n_rows"]), np.complex128)
    err = lib().or_assemble_coupled(C.byref(bt), C.byref(bu), C.cast(terms_ptr, C.c_void_p), n_terms, freq, ai.ctypes.data,
                                    aj.ctypes.data, et.ctypes.data, tt.ctypes.data, eu.ctypes.data, tu.ctypes.data,
                                    dirichlet.ctypes.data if dirichlet.size else None, values.ctypes.data,
                                    rhs.ctypes.data if with_rhs else None)
    if err == 4:
        raise ValueError("oracle: lifting through a block of different test and unknown DOF counts has no defined value")
    if err == 5:
        raise ValueError("oracle: linked DOFs in two-field terms are not restated")
    if err == 6:
        raise ValueError("oracle: two-field terms of scalar H1 fields only")
    if err == 2:
        raise ValueError("oracle: an integration point lies outside a Jacobian modificator's shell")
    if err:
        raise RuntimeError("oracle: an element DOF pair is missing from the pattern")
    return values, rhs


def assemble_blocks(prob, freq=0.0, with_rhs=True):
    """The whole system of a multi-field femg.Problem: every block's terms
    into one CSR value array and right-hand side."""
    values = np.zeros(prob.nnz, np.complex128)
    rhs = np.zeros(int(prob.sys.n_rows), np.complex128) if with_rhs else None
    for test, unknown, tp, nt in prob.blocks():
        at = prob.field_arrays(test)
        if test == unknown:
            v, b = assemble(at, tp, nt, freq, with_rhs)
            values += v
            if with_rhs:
                rhs += b
        else:
            assemble_coupled(at, prob.field_arrays(unknown), tp, nt, freq, with_rhs, values, rhs)
    return values, rhs


def pattern(edof, etype, n_rows, upper=False, linked_row=None):
    edof = np.ascontiguousarray(edof, np.uint64)
    etype = np.ascontiguousarray(etype, np.int32)
    E, n = edof.shape
    ai = np.zeros(int(n_rows) + 1, np.uint64)
    ajp = C.c_void_p()
    lrow = None if linked_row is None else np.ascontiguousarray(linked_row, np.uint64)
    st = lib().or_pattern(E, n, edof.ctypes.data, etype.ctypes.data, int(n_rows), ai.ctypes.data, C.byref(ajp), 1 if upper else 0,
                          lrow.ctypes.data if lrow is not None and lrow.size else None)
    if st:
        raise ValueError("oracle: linked DOFs without their master rows (linked_row)")
    nnz = int(ai[-1])
    aj = np.ctypeslib.as_array(C.cast(ajp, C.POINTER(C.c_uint64)), shape=(max(nnz, 1),))[:nnz].copy()
    lib().or_free(ajp)
    return ai, aj


def reorder_hilbert(dim, bbox, xyz, atype, n_unknown, n_bubble):
    xyz = np.ascontiguousarray(xyz, np.float32)
    atype = np.ascontiguousarray(atype, np.int32)
    bbox = np.ascontiguousarray(bbox, np.float64)
    out = np.zeros(len(atype), np.uint64)
    lib().or_reorder_hilbert(dim, bbox.ctypes.data, len(atype), xyz.ctypes.data, atype.ctypes.data, n_unknown, n_bubble,
                             out.ctypes.data)
    return out


def hilbert_keys(dim, pts, mn, mx):
    pts = np.ascontiguousarray(pts, np.float32)
    mn = np.ascontiguousarray(mn, np.float32)
    mx = np.ascontiguousarray(mx, np.float32)
    keys = np.zeros(len(pts), np.uint64)
    lib().or_hilbert_keys(dim, len(pts), pts.ctypes.data, mn.ctypes.data, mx.ctypes.data, keys.ctypes.data)
    return keys


def hilbert_order(dim, pts, mn, mx):
    keys = hilbert_keys(dim, pts, mn, mx)
    perm = np.zeros(len(keys), np.uint32)
    lib().or_hilbert_sort(len(keys), keys.ctypes.data, perm.ctypes.data)
    return perm


def robin_script(n_created, reserve_at, reserve_arg):
    """reserve/insert event script: reserve k happens before DOF reserve_at[k]"""
    kinds, args = [], []
    r = 0
    for i in range(n_created):
        while r < len(reserve_at) and reserve_at[r] == i:
            kinds.append(0)
            args.append(int(reserve_arg[r]))
            r += 1
        kinds.append(1)
        args.append(i)
    while r < len(reserve_at):
        kinds.append(0)
        args.append(int(reserve_arg[r]))
        r += 1
    return np.array(kinds, np.int32), np.array(args, np.uint64)


def robin_order(kinds, args, num_type, entity, use_ref=False):
    L = ref() if use_ref else lib()
    fn = L.ref_robin_order if use_ref else L.or_robin_order
    num_type = np.ascontiguousarray(num_type, np.uint64)
    entity = np.ascontiguousarray(entity, np.uint64)
    out = np.zeros(len(num_type), np.uint32)
    cnt = fn(len(kinds), kinds.ctypes.data, args.ctypes.data, num_type.ctypes.data, entity.ctypes.data, out.ctypes.data)
    return out[:cnt]


def ref_hilbert_order(dim, pts, mn, mx):
    R = ref()
    pts = np.ascontiguousarray(pts, np.float32)
    mn = np.ascontiguousarray(mn, np.float32)
    mx = np.ascontiguousarray(mx, np.float32)
    perm = np.zeros(len(pts), np.uint32)
    R.ref_hilbert_order(dim, len(pts), pts.ctypes.data, mn.ctypes.data, mx.ctypes.data, perm.ctypes.data)
    return perm
