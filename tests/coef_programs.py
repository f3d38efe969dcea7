"""Coefficient programs of the operator tests (shared by the CPU tests
against the reference and the GPU tests against the oracle): every scalar
operator of the coefficient language applied to a complex, point-dependent
argument that stays away from the branch cuts,
    a(x, y) = 0.4 + 0.3 x + 0.2 y + 0.1 i (x - y),
as the mass coefficient m = op(a) and the source f = op(a) / 2 of
    integral(grad(dof u), grad(tf u)) + integral(m dof(u), tf(u)) + integral(f, tf(u))."""
import ctypes as C


def argument(F):
    return [(F.FG_OP_CONST, 0, 0.4, 0.0), (F.FG_OP_X, 0, 0, 0), (F.FG_OP_CONST, 0, 0.3, 0.0), (F.FG_OP_MUL, 0, 0, 0),
            (F.FG_OP_ADD, 0, 0, 0), (F.FG_OP_Y, 0, 0, 0), (F.FG_OP_CONST, 0, 0.2, 0.0), (F.FG_OP_MUL, 0, 0, 0),
            (F.FG_OP_ADD, 0, 0, 0), (F.FG_OP_X, 0, 0, 0), (F.FG_OP_Y, 0, 0, 0), (F.FG_OP_SUB, 0, 0, 0),
            (F.FG_OP_CONST, 0, 0.0, 0.1), (F.FG_OP_MUL, 0, 0, 0), (F.FG_OP_ADD, 0, 0, 0)]


OPS = ["SQRT", "EXP", "LN", "LOG10", "POW2", "POW5", "CBRT", "SIN", "COS", "TAN", "SINH", "COSH", "TANH", "ASIN", "ACOS",
       "ATAN", "ASINH", "ACOSH", "ATANH", "ABS", "CONJ", "REAL", "IMAG", "ATAN2", "HEAVISIDE"]


def program(F, name):
    a = argument(F)
    if name.startswith("POW"):
        return a + [(F.FG_OP_POW, int(name[3:]), 0, 0)]
    if name == "ACOSH":  # argument moved right of the cut (-inf, 1]
        return a + [(F.FG_OP_CONST, 0, 1.0, 0.0), (F.FG_OP_ADD, 0, 0, 0), (F.FG_OP_ACOSH, 0, 0, 0)]
    if name == "ATAN2":  # real arguments: atan2(Re a, 0.7 + y)
        return a + [(F.FG_OP_CONST, 0, 0.7, 0.0), (F.FG_OP_Y, 0, 0, 0), (F.FG_OP_ADD, 0, 0, 0), (F.FG_OP_ATAN2, 0, 0, 0)]
    if name == "HEAVISIDE":  # of Re(a) - 0.6: both sides of the step inside the domain
        return a + [(F.FG_OP_CONST, 0, 0.6, 0.0), (F.FG_OP_SUB, 0, 0, 0), (F.FG_OP_HEAVISIDE, 0, 0, 0)]
    return a + [(getattr(F, "FG_OP_" + name), 0, 0, 0)]


def halved(F, code):
    return code + [(F.FG_OP_CONST, 0, 0.5, 0.0), (F.FG_OP_MUL, 0, 0, 0)]


def set_expr(expr, code):
    expr.n_code = len(code)
    expr.n_arrays = 0
    for i, (op, arg, re, im) in enumerate(code):
        expr.code[i].op, expr.code[i].arg, expr.code[i].re, expr.code[i].im = op, arg, re, im


def terms(F, name):
    """(TermDesc array, count, programs for the reference program)"""
    m = program(F, name)
    f = halved(F, m)
    arr = (F.TermDesc * 3)()
    for t in arr:
        C.memset(C.byref(t), 0, C.sizeof(F.TermDesc))
    arr[0].kind = F.FG_TERM_GRAD_GRAD
    set_expr(arr[0].coef, [(F.FG_OP_CONST, 0, 1.0, 0.0)])
    arr[1].kind = F.FG_TERM_MASS
    set_expr(arr[1].coef, m)
    arr[2].kind = F.FG_TERM_SOURCE
    set_expr(arr[2].coef, f)
    programs = {"grad": [(F.FG_OP_CONST, 0, 1.0, 0.0)], "mass": m, "source": f}
    return arr, 3, programs


def configs(F):
    return {"tri_p2": F.config(dim=2, m=6, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=3),
            "tet_h1_p2": F.config(dim=3, m=2, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=2, gauss=4, jitter=0.15,
                                  seed=3)}


# ----------------------------------------------------- non-symmetric terms
# A general (not symmetric) diffusion tensor and an advection vector, point-
# dependent and partly complex:
#   D = [[1 + 0.2 x, 0.3 + 0.5 y, 0.1 y], [-0.3 + 0.1 i, 1.1, 0.2 x], [0.05 x, -0.2, 0.9 + 0.1 i y]]
# (a constant antisymmetric part would cancel in the assembled interior rows)
#   b = (0.5 + x, -0.3 y + 0.2 i, 0.1)
def _lin(F, c0, cx=0.0, cy=0.0, im=0.0):
    code = [(F.FG_OP_CONST, 0, c0, im)]
    if cx:
        code += [(F.FG_OP_X, 0, 0, 0), (F.FG_OP_CONST, 0, cx, 0.0), (F.FG_OP_MUL, 0, 0, 0), (F.FG_OP_ADD, 0, 0, 0)]
    if cy:
        code += [(F.FG_OP_Y, 0, 0, 0), (F.FG_OP_CONST, 0, cy, 0.0), (F.FG_OP_MUL, 0, 0, 0), (F.FG_OP_ADD, 0, 0, 0)]
    return code


def full_tensor(F):
    return [_lin(F, 1.0, cx=0.2), _lin(F, 0.3, cy=0.5), _lin(F, 0.0, cy=0.1),
            _lin(F, -0.3, im=0.1), _lin(F, 1.1), _lin(F, 0.0, cx=0.2),
            _lin(F, 0.0, cx=0.05), _lin(F, -0.2), [(F.FG_OP_CONST, 0, 0.9, 0.0), (F.FG_OP_Y, 0, 0, 0),
                                                  (F.FG_OP_CONST, 0, 0.0, 0.1), (F.FG_OP_MUL, 0, 0, 0),
                                                  (F.FG_OP_ADD, 0, 0, 0)]]


def advection_vector(F):
    return [_lin(F, 0.5, cx=1.0), _lin(F, 0.0, cy=-0.3, im=0.2), _lin(F, 0.1)]


def vector_dof(F):
    return [_lin(F, 0.7, cy=0.4), _lin(F, -0.2, cx=0.3, im=0.15), _lin(F, 0.35)]


def vector_source(F):
    return [_lin(F, 1.0, cy=-0.5), _lin(F, 0.2, cx=0.6), _lin(F, -0.4, im=0.3)]


def nonsym_terms(F, what):
    """(TermDesc array, count, reference programs, keep-alive list) for
    what in ("full", "advect", "both", "vdof", "vsrc", "vector"): the
    non-symmetric term(s) (general tensor diffusion, advection b . grad(u)
    tested by v, b u tested by grad(v), a vector source tested by grad(v)),
    a mass term -4 dof(u) tf(u) and a source 1 + x y."""
    keep = []
    one = [(F.FG_OP_CONST, 0, 1.0, 0.0)]
    mass = [(F.FG_OP_CONST, 0, -4.0, 0.0)]
    src = [(F.FG_OP_CONST, 0, 1.0, 0.0), (F.FG_OP_X, 0, 0, 0), (F.FG_OP_Y, 0, 0, 0), (F.FG_OP_MUL, 0, 0, 0),
           (F.FG_OP_ADD, 0, 0, 0)]
    kinds = []
    programs = {"mass": mass, "source": src}
    if what in ("full", "both"):
        D = full_tensor(F)
        kinds.append((F.FG_TERM_GRAD_GRAD_TENSOR_FULL, D))
        for k in range(9):
            programs["dfull_%d" % k] = D[k]
    if what in ("advect", "both"):
        b = advection_vector(F)
        kinds.append((F.FG_TERM_ADVECTION, b))
        for k in range(3):
            programs["adv_%d" % k] = b[k]
    if what in ("vdof", "vector"):
        b = vector_dof(F)
        kinds.append((F.FG_TERM_VECTOR_GRAD_TEST, b))
        for k in range(3):
            programs["vdof_%d" % k] = b[k]
    if what in ("vsrc", "vector"):
        f = vector_source(F)
        kinds.append((F.FG_TERM_SOURCE_GRAD, f))
        for k in range(3):
            programs["vsrc_%d" % k] = f[k]
    arr = (F.TermDesc * (len(kinds) + 2))()
    for t in arr:
        C.memset(C.byref(t), 0, C.sizeof(F.TermDesc))
    for k, (kind, progs) in enumerate(kinds):
        arr[k].kind = kind
        set_expr(arr[k].coef, one)
        ex = (F.Expr * len(progs))()
        for q, code in enumerate(progs):
            set_expr(ex[q], code)
        keep.append(ex)
        arr[k].tensor = C.cast(ex, C.POINTER(F.Expr))
    k = len(kinds)
    arr[k].kind = F.FG_TERM_MASS
    set_expr(arr[k].coef, mass)
    arr[k + 1].kind = F.FG_TERM_SOURCE
    set_expr(arr[k + 1].coef, src)
    return arr, k + 2, programs, keep


def nonsym_configs(F):
    c = {"tri_p2_dirichlet1": F.config(dim=2, m=6, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2, seed=3,
                                       dirichlet=1, dirichlet_value=1.0),
         "tri_h1_p3": F.config(dim=2, m=5, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=3, gauss=6, jitter=0.2,
                               seed=4),
         "tet_h1_p2": F.config(dim=3, m=2, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=2, gauss=4, jitter=0.15,
                               seed=3)}
    return c
