"""Element DOFs of type UnknownGlobal: the lumped unknown of a global quantity,
which every DOF of a field on the quantity's domain becomes
(DofsFactory::_generateUnknownGlobalDofs, src/dofs/DofsFactory.cpp:465-527).
MatrixFactory::addPattern and addValues take them as rows and columns like
Unknown DOFs (src/system/MatrixFactory.cpp:240-251, :466-481), so several
local DOFs of one element can land on one row and one column. The host
mirror builds no global quantities; these tests make one by merging the
boundary DOFs of a problem into a single row.

On the CPU, the oracle's merged system is pinned without its global-DOF code:
with P the 0/1 map from the original rows to the merged ones, the merged
matrix is P^T A P and the merged right-hand side P^T b, with A and b the
oracle's assembly of the original problem, and the merged pattern is the
structure of P^T S P."""
import numpy as np
import pytest

AT_UNKNOWN_GLOBAL = 4


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


CFGS = {
    "tri_p2": dict(dim=2, m=6, mesh_order=2, space=0, gauss=4, jitter=0.2, seed=3, k=4.0, source=1),
    "tri_h1_p3": dict(dim=2, m=5, mesh_order=1, space=1, order=3, gauss=6, jitter=0.2, seed=4, k=3.0, source=1),
}


def merged_system(femg, oracle, name):
    """(problem, arrays of the merged system, map old row -> new row)"""
    prob = femg.Problem(femg.config(**CFGS[name]))
    a = prob.arrays()
    rd = prob.raw_dofs()
    n = int(a["n_rows"])
    # the DOFs on the boundary of the unit square merge into one global row
    x, y = rd["xyz"][:, 0].astype(np.float64), rd["xyz"][:, 1].astype(np.float64)
    unknown = (rd["assemble_type"] == femg.FG_AT_UNKNOWN)
    on = unknown & ((np.abs(x) < 1e-6) | (np.abs(x - 1) < 1e-6) | (np.abs(y) < 1e-6) | (np.abs(y - 1) < 1e-6))
    merge = np.zeros(n, bool)
    merge[(rd["num_dof"][on] - 1).astype(np.int64)] = True
    assert merge.sum() > 4
    keep = np.flatnonzero(~merge)
    newrow = np.empty(n, np.int64)
    newrow[keep] = np.arange(len(keep))
    g = len(keep)
    newrow[merge] = g
    edof = a["edof"].astype(np.int64)
    etype = a["etype"].copy()
    rows = (etype == femg.FG_AT_UNKNOWN) | (etype == femg.FG_AT_UNKNOWN_BUBBLE)
    e2 = edof.copy()
    e2[rows] = newrow[edof[rows]]
    etype[rows & merge[np.where(rows, edof, 0)]] = AT_UNKNOWN_GLOBAL
    ai, aj = oracle.pattern(e2.astype(np.uint64), etype, g + 1)
    b = dict(a, edof=e2.astype(np.uint64), etype=etype, n_rows=g + 1, ai=ai, aj=aj)
    return prob, a, b, newrow


# order-3 tetrahedra (20 DOFs per element, rows under 254 entries): the
# vector-load reduction of the mixed path takes them, five lanes per element
# row, lane l owning columns 4l .. 4l + 3
PAIR_CFG = dict(dim=3, m=3, mesh_order=1, space=1, order=3, gauss=6, jitter=0.15, seed=5, k=3.0, source=1)
# local DOF 0 (vertex 0, lane 0) and local DOF 4 (the first DOF of edge
# (0, 1), lane 1): every element around that edge holds vertex 0, so the
# merged row is no longer than the vertex's own
PAIR_LOCAL = (0, 4)


def pair_merged_system(femg, oracle, every=5):
    """DOF pairs merged into global rows: for every `every`-th element whose
    local DOFs PAIR_LOCAL are still free, those two DOFs become one row, so
    that the element has two columns (and two local rows) on one CSR row and
    one slot, held by two lanes of the vector-load reduction.
    (problem, arrays, merged arrays, map old row -> new row)"""
    prob = femg.Problem(femg.config(**PAIR_CFG))
    a = prob.arrays()
    n = int(a["n_rows"])
    edof = a["edof"].astype(np.int64)
    etype = a["etype"].copy()
    rows = (etype == femg.FG_AT_UNKNOWN) | (etype == femg.FG_AT_UNKNOWN_BUBBLE)
    target = np.arange(n)
    used = np.zeros(n, bool)
    for e in range(0, edof.shape[0], every):
        a0, a1 = PAIR_LOCAL
        if not (rows[e, a0] and rows[e, a1]):
            continue
        i, j = edof[e, a0], edof[e, a1]
        if used[i] or used[j]:
            continue
        used[i] = used[j] = True
        target[max(i, j)] = min(i, j)
    keep = np.flatnonzero(target == np.arange(n))
    newrow = np.empty(n, np.int64)
    newrow[keep] = np.arange(len(keep))
    newrow = newrow[target]
    e2 = edof.copy()
    e2[rows] = newrow[edof[rows]]
    etype[rows & used[np.where(rows, edof, 0)]] = AT_UNKNOWN_GLOBAL
    m = len(keep)
    ai, aj = oracle.pattern(e2.astype(np.uint64), etype, m)
    b = dict(a, edof=e2.astype(np.uint64), etype=etype, n_rows=m, ai=ai, aj=aj)
    return prob, a, b, newrow


def test_oracle_pairs_equal_lumped_system(femg, oracle):
    prob, a, b, newrow = pair_merged_system(femg, oracle)
    e2 = b["edof"].astype(np.int64)
    assert (e2[:, PAIR_LOCAL[0]] == e2[:, PAIR_LOCAL[1]]).sum() >= 10  # elements with two columns on one row
    assert np.diff(b["ai"].astype(np.int64)).max() < 254  # one-byte slots
    t, nt = prob.terms()
    v, r = oracle.assemble(a, t, nt)
    vm, rm = oracle.assemble(b, t, nt)
    n, m = int(a["n_rows"]), int(b["n_rows"])
    P = np.zeros((n, m))
    P[np.arange(n), newrow] = 1.0
    assert rel(csr_dense(b["ai"], b["aj"], vm, m), P.T @ csr_dense(a["ai"], a["aj"], v, n) @ P) <= 1e-13
    assert rel(rm, P.T @ r) <= 1e-13


def csr_dense(ai, aj, v, n):
    A = np.zeros((n, n), np.complex128)
    r = np.repeat(np.arange(n), np.diff(ai.astype(np.int64)))
    np.add.at(A, (r, aj.astype(np.int64)), v)
    return A


@pytest.mark.parametrize("name", list(CFGS))
def test_oracle_global_rows_equal_lumped_system(femg, oracle, name):
    prob, a, b, newrow = merged_system(femg, oracle, name)
    t, nt = prob.terms()
    v, r = oracle.assemble(a, t, nt)
    vm, rm = oracle.assemble(b, t, nt)
    n, m = int(a["n_rows"]), int(b["n_rows"])
    P = np.zeros((n, m))
    P[np.arange(n), newrow] = 1.0
    A = csr_dense(a["ai"], a["aj"], v, n)
    Am = csr_dense(b["ai"], b["aj"], vm, m)
    want = P.T @ A @ P
    assert rel(Am, want) <= 1e-13
    assert rel(rm, P.T @ r) <= 1e-13
    S = (csr_dense(a["ai"], a["aj"], np.ones(len(v)), n) != 0).astype(np.float64)
    nz = (P.T @ S @ P) != 0
    assert np.array_equal(nz, csr_dense(b["ai"], b["aj"], np.ones(len(vm)), m) != 0)
    assert len(vm) == int(nz.sum())
