"""Linked bubble DOFs: the interior DOFs of an element linked to those of
another element, which DofsFactory::_generateLinkedDofs makes when the
periodic slave entity has the mesh's dimension (src/dofs/DofsFactory.cpp:
559-583, LinkedBubbleDof). MatrixFactory::addValues and VectorFactory add
them as linked DOFs: into the master's row times conj(c), the master's column
times c (src/system/MatrixFactory.cpp:306-309, :373-380, :409-442;
src/system/VectorFactory.cpp:134, :195). addPattern takes them as bubble rows
(:505-535): the first bubble row of an element takes the element's columns
into the list its row points at and the later ones are pointed at that list,
so the bubble rows of a master element and of its linked element share one
list holding both elements' columns.

The systems here link the interior DOFs of every element right of x = 0.5 to
those of the element 0.5 to its left, local DOF to local DOF, with e^(i phi).
The oracle is pinned by the identity the linking implies, A_linked = P^H A P
and b_linked = P^H b with A and b the oracle's assembly without links (full
storage), the pattern by the structure of P^T S P, and with symmetric
storage by a restatement of addPattern's pointer assignments run over the
elements in two orders."""
import numpy as np
import pytest
import scipy.sparse as sp

AT_UNKNOWN, AT_BUBBLE, AT_FIXED, AT_LINKED_BUBBLE = 2, 3, 1, 6

CFGS = {
    # three interior DOFs per triangle: the aliasing of an element's later bubble rows matters
    "tri_h1_p4": dict(dim=2, m=6, mesh_order=1, space=1, order=4, gauss=8, jitter=0.0, seed=1, k=2.0, source=1),
    # one interior DOF per triangle
    "tri_h1_p3": dict(dim=2, m=6, mesh_order=1, space=1, order=3, gauss=6, jitter=0.0, seed=3, k=2.0, source=1),
}


def volume_periodic(femg, prob, phi):
    """(b, P): prob's arrays with the interior DOFs of the elements right of
    x = 0.5 linked to those of their partners 0.5 to the left, and P."""
    a = prob.arrays()
    n_rows = int(a["n_rows"])
    xyz, en = a["xyz"], a["enodes"]
    cen = xyz[en].mean(axis=1)
    key = {(round(c[0], 9), round(c[1], 9)): e for e, c in enumerate(cen)}
    edof, etype = a["edof"].astype(np.int64), a["etype"]
    slave_of = {}  # full row -> master full row
    for e, c in enumerate(cen):
        if c[0] <= 0.5:
            continue
        m = key[(round(c[0] - 0.5, 9), round(c[1], 9))]
        bs, bm = np.flatnonzero(etype[e] == AT_BUBBLE), np.flatnonzero(etype[m] == AT_BUBBLE)
        assert len(bs) == len(bm) > 0
        for i, j in zip(bs, bm):
            slave_of[int(edof[e, i])] = int(edof[m, j])
    slaves = np.array(sorted(slave_of), np.int64)
    keep = np.ones(n_rows, bool)
    keep[slaves] = False
    red = np.full(n_rows, -1, np.int64)
    red[keep] = np.arange(int(keep.sum()))
    lidx = {int(s): k for k, s in enumerate(slaves)}
    coef = np.exp(1j * phi)
    e2, t2 = edof.copy(), etype.copy()
    for (e, i), t in np.ndenumerate(etype):
        if t in (AT_UNKNOWN, AT_BUBBLE):
            r = int(edof[e, i])
            if r in lidx:
                t2[e, i] = AT_LINKED_BUBBLE
                e2[e, i] = lidx[r]
            else:
                e2[e, i] = red[r]
    b = dict(a)
    b.update(edof=e2.astype(np.uint64), etype=t2, n_rows=int(keep.sum()),
             linked_row=np.array([red[slave_of[int(s)]] for s in slaves], np.uint64),
             linked_value=np.full(len(slaves), coef, np.complex128))
    P = sp.lil_matrix((n_rows, int(keep.sum())), dtype=np.complex128)
    for r in range(n_rows):
        P[r, red[r] if keep[r] else red[slave_of[r]]] = 1.0 if keep[r] else coef
    return b, P.tocsr()


def csr(ai, aj, v, n):
    return sp.csr_matrix((v, aj.astype(np.int64), ai.astype(np.int64)), shape=(n, n))


def linked_bubble_system(femg, oracle, name, phi, upper=False):
    prob = femg.Problem(femg.config(**CFGS[name]))
    b, P = volume_periodic(femg, prob, phi)
    ai, aj = oracle.pattern(b["edof"], b["etype"], b["n_rows"], upper=upper, linked_row=b["linked_row"])
    b.update(ai=ai, aj=aj, upper=int(upper))
    return prob, b, P


def reference_pattern(edof, etype, n_rows, linked_row, upper, order):
    """addPattern (MatrixFactory.cpp:459-539) and finalizePattern (:188-213)
    restated with the reference's array of list pointers, over the elements
    in the given order."""
    lists = [[] for _ in range(n_rows)]
    ptr = list(range(n_rows))

    def rc(t, v):
        if t in (AT_UNKNOWN, AT_BUBBLE, 4):
            return int(v)
        if t in (5, AT_LINKED_BUBBLE):
            return int(linked_row[v])
        return None

    for e in order:
        bubble = None
        for i in range(edof.shape[1]):
            I = rc(etype[e, i], edof[e, i])
            if I is None:
                continue
            if etype[e, i] in (AT_BUBBLE, AT_LINKED_BUBBLE):
                if bubble is not None:
                    ptr[I] = bubble
                    continue
                bubble = ptr[I]
            dst = lists[ptr[I]]
            for j in range(edof.shape[1]):
                J = rc(etype[e, j], edof[e, j])
                if J is None or (upper and J < I):
                    continue
                if J not in dst:
                    dst.append(J)
    rows = [sorted(lists[ptr[r]]) for r in range(n_rows)]
    ai = np.zeros(n_rows + 1, np.uint64)
    ai[1:] = np.cumsum([len(r) for r in rows])
    return ai, np.array([c for r in rows for c in r], np.uint64)


@pytest.mark.parametrize("name", list(CFGS))
def test_linked_bubble_pattern_is_the_reduced_structure(femg, oracle, name):
    prob, b, P = linked_bubble_system(femg, oracle, name, 0.7)
    a = prob.arrays()
    assert (b["etype"] == AT_LINKED_BUBBLE).sum() > 0
    n = int(a["n_rows"])
    S = csr(a["ai"], a["aj"], np.ones(len(a["aj"])), n)
    Pb = (abs(P) > 0).astype(np.float64)
    R = (Pb.T @ S @ Pb).tocsr()
    R.sort_indices()
    assert np.array_equal(R.indptr.astype(np.uint64), b["ai"]) and np.array_equal(R.indices.astype(np.uint64), b["aj"])


@pytest.mark.parametrize("name", list(CFGS))
@pytest.mark.parametrize("phi", [0.0, 0.7])
def test_linked_bubble_values_are_the_reduced_system(femg, oracle, name, phi):
    prob, b, P = linked_bubble_system(femg, oracle, name, phi)
    a = prob.arrays()
    t, nt = prob.terms()
    vf, bf = oracle.assemble(a, t, nt)
    vl, bl = oracle.assemble(b, t, nt)
    n, nr = int(a["n_rows"]), int(b["n_rows"])
    Ar = (P.conj().T @ csr(a["ai"], a["aj"], vf, n) @ P).tocsr()
    Al = csr(b["ai"], b["aj"], vl, nr)
    assert abs(Al - Ar).max() <= 1e-13 * np.abs(vf).max()
    assert np.abs(bl - P.conj().T @ bf).max() <= 1e-13 * max(np.abs(bf).max(), 1.0)


@pytest.mark.parametrize("name", ["tri_h1_p4", "tri_h1_p3"])
@pytest.mark.parametrize("upper", [False, True])
def test_linked_bubble_pattern_follows_the_pointer_assignments(femg, oracle, name, upper):
    _, b, _ = linked_bubble_system(femg, oracle, name, 0.7, upper=upper)
    E = b["edof"].shape[0]
    for order in (range(E), range(E - 1, -1, -1)):
        ai, aj = reference_pattern(b["edof"], b["etype"], int(b["n_rows"]), b["linked_row"], upper, order)
        assert np.array_equal(ai, b["ai"]) and np.array_equal(aj, b["aj"])


def test_linked_bubble_with_upper_storage(femg, oracle):
    """Symmetric storage: a row that is no bubble row keeps the columns J >= I
    and their values are the full system's. A bubble row shares its list,
    whose columns start at the row of the first bubble of each element that
    filled it; an entry J >= I missing from it is added at the next column of
    the row, unchecked, as the reference's lower_bound does
    (MatrixFactory.cpp:267-268), so those rows are left to the GPU-against-
    oracle comparison."""
    prob, b, _ = linked_bubble_system(femg, oracle, "tri_h1_p4", 0.0)
    _, bu, _ = linked_bubble_system(femg, oracle, "tri_h1_p4", 0.0, upper=True)
    t, nt = prob.terms()
    vl, _ = oracle.assemble(b, t, nt)
    vu, _ = oracle.assemble(bu, t, nt)
    nr = int(b["n_rows"])
    lr = b["linked_row"].astype(np.int64)
    bubble_rows = set(int(b["edof"][e, i]) for e, i in zip(*np.nonzero(b["etype"] == AT_BUBBLE)))
    bubble_rows |= set(int(lr[v]) for v in b["edof"][b["etype"] == AT_LINKED_BUBBLE].astype(np.int64))
    full = csr(b["ai"], b["aj"], vl, nr).tolil()
    rows = np.repeat(np.arange(nr), np.diff(bu["ai"].astype(np.int64)))
    cols = bu["aj"].astype(np.int64)
    plain = np.array([r not in bubble_rows for r in rows])
    assert plain.sum() > 0 and (~plain).sum() > 0
    assert np.all(cols[plain] >= rows[plain])
    ref = np.array([full[r, c] for r, c in zip(rows[plain], cols[plain])])
    assert np.allclose(vu[plain], ref, rtol=0, atol=1e-13 * np.abs(vl).max())
