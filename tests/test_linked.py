"""Linked DOFs (periodic / Bloch conditions): the DOFs on x = 1 are linked to
those on x = 0 at the same y with the coefficient e^(i phi)
(DofsFactory::_generateLinkedDofs, src/dofs/DofsFactory.cpp:529-620). The
reference adds a linked row into its master's row scaled by
conj(coefficient) and a linked column into the master's column scaled by the
coefficient (MatrixFactory::addPattern/addValues, src/system/MatrixFactory.cpp:
459-539 and 233-448; VectorFactory::addValues/addValuesDC,
src/system/VectorFactory.cpp:122-210). The oracle's linked assembly is pinned
by the identity it implies: with P the map from the reduced DOFs to all DOFs
(1 for a kept DOF, the coefficient for a linked one), A_linked = P^H A P and
b_linked = P^H b, where A and b are the oracle's own assembly without links;
the linked pattern is the structure of P^T S P for the full structure S."""
import numpy as np
import pytest
import scipy.sparse as sp

CFGS = {
    "tri_p1": (dict(dim=2, m=6, mesh_order=1, space=0, gauss=2), 1.0, 0.0),
    "tri_p2_source": (dict(dim=2, m=5, mesh_order=2, space=0, gauss=4, source=1), 1.0, 0.0),
    # interior lines (no jitter) next to fixed boundary DOFs: linked rows with Dirichlet lifting
    "tri_p2_dirichlet": (dict(dim=2, m=8, mesh_order=2, space=0, gauss=4, jitter=0.0, dirichlet=1, dirichlet_value=1.5,
                              source=1), 0.5, 0.25),
}


def periodic(femg, prob, phi, xs=1.0, xm=0.0):
    """(b, P): the arrays of prob with the DOFs on x = xs linked to those on
    x = xm at the same y, and P."""
    a = prob.arrays()
    rd = prob.raw_dofs()
    n_rows = int(a["n_rows"])
    unk = (rd["assemble_type"] == 2) | (rd["assemble_type"] == 3)
    row = (rd["num_dof"].astype(np.int64) - 1)
    xyz = rd["xyz"]
    key = {float(xyz[d, 1]): int(row[d]) for d in np.nonzero(unk)[0] if xyz[d, 0] == np.float32(xm)}
    slave_of = {}  # full row -> master full row
    for d in np.nonzero(unk)[0]:
        if xyz[d, 0] == np.float32(xs) and float(xyz[d, 1]) in key:
            slave_of[int(row[d])] = key[float(xyz[d, 1])]
    slaves = np.array(sorted(slave_of), np.int64)
    keep = np.ones(n_rows, bool)
    keep[slaves] = False
    red = np.full(n_rows, -1, np.int64)
    red[keep] = np.arange(int(keep.sum()))
    lidx = {int(s): k for k, s in enumerate(slaves)}
    coef = np.exp(1j * phi)
    linked_row = np.array([red[slave_of[int(s)]] for s in slaves], np.uint64)
    linked_value = np.full(len(slaves), coef, np.complex128)
    edof, etype = a["edof"].astype(np.int64).copy(), a["etype"].copy()
    for (e, i), t in np.ndenumerate(etype):
        if t in (2, 3):
            r = int(edof[e, i])
            if r in lidx:
                etype[e, i] = 5  # FG_AT_LINKED
                edof[e, i] = lidx[r]
            else:
                edof[e, i] = red[r]
    b = dict(a)
    b.update(edof=edof.astype(np.uint64), etype=etype, n_rows=int(keep.sum()), linked_row=linked_row, linked_value=linked_value)
    P = sp.lil_matrix((n_rows, int(keep.sum())), dtype=np.complex128)
    for r in range(n_rows):
        if keep[r]:
            P[r, red[r]] = 1.0
        else:
            P[r, red[slave_of[r]]] = coef
    return b, P.tocsr()


def csr(ai, aj, v, n):
    return sp.csr_matrix((v, aj.astype(np.int64), ai.astype(np.int64)), shape=(n, n))


def linked_pattern(femg, oracle, name, phi):
    cfg, xs, xm = CFGS[name]
    prob = femg.Problem(femg.config(**cfg))
    b, P = periodic(femg, prob, phi, xs, xm)
    ai, aj = oracle.pattern(b["edof"], b["etype"], b["n_rows"], linked_row=b["linked_row"])
    b.update(ai=ai, aj=aj)
    return prob, b, P


@pytest.mark.parametrize("name", list(CFGS))
def test_linked_pattern_is_the_reduced_structure(femg, oracle, name):
    prob, b, P = linked_pattern(femg, oracle, name, 0.7)
    a = prob.arrays()
    assert len(b["linked_row"]) > 0
    n = int(a["n_rows"])
    S = csr(a["ai"], a["aj"], np.ones(len(a["aj"])), n)
    Pb = (abs(P) > 0).astype(np.float64)
    R = (Pb.T @ S @ Pb).tocsr()
    R.sort_indices()
    assert np.array_equal(R.indptr.astype(np.uint64), b["ai"]) and np.array_equal(R.indices.astype(np.uint64), b["aj"])


@pytest.mark.parametrize("name", list(CFGS))
@pytest.mark.parametrize("phi", [0.0, 0.7])
def test_linked_values_are_the_reduced_system(femg, oracle, name, phi):
    prob, b, P = linked_pattern(femg, oracle, name, phi)
    a = prob.arrays()
    t, nt = prob.terms()
    vf, bf = oracle.assemble(a, t, nt)
    vl, bl = oracle.assemble(b, t, nt)
    n = int(a["n_rows"])
    Ar = (P.conj().T @ csr(a["ai"], a["aj"], vf, n) @ P).tocsr()
    nr = int(b["n_rows"])
    Al = csr(b["ai"], b["aj"], vl, nr)
    scale = np.abs(vf).max()
    assert abs(Al - Ar).max() <= 1e-13 * scale
    assert np.abs(bl - P.conj().T @ bf).max() <= 1e-13 * max(np.abs(bf).max(), 1.0)


def test_linked_with_upper_storage(femg, oracle):
    """Symmetric storage on a linked system: rows and columns map to the
    masters first, then the entries left of the diagonal drop (MatrixFactory.cpp:
    265, 491); the result is the upper triangle of the linked system's values."""
    prob, b, P = linked_pattern(femg, oracle, "tri_p1", 0.0)
    t, nt = prob.terms()
    vl, _ = oracle.assemble(b, t, nt)
    bu = dict(b, upper=1)
    ai, aj = oracle.pattern(bu["edof"], bu["etype"], bu["n_rows"], upper=True, linked_row=bu["linked_row"])
    bu.update(ai=ai, aj=aj)
    vu, _ = oracle.assemble(bu, t, nt)
    rows = np.repeat(np.arange(len(b["ai"]) - 1), np.diff(b["ai"].astype(np.int64)))
    keep = b["aj"].astype(np.int64) >= rows
    assert np.array_equal(aj, b["aj"][keep])
    assert np.allclose(vu, vl[keep], rtol=0, atol=1e-13 * np.abs(vl).max())
