"""Symmetric / hermitian (upper-triangle) storage: the formulation option
under which MatrixFactory::addPattern and addValues drop the entries with
column < row (src/system/MatrixFactory.cpp:491 and :265). The host pre()
pattern against the oracle's restatement, bit for bit, including aliased
bubble rows (which keep the first bubble's columns), and the upper values
against full storage."""
import numpy as np
import pytest

CFGS = {
    "tri_p2_dirichlet": dict(dim=2, m=6, mesh_order=2, space=0, gauss=4, dirichlet=1, source=1),
    "tri_h1_p4_bubbles": dict(dim=2, m=4, mesh_order=1, space=1, order=4, gauss=8),
    "tet_h1_p3": dict(dim=3, m=3, mesh_order=1, space=1, order=3, gauss=6),
    "tet_h1_p4_bubbles": dict(dim=3, m=2, mesh_order=1, space=1, order=4, gauss=8),
}


def problems(femg, name):
    c = CFGS[name]
    return femg.Problem(femg.config(**c)), femg.Problem(femg.config(upper=1, **c))


@pytest.mark.parametrize("name", list(CFGS))
def test_host_upper_pattern_matches_oracle(femg, oracle, name):
    full, up = problems(femg, name)
    a, b = full.arrays(), up.arrays()
    assert b["upper"] == 1 and a["upper"] == 0
    assert np.array_equal(a["edof"], b["edof"])  # same numbering
    ai, aj = oracle.pattern(b["edof"], b["etype"], b["n_rows"], upper=True)
    assert np.array_equal(ai, b["ai"]) and np.array_equal(aj, b["aj"])
    # rows that own their pattern keep exactly the full row's columns >= row
    fai, faj = a["ai"].astype(np.int64), a["aj"]
    uai, uaj = b["ai"].astype(np.int64), b["aj"]
    bubble = set(b["edof"][b["etype"] == 3].tolist())  # rows that may alias another bubble's row
    checked = 0
    for r in range(0, int(a["n_rows"]), max(1, int(a["n_rows"]) // 200)):
        if r in bubble:
            continue
        fr = faj[fai[r]:fai[r + 1]]
        ur = uaj[uai[r]:uai[r + 1]]
        assert np.array_equal(ur, fr[fr >= r])
        checked += 1
    assert checked > 0


@pytest.mark.parametrize("name", ["tri_p2_dirichlet", "tet_h1_p3"])
def test_upper_values_are_the_full_upper_triangle(femg, oracle, name):
    full, up = problems(femg, name)
    a, b = full.arrays(), up.arrays()
    t, nt = full.terms()
    vf, bf = oracle.assemble(a, t, nt)
    vu, bu = oracle.assemble(b, t, nt)
    fai = a["ai"].astype(np.int64)
    rows_f = np.repeat(np.arange(len(fai) - 1), np.diff(fai))
    keep = a["aj"].astype(np.int64) >= rows_f
    uai = b["ai"].astype(np.int64)
    rows_u = np.repeat(np.arange(len(uai) - 1), np.diff(uai))
    # no aliased bubbles here: the upper pattern is the full pattern's upper part
    assert np.array_equal(b["aj"], a["aj"][keep]) and np.array_equal(rows_u, rows_f[keep])
    assert np.allclose(vu, vf[keep], rtol=0, atol=1e-13 * np.abs(vf).max())
    # the right-hand side (sources, Dirichlet lifting) does not depend on the storage
    assert np.allclose(bu, bf, rtol=0, atol=1e-13 * max(np.abs(bf).max(), 1.0))


def test_upper_aliased_bubble_rows_follow_the_reference_lookup(femg, oracle):
    """Order-4 triangles: some aliased bubble rows have a first bubble with a
    larger index, so their row lacks the columns in between; the reference
    adds those entries at the lower_bound position without checking it, and
    the oracle does the same instead of failing."""
    _, up = problems(femg, "tri_h1_p4_bubbles")
    b = up.arrays()
    ai, aj = b["ai"].astype(np.int64), b["aj"].astype(np.int64)
    edof, etype = b["edof"].astype(np.int64), b["etype"]
    short = 0
    for e in range(len(edof)):
        bub = edof[e][etype[e] == 3]
        for r in bub[1:]:  # aliased rows
            if r < bub[0]:
                short += 1
                assert aj[ai[r]] == bub[0] or aj[ai[r]] > r
    assert short > 0
    t, nt = up.terms()
    v, _ = oracle.assemble(b, t, nt)
    assert np.all(np.isfinite(v))
