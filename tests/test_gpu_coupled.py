"""Two-field terms on the GPU: every block of a two-field formulation through
its own plan (fg_plan_create for a field with itself, fg_plan_create_coupled
for a test field with another unknown field), accumulated into one device
CSR and right-hand side, against the oracle's block-by-block assembly (which
test_coupled.py pins to the reference's own assembly) at the FP64 tolerance.
Also the refusals: the mixed path and batches on two-field plans, and the
lifting whose reference read leaves the element matrix."""

import numpy as np
import pytest

from coupled_cases import coupled_configs, lifting_undefined_config

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def assemble_blocks_gpu(femg, torch, prob, with_rhs=True, static=False):
    """All blocks into zeroed device outputs (the plans accumulate)."""
    dv = torch.zeros(2 * prob.nnz, dtype=torch.float64, device="cuda")
    db = torch.zeros(2 * int(prob.sys.n_rows), dtype=torch.float64, device="cuda") if with_rhs else None
    plans = []
    for test, unknown, tp, nt in prob.blocks():
        pl = prob.block_plan(test, unknown)
        plans.append(pl)
        if static:
            assert femg.lib().fg_plan_bind_terms(pl.ptr, tp, nt, 0.0) == femg.FG_OK, femg.lib().fg_last_error()
            dd = None
            if prob.sys.n_fixed:
                dd = torch.from_numpy(np.ascontiguousarray(prob.arrays()["dirichlet"]).view(np.float64).copy()).cuda()
            st = femg.lib().fg_assemble_fp64_static(pl.ptr, dd.data_ptr() if dd is not None else None, dv.data_ptr(),
                                                    db.data_ptr() if db is not None else None, None)
            assert st == femg.FG_OK, femg.lib().fg_last_error()
        else:
            pl.assemble("fp64", values=dv.data_ptr(), rhs=db.data_ptr() if db is not None else False, terms=(tp, nt))
    torch.cuda.synchronize()
    v = dv.cpu().numpy().view(np.complex128).copy()
    b = db.cpu().numpy().view(np.complex128).copy() if db is not None else None
    for pl in plans:
        pl.close()
    return v, b


@pytest.mark.parametrize("name", ["tri_lagrange_p2_dirichlet", "tri_h1_p3_p2", "tet_h1_p2_p1", "tet_h1_p1_p3"])
def test_coupled_blocks_match_oracle(femg, oracle, cuda, name):
    prob = femg.Problem(coupled_configs(femg)[name])
    ref_v, ref_b = oracle.assemble_blocks(prob)
    v, b = assemble_blocks_gpu(femg, cuda, prob)
    assert rel(v, ref_v) <= FP64_TOL, rel(v, ref_v)
    if np.linalg.norm(ref_b) > 0:
        assert rel(b, ref_b) <= FP64_TOL, rel(b, ref_b)
    else:
        assert np.all(b == 0)
    # the coupling blocks alone (rows of one field, columns of the other)
    for test, unknown, tp, nt in prob.blocks():
        if test == unknown:
            continue
        at, au = prob.field_arrays(test), prob.field_arrays(unknown)
        ov, _ = oracle.assemble_coupled(at, au, tp, nt, with_rhs=False)
        pl = prob.block_plan(test, unknown)
        dv = cuda.zeros(2 * prob.nnz, dtype=cuda.float64, device="cuda")
        pl.assemble("fp64", values=dv.data_ptr(), rhs=False, terms=(tp, nt))
        cuda.cuda.synchronize()
        gv = dv.cpu().numpy().view(np.complex128)
        assert np.linalg.norm(ov) > 0
        assert rel(gv, ov) <= FP64_TOL, (test, unknown, rel(gv, ov))
        pl.close()


def test_coupled_larger_mesh(femg, oracle, cuda):
    cfg = coupled_configs(femg)["tet_h1_p1_p3"]
    cfg.m = 10
    prob = femg.Problem(cfg)
    ref_v, ref_b = oracle.assemble_blocks(prob)
    v, b = assemble_blocks_gpu(femg, cuda, prob)
    assert rel(v, ref_v) <= FP64_TOL and rel(b, ref_b) <= FP64_TOL


def test_coupled_static_entry(femg, oracle, cuda):
    prob = femg.Problem(coupled_configs(femg)["tri_lagrange_p2_dirichlet"])
    ref_v, ref_b = oracle.assemble_blocks(prob)
    v, b = assemble_blocks_gpu(femg, cuda, prob, static=True)
    assert rel(v, ref_v) <= FP64_TOL and rel(b, ref_b) <= FP64_TOL


def test_coupled_refusals(femg, oracle, cuda):
    L = femg.lib()
    prob = femg.Problem(lifting_undefined_config(femg))
    _, _, tp, nt = [b for b in prob.blocks() if b[0] == 1 and b[1] == 0][0]
    pl = prob.block_plan(1, 0)  # v rows (6 DOFs), u columns (3 DOFs, some fixed)
    dv = cuda.zeros(2 * prob.nnz, dtype=cuda.float64, device="cuda")
    db = cuda.zeros(2 * int(prob.sys.n_rows), dtype=cuda.float64, device="cuda")
    with pytest.raises(femg.FgError) as e:
        pl.assemble("fp64", values=dv.data_ptr(), rhs=db.data_ptr(), terms=(tp, nt))
    assert e.value.status == femg.FG_ERR_UNSUPPORTED
    assert b"addValuesDC" in L.fg_last_error()
    # the values alone: defined, and equal to the oracle's
    pl.assemble("fp64", values=dv.data_ptr(), rhs=False, terms=(tp, nt))
    cuda.cuda.synchronize()
    ov, _ = oracle.assemble_coupled(prob.field_arrays(1), prob.field_arrays(0), tp, nt, with_rhs=False)
    assert rel(dv.cpu().numpy().view(np.complex128), ov) <= FP64_TOL
    # the mixed path and batches do not take two-field plans
    with pytest.raises(femg.FgError) as e:
        pl.assemble("mixed", values=dv.data_ptr(), rhs=False, terms=(tp, nt))
    assert e.value.status == femg.FG_ERR_UNSUPPORTED
    pl.set_accumulate(False)
    with pytest.raises(femg.FgError) as e:
        femg.Batch([pl], mixed=False, bound=True)
    assert e.value.status == femg.FG_ERR_UNSUPPORTED
    # source terms belong to the test field's own plan
    src = (femg.TermDesc * 1)()
    src[0].kind = femg.FG_TERM_SOURCE
    st = L.fg_assemble_fp64(pl.ptr, src, 1, 0.0, None, dv.data_ptr(), None, None)
    assert st == femg.FG_ERR_UNSUPPORTED
    pl.close()
