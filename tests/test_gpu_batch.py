"""fg_batch: many problems of different mesh size, order, rule and wavenumber
in one graph-captured sequence of batched launches. Every problem's CSR
against the single-plan FP64 path (1e-12) and the oracle (mixed: 1e-6); the
graph replay against the first (tuning) run; device outputs; refusals."""
import ctypes as C
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def small_batch(femg):
    """Seven problems: orders 1-4, m 2-4, complex per-element coefficient and a
    source term in two of them."""
    cfgs = femg.config_c4(n=5, seed=11, m_lo=2, m_hi=4)
    cfgs[0].order, cfgs[0].gauss = 4, 8
    c = femg.config_c3(m=3)
    cfgs.append(c)
    s = femg.config(dim=3, m=3, mesh_order=1, space=femg.FG_SPACE_HIERARCHICAL_H1, order=2, gauss=4, jitter=0.15,
                    seed=5, k=12.0, source=1)
    cfgs.append(s)
    return [femg.Problem(c) for c in cfgs]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_and_oracle(femg, oracle, cuda, precision):
    probs = small_batch(femg)
    plans = [p.plan() for p in probs]
    batch = femg.Batch(plans, mixed=precision == "mixed")
    rhs = [np.zeros(int(p.sys.n_rows), np.complex128) for p in probs]
    vals, rhs = batch.run(rhs=rhs)
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    for p, pl, v, b in zip(probs, plans, vals, rhs):
        a = p.arrays()
        t, nt = p.terms()
        ref_v, ref_b = oracle.assemble(a, t, nt)
        assert rel(v, ref_v) <= tol
        if np.linalg.norm(ref_b) > 0:
            assert rel(b, ref_b) <= FP64_TOL  # element right-hand sides stay FP64
        if precision == "fp64":
            v1, b1 = pl.assemble("fp64")
            assert rel(v, v1) <= FP64_TOL
    # second run: the captured graph, same values bit for bit
    vals2, rhs2 = batch.run(rhs=[np.zeros_like(r) for r in rhs])
    for v, v2, b, b2 in zip(vals, vals2, rhs, rhs2):
        assert np.array_equal(v.view(np.uint64), v2.view(np.uint64))
        assert np.array_equal(b.view(np.uint64), b2.view(np.uint64))
    tun = json.loads(batch.tuning())
    assert len(tun["gather"]) >= 4
    if precision == "mixed":
        assert all(c["mma_n"] in (16, 32, 48, 64, 112, 128, 208, 256) or c["mma_n"] % 16 == 0 for c in tun["contract"])


def test_batch_device_outputs(femg, cuda):
    torch = cuda
    probs = small_batch(femg)[:4]
    plans = [p.plan() for p in probs]
    batch = femg.Batch(plans, mixed=True)
    host, _ = batch.run()
    dv = [torch.zeros(2 * p.nnz, dtype=torch.float64, device="cuda") for p in probs]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        batch.run(values=[d.data_ptr() for d in dv], stream=stream)
        torch.cuda.synchronize()
        for h, d in zip(host, dv):
            assert np.array_equal(d.cpu().numpy().view(np.uint64), h.view(np.uint64))


def test_batch_bound_terms(femg, cuda):
    probs = small_batch(femg)[:3]
    plans = [p.plan() for p in probs]
    for pl in plans:
        pl.bind_terms()
    batch = femg.Batch(plans, mixed=False, bound=True)
    vals, _ = batch.run()
    for pl, v in zip(plans, vals):
        v1, _ = pl.assemble("fp64")
        assert rel(v, v1) <= FP64_TOL


def test_batch_rejects(femg, cuda):
    L = femg.lib()
    prob = femg.Problem(femg.config_c1(m=4))  # Dirichlet DOFs
    plan = prob.plan()
    ptrs = (C.c_void_p * 1)(plan.ptr.value)
    tl = (C.c_void_p * 1)(C.cast(prob.terms()[0], C.c_void_p).value)
    nl = (C.c_int32 * 1)(prob.terms()[1])
    out = C.c_void_p()
    assert L.fg_batch_create(ptrs, tl, nl, 1, 0, C.byref(out)) == femg.FG_ERR_UNSUPPORTED
    assert not out
    assert L.fg_batch_create(ptrs, tl, nl, 0, 0, C.byref(out)) == femg.FG_ERR_ARG
    prob2 = femg.Problem(femg.config_c2(m=2))
    plan2 = prob2.plan()
    ptrs2 = (C.c_void_p * 1)(plan2.ptr.value)
    assert L.fg_batch_create(ptrs2, None, None, 1, 0, C.byref(out)) == femg.FG_ERR_ARG  # nothing bound
