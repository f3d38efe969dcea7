"""The GPU paths at the full sizes of the benchmark workloads, entry by entry
against the oracle (which test_reference.py pins to the reference's own
assembly):
  * 3D Helmholtz, 384,000 order-3 tets (84,640,201 nonzeros), constant and
    per-tet coefficients: FP64 to 1e-12, mixed (fused and split) to 1e-6;
  * 3D Navier P2 x 3 components on 30^3 x 6 = 162,000 tets at 16
    frequencies in one pass: four frequencies against the oracle, all
    sixteen against K - omega^2 M from the separate K and M matrices;
  * the batch of 64 Helmholtz problems of orders 1-4 (15.2 M tets): the
    smallest problem of each order against the oracle, mixed and FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("cfg", ["c2", "c3"])
def test_full_size_helmholtz_entrywise(femg, oracle, cuda, cfg):
    prob = femg.Problem(femg.config_c2() if cfg == "c2" else femg.config_c3())
    a = prob.arrays()
    assert a["E"] == 384000 and prob.nnz == 84640201
    t, nt = prob.terms()
    ref_v, _ = oracle.assemble(a, t, nt, with_rhs=False)
    plan = prob.plan()
    v, _ = plan.assemble("fp64", rhs=False)
    assert rel(v, ref_v) <= 1e-12, rel(v, ref_v)
    assert plan.fused_info()["applies"]
    plan.set_mixed_fused(True)
    vm, _ = plan.assemble("mixed", rhs=False)
    assert rel(vm, ref_v) <= 1e-6, rel(vm, ref_v)
    plan.set_mixed_fused(False)
    vs, _ = plan.assemble("mixed", rhs=False)
    assert rel(vs, ref_v) <= 1e-6, rel(vs, ref_v)


def test_navier_16_frequencies_m30(femg, oracle, cuda):
    prob = femg.Problem(femg.config_c5(m=30, omega=0.0))
    a = prob.arrays()
    assert a["E"] == 162000
    t, nt = prob.terms()
    plan = prob.plan()
    omegas = np.random.default_rng(5).uniform(1.0, 10.0, 16)
    vals, _ = plan.assemble_multi_freq(omegas, precision="mixed", rhs=False)
    vals64, _ = plan.assemble_multi_freq(omegas, precision="fp64", rhs=False)
    K, _, M, _ = plan.assemble_separate("fp64", with_rhs=False)
    for f in (0, 5, 10, 15):
        ref_v, _ = oracle.assemble(a, t, nt, freq=float(omegas[f]), with_rhs=False)
        assert rel(vals64[f], ref_v) <= 1e-12, (f, rel(vals64[f], ref_v))
        assert rel(vals[f], ref_v) <= 1e-6, (f, rel(vals[f], ref_v))
    for f, w in enumerate(omegas):
        want = K - w * w * M
        assert rel(vals64[f], want) <= 1e-12, (f, rel(vals64[f], want))
        assert rel(vals[f], want) <= 1e-6, (f, rel(vals[f], want))


def test_batch_64_problems(femg, oracle, cuda):
    import concurrent.futures
    cfgs = femg.config_c4()
    with concurrent.futures.ThreadPoolExecutor(max_workers=4) as ex:
        probs = list(ex.map(femg.Problem, cfgs))
    assert len(probs) == 64
    plans = [p.plan() for p in probs]
    check = {}
    for q, c in enumerate(cfgs):  # the smallest problem of each order
        o = int(c.order)
        if o not in check or probs[q].E < probs[check[o]].E:
            check[o] = q
    assert sorted(check) == [1, 2, 3, 4]
    # device outputs (4.9 G nonzeros, 78 GB): only the checked problems come
    # back to the host
    torch = cuda
    dev = [torch.empty(2 * p.nnz, dtype=torch.float64, device="cuda") for p in probs]
    refs = {}
    for o, q in check.items():
        t, nt = probs[q].terms()
        refs[q] = oracle.assemble(probs[q].arrays(), t, nt, with_rhs=False)[0]
    for mixed, tol in ((True, 1e-6), (False, 1e-12)):
        b = femg.Batch(plans, mixed=mixed)
        b.run(values=[d.data_ptr() for d in dev])
        torch.cuda.synchronize()
        b.close()
        for o, q in check.items():
            v = dev[q].cpu().numpy().view(np.complex128)
            assert rel(v, refs[q]) <= tol, (mixed, o, rel(v, refs[q]))
    del dev
    torch.cuda.empty_cache()
