"""Benchmark of the GB300 assembly path (one JSON line on rank 0).

Headline workload: the 3D Helmholtz system on the unit cube, 40^3 cubes x 6
Kuhn tetrahedra = 384,000 tets, hierarchical H1 order 3 (20 DOFs per tet),
Gauss6, k = 20, per-tet coefficient -k^2 (1 + 0.3 xi), xi ~ N(0,1): 84,640,201
CSR nonzeros, 1,771,561 unknowns. Inputs are seeded synthetic data with the
reference configuration's shapes.

A step is one full assembly (every element matrix and vector, scatter into
the CSR values and right-hand side) on inputs resident in HBM. The headline
value is element matrices/s of the mixed-precision path (FP64 geometry,
3xTF32 tensor-core contraction, FP64 CSR), with the plain FP64 path beside it
and the relative Frobenius error between the two. The CSR output (1.35 GB)
is larger than L2, so no flush is needed between steps.

The default line also carries, as "c4" and "c5mf", the batched workload (64
Helmholtz problems of orders 1-4 in one graph replay) and the multi-frequency
workload (Navier P2 x 3 on 1,296,000 tets at 16 frequencies in one pass),
each with its own FP64 comparisons, clocks, roofline, CPU baseline and
end-to-end figure (--no-c4 / --no-c5 leave them out; --workload c4 or c5mf
prints one of them alone).

--impl reference times the reference's CPU implementation on the host cores
in a process that does not load the GPU library: the reference's own
Formulation::assemble where its library was built (its sources with the gmsh
stand-in; kind "reference"), else the oracle's C restatement of it, pinned to
the reference at 1e-13 (kind "port"), on a bounded sample of the elements.

Multi-GPU: every rank assembles its own replica of the workload (the path
has no exchange step); value = all ranks' element matrices / max rank time.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "element matrices/s and CSR nnz/s: mixed vs FP64 GPU at <=1e-6 rel error, 1 GB300"

# DRAM bytes (read + write) per CSR nonzero of one reduction launch on the 3D
# P3 Helmholtz meshes, from ncu captures of the 30^3 x 6 mesh (162,000 tets,
# 35,811,451 nonzeros); the per-launch traffic of other sizes of that family
# is this figure times their nonzeros. k_gather: 555.2 MB read + 550.5 MB
# written; k_gather_v4: 566.2 MB read + 548.5 MB written.
GATHER_TRAFFIC_PER_NNZ_P3 = {"k_gather": (555.207680e6 + 550.488064e6) / 35811451,
                             "k_gather_v4": (566.168064e6 + 548.542976e6) / 35811451}

# FP64-pipe activity of the plain FP64 element kernel (k_element_fp64<8, 0>,
# the quadrature loop) in an ncu capture on the 30^3 x 6 P3 mesh: the loop is
# bound by GB300's FP64 pipe
ELEMENT_FP64_PIPE_ACTIVE_P3 = 0.910


def load_femg():
    import __graft_entry__ as g
    g.build()
    return g._femg()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(femg, name, m):
    if name == "c3":
        return femg.config_c3(m=m or 40), "helmholtz3d_tet_h1p3_%d3x6_gauss6_percell_coef" % (m or 40)
    if name == "c2":
        return femg.config_c2(m=m or 40), "helmholtz3d_tet_h1p3_%d3x6_gauss6_k20" % (m or 40)
    if name == "c1":
        return femg.config_c1(m=m or 64), "helmholtz2d_tri_p2_%d2x2_gauss4_k10_dirichlet" % (m or 64)
    if name == "c5":
        return femg.config_c5(m=m or 60), "navier3d_tet_h1p2x3_%d3x6_gauss4_lame" % (m or 60)
    if name == "c3p4":  # the c3 mesh with order-4 hierarchical H1 (35 DOFs/tet), Gauss8
        c = femg.config_c3(m=m or 30, order=4)
        c.gauss = 8
        return c, "helmholtz3d_tet_h1p4_%d3x6_gauss8_percell_coef" % (m or 30)
    raise SystemExit("unknown workload " + name)


def sub_arrays(a, S):
    b = dict(a)
    for k in ("enodes", "edof", "etype", "orient"):
        b[k] = a[k][:S]
    b["E"] = S
    return b


def cpu_rate(prob, a, target_s, freq=0.0):
    """Oracle assemble on the first S elements (all host threads): element
    matrices/s. S grows until one run takes target_s seconds or covers the mesh."""
    from oracle import oracle as O
    t, nt = prob.terms()
    S = min(2000, a["E"])
    while True:
        b = sub_arrays(a, S)
        t0 = time.perf_counter()
        O.assemble(b, t, nt, freq=freq)
        dt = time.perf_counter() - t0
        if dt >= target_s or S >= a["E"]:
            return S / dt, S, dt, O.num_threads()
        S = int(min(a["E"], max(S * 2, S * target_s / max(dt, 1e-3) * 1.1)))


def timed_events(torch, stream, fn, warmup, steps):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def profile_run(femg, torch, fn):
    """{kernel: (launches, total ms)} of one call of fn with the kernel timer on."""
    torch.cuda.synchronize()
    femg.profile_read()
    femg.profile_enable(True)
    fn()
    torch.cuda.synchronize()
    femg.profile_enable(False)
    return femg.profile_read()


def roofline(prof, alg_bytes, pk, pk_kind, traffic=None, traffic_src=None, steps=1):
    """Roofline of the dominant kernel: the algorithmic bytes its launches
    carry per step over their summed device time per step. alg_bytes is the
    fused-minimum byte count of the whole step, or {kernel: bytes} where
    kernels cover different problems (the per-class reductions of a batch):
    the fused-minimum bytes of the problems that kernel's launches process."""
    dom, (dcount, dms) = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (1, 0.0))
    per_step_ms = dms / max(steps, 1)
    if isinstance(alg_bytes, dict):
        alg_bytes = alg_bytes.get(dom, 0)
    achieved = alg_bytes / (per_step_ms / 1000.0) / 1e9 if per_step_ms > 0 else 0.0
    return {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
            "traffic": traffic, "traffic_source": traffic_src, "kernel": dom,
            "kernel_launches_per_step": dcount / max(steps, 1), "kernel_ms_per_step": per_step_ms,
            "kernel_avg_ms": dms / max(dcount, 1), "algorithmic_bytes": alg_bytes, "peak_source": pk_kind,
            "kernels": {k: {"launches": v[0], "total_ms": v[1]} for k, v in prof.items()}}


def fused_bytes(E, n, nnz, nrows, nv=4, coef=16):
    """Algorithmic bytes of one assembly, the fused minimum: per element its
    vertices (3 doubles) and connectivity (4-byte indices), its coefficient
    and its n^2 element-to-nonzero map entries (4 bytes); per nonzero one
    complex double written; per row one complex double of right-hand side."""
    return E * (nv * 3 * 8 + nv * 4 + coef + n * n * 4) + nnz * 16 + nrows * 16


def build_problems(femg, cfgs, workers=4):
    """The host pre() of many problems, a few at a time (each is threaded)."""
    import concurrent.futures
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(femg.Problem, cfgs))


def bench_batch(args, femg, torch):
    """Batched workload: 64 3D Helmholtz problems, m ~ U{m_lo..m_hi}, orders
    U{1..4}, k ~ U[5, 40], Gauss(2p), one seed; one step = one fg_batch_run
    (graph replay) over all problems, outputs resident in HBM. The host
    problems (their CSR patterns: 8 bytes per nonzero, 39 GB here) are
    released before the end-to-end run allocates its host outputs (16 bytes
    per nonzero)."""
    cfgs = femg.config_c4(n=args.c4_n, m_lo=args.c4_m_lo, m_hi=args.c4_m_hi)
    w0 = time.perf_counter()
    probs = build_problems(femg, cfgs, workers=2)
    pre_wall = time.perf_counter() - w0
    pre_s = sum(p.pre_seconds() for p in probs)
    plans = [p.plan() for p in probs]
    infos = [p.info() for p in plans]
    nnzs = [p.nnz for p in probs]
    rowsq = [int(p.sys.n_rows) for p in probs]
    E = sum(i["E"] for i in infos)
    nnz = sum(nnzs)
    rows = sum(rowsq)
    algq = [fused_bytes(i["E"], i["n"], z, r, coef=0) for i, z, r in zip(infos, nnzs, rowsq)]
    alg = sum(algq)
    # CPU baseline: the oracle per order on the largest problem of that order,
    # a bounded sample each; the batch rate is the element-weighted harmonic mean
    cpu = None
    if not args.no_cpu:
        by_order = {}
        for q, p in enumerate(probs):
            o = int(p.cfg.order)
            if o not in by_order or p.E > probs[by_order[o]].E:
                by_order[o] = q
        rates, samples, cores = {}, [], 1
        for o, q in sorted(by_order.items()):
            p = probs[q]
            r, S, dt, cores = cpu_rate(p, p.arrays(), args.cpu_seconds / max(len(by_order), 1))
            rates[o] = r
            samples.append("order %d: first %d of %d elements, %.1f s" % (o, S, p.E, dt))
        t_all = sum(i["E"] / rates[int(c.order)] for i, c in zip(infos, cfgs))
        cpu = {"value": E / t_all, "unit": "element matrices/s", "cores": cores, "kind": "port",
               "sample": "; ".join(samples) + "; batch rate = all elements / sum over problems of elements / rate of its order"}
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    outs = [torch.empty(2 * z, dtype=torch.float64, device="cuda") for z in nnzs]
    ptrs = [o.data_ptr() for o in outs]
    res = {}
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    for prec in ("mixed", "fp64_factored", "fp64"):
        for p in plans:
            p.set_fp64_method(femg.FG_FP64_FACTORED if prec == "fp64_factored" else femg.FG_FP64_QUADRATURE)
        b = femg.Batch(plans, mixed=prec == "mixed")
        t0 = time.perf_counter()
        b.run(values=ptrs, stream=sptr)
        torch.cuda.synchronize()
        first_s = time.perf_counter() - t0
        l0 = femg.lib().fg_launch_count()
        steps = args.steps if prec == "mixed" else (3 if prec == "fp64_factored" else 2)
        warm = args.warmup if prec == "mixed" else 1
        ms = timed_events(torch, stream, lambda: b.run(values=ptrs, stream=sptr), warm, steps)
        launches = (femg.lib().fg_launch_count() - l0) // (warm + steps)
        res[prec] = {"ms": ms, "first_run_s": first_s, "tuning": json.loads(b.tuning()), "launches_per_step": int(launches)}
        if prec == "mixed":
            res["prof"] = profile_run(femg, torch, lambda: b.run(values=ptrs, stream=sptr))
        b.close()
        if prec == "mixed":
            # relative Frobenius error of every problem's CSR against the FP64 path
            tmp = torch.empty(2 * max(nnzs), dtype=torch.float64, device="cuda")
            d2 = r2 = 0.0
            worst = 0.0
            for p, o, z in zip(plans, outs, nnzs):
                p.assemble("fp64", values=tmp.data_ptr(), rhs=False, stream=sptr)
                torch.cuda.synchronize()
                dd = torch.linalg.vector_norm(o - tmp[:2 * z]).item() ** 2
                rr = torch.linalg.vector_norm(tmp[:2 * z]).item() ** 2
                d2 += dd
                r2 += rr
                worst = max(worst, (dd / rr) ** 0.5 if rr > 0 else 0.0)
            res["rel_fro"] = (d2 / r2) ** 0.5
            res["worst_problem_rel_fro"] = worst
            del tmp
    clk = clocks.stop()
    outs.clear()
    ptrs = None
    torch.cuda.empty_cache()
    # end to end: the batch's CSR values into host memory, as the reference's
    # module arrays hold them (ordinary pageable memory); the batch stages
    # them on the device. Its plans keep their device tables; the host
    # problems go first.
    for p in plans:
        p.set_fp64_method(femg.FG_FP64_QUADRATURE)
    be = femg.Batch(plans, mixed=True)
    for p in probs:
        p.close()
    hv = [np.empty(z, np.complex128) for z in nnzs]
    hptrs = [h.ctypes.data for h in hv]
    be.run(values=hptrs, stream=sptr)  # tunes, and first touch of the host pages
    e2e_steps = 2
    e0 = time.perf_counter()
    for _ in range(e2e_steps):
        be.run(values=hptrs, stream=sptr)
    torch.cuda.synchronize()
    e2e_ms = 1000.0 * (time.perf_counter() - e0) / e2e_steps
    del hv, hptrs
    be.close()
    pk, pk_kind = peaks()
    # the reduction kernels by class (element DOFs n): vector-load or scalar
    v4n = {c["n"] for c in res["mixed"]["tuning"]["gather"] if c.get("vector_loads")}
    alg_by = {k: alg for k in res["prof"] if not k.startswith("k_gather")}
    alg_by["k_gather_batch_v4"] = sum(a for i, a in zip(infos, algq) if i["n"] in v4n)
    alg_by["k_gather_batch"] = sum(a for i, a in zip(infos, algq) if i["n"] not in v4n)
    roof = roofline(res["prof"], alg_by, pk, pk_kind)
    step_gbs = alg / (res["mixed"]["ms"] / 1000.0) / 1e9
    roof["step"] = {"achieved": step_gbs, "frac": step_gbs / pk["hbm_gbs"], "algorithmic_bytes": alg,
                    "note": "fused-minimum bytes of all problems over the whole step"}
    orders = {}
    for c in cfgs:
        orders[str(c.order)] = orders.get(str(c.order), 0) + 1
    for p in plans:
        p.close()
    return {"metric": METRIC, "value": E / (res["mixed"]["ms"] / 1000.0), "unit": "element matrices/s",
            "ms_per_step": res["mixed"]["ms"], "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": "helmholtz3d_batch%d_m%d-%d_p1-4_k5-40_gauss2p" % (args.c4_n, args.c4_m_lo, args.c4_m_hi),
                       "problems": len(cfgs), "elements": E, "nnz": nnz, "unknowns": rows, "orders": orders,
                       "l2": "CSR outputs larger than L2, no flush"},
            "nnz_per_s": nnz / (res["mixed"]["ms"] / 1000.0),
            "fp64": {"value": E / (res["fp64"]["ms"] / 1000.0), "ms_per_step": res["fp64"]["ms"],
                     "method": "plain: quadrature loop of BilinearTerm::evaluate in FP64",
                     "quadrature_points": {str(c["n"]): c["nq"] for c in res["mixed"]["tuning"]["gather"]},
                     "note": "quadrature points per class (element DOFs: points) of the stand-in Gauss(2p) rules"},
            "fp64_factored": {"value": E / (res["fp64_factored"]["ms"] / 1000.0), "ms_per_step": res["fp64_factored"]["ms"],
                              "method": "exact factorization of the affine element matrices, FP64 on the CUDA cores"},
            "speedup_mixed_vs_fp64": res["fp64"]["ms"] / res["mixed"]["ms"],
            "speedup_mixed_vs_fp64_factored": res["fp64_factored"]["ms"] / res["mixed"]["ms"],
            "mixed_vs_fp64_rel_fro": res["rel_fro"], "worst_problem_rel_fro": res["worst_problem_rel_fro"],
            "first_run_s": {k: res[k]["first_run_s"] for k in ("mixed", "fp64", "fp64_factored")},
            "tuning": {"mixed": res["mixed"]["tuning"], "fp64": res["fp64"]["tuning"]},
            "gpu_launches": res["mixed"]["launches_per_step"] * args.steps,
            "e2e": {"value": E / (e2e_ms / 1000.0), "unit": "element matrices/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": nnz * 16,
                    "note": "fg_batch_run into pageable host arrays; the coefficients are constants (no input arrays)"},
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "pre_seconds": pre_s, "pre_wall_seconds": pre_wall}


def bench_multi_freq(args, femg, torch):
    """Navier 3-component P2 on m^3 x 6 tets, Lame lognormal per tet, 16
    frequencies omega ~ U[1, 10] in one pass; one step = one
    fg_assemble_multi_freq writing all 16 CSR value arrays in HBM."""
    m = args.c5_m or 60
    prob = femg.Problem(femg.config_c5(m=m, omega=0.0))
    pre_s = prob.pre_seconds()
    plan = prob.plan()
    info = plan.info()
    E, nnz, n = info["E"], prob.nnz, info["n"]
    rows = int(prob.sys.n_rows)
    F = args.n_freq
    omegas = np.random.default_rng(5).uniform(1.0, 10.0, F)
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    out = torch.empty(F * 2 * nnz, dtype=torch.float64, device="cuda")
    res = {}
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    for prec in ("mixed", "fp64"):
        steps = args.steps if prec == "mixed" else 2
        fn = lambda: plan.assemble_multi_freq(omegas, precision=prec, values=out.data_ptr(), rhs=False, stream=sptr)
        l0 = femg.lib().fg_launch_count()
        ms = timed_events(torch, stream, fn, args.warmup if prec == "mixed" else 1, steps)
        launches = (femg.lib().fg_launch_count() - l0) // ((args.warmup if prec == "mixed" else 1) + steps)
        if prec == "mixed":
            res["prof"] = profile_run(femg, torch, fn)
            res["launches"] = int(launches)
            first = out[: 2 * nnz].clone()
        else:
            ref = out[: 2 * nnz]
            res["rel_fro"] = torch.linalg.vector_norm(first - ref).item() / torch.linalg.vector_norm(ref).item()
            del first
        res[prec] = ms
    clk = clocks.stop()
    del out
    torch.cuda.empty_cache()
    # end to end: the Lame arrays from the host, all frequencies' CSR values
    # into pageable host memory (the reference's module arrays)
    tt, nt = prob.terms()
    h2d = sum(ex.n_arrays * E * 16 for k in range(nt) for ex in (tt[k].coef, tt[k].coef2)) + F * 8
    hv = np.empty((F, nnz), np.complex128)
    efn = lambda: plan.assemble_multi_freq(omegas, precision="mixed", values=hv, rhs=False, stream=sptr)
    efn()  # warm-up: first touch of the host pages
    e0 = time.perf_counter()
    for _ in range(2):
        efn()
    e2e_ms = 1000.0 * (time.perf_counter() - e0) / 2
    del hv
    pk, pk_kind = peaks()
    # fused minimum with all frequencies written: elements' geometry, Lame
    # pair and map once, F complex values per nonzero
    alg = E * (4 * 3 * 8 + 4 * 4 + 32 + n * n * 4) + F * nnz * 16
    roof = roofline(res["prof"], alg, pk, pk_kind)
    step_gbs = alg / (res["mixed"] / 1000.0) / 1e9
    roof["step"] = {"achieved": step_gbs, "frac": step_gbs / pk["hbm_gbs"],
                    "note": "the same fused-minimum bytes over the whole step (all kernels)"}
    cpu = None
    if not args.no_cpu:
        a = prob.arrays()
        r, S, dt, cores = cpu_rate(prob, a, args.cpu_seconds, freq=float(omegas[0]))
        cpu = {"value": r, "unit": "element matrices/s", "cores": cores, "kind": "port",
               "sample": "one frequency, first %d of %d elements, %.1f s (every frequency is a full assembly)" % (S, E, dt)}
    plan.close()
    prob.close()
    return {"metric": METRIC, "value": F * E / (res["mixed"] / 1000.0), "unit": "element matrices/s",
            "ms_per_step": res["mixed"], "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": "navier3d_tet_h1p2x3_%d3x6_gauss4_lame_%dfreq" % (m, F), "elements": E, "nnz_per_freq": nnz,
                       "unknowns": rows, "frequencies": F, "units": "element matrices: elements x frequencies",
                       "l2": "CSR outputs larger than L2, no flush"},
            "nnz_per_s": F * nnz / (res["mixed"] / 1000.0),
            "fp64": {"value": F * E / (res["fp64"] / 1000.0), "ms_per_step": res["fp64"]},
            "speedup_mixed_vs_fp64": res["fp64"] / res["mixed"], "mixed_vs_fp64_rel_fro_freq0": res["rel_fro"],
            "gpu_launches": res["launches"] * args.steps,
            "e2e": {"value": F * E / (e2e_ms / 1000.0), "unit": "element matrices/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": F * nnz * 16,
                    "note": "fg_assemble_multi_freq with host coefficient arrays and pageable host outputs"},
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "pre_seconds": pre_s}


def max_over_ranks(x, dist, device):
    """The largest x over the ranks (x on every rank; returns it everywhere)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, ms_max, world_size):
    """Whole-job throughput of independent replicas: all ranks' units over the
    slowest rank's time."""
    return world_size * units_per_rank / (ms_max / 1000.0)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_femg_host():
    """The ctypes binding without the GPU library: problems come from
    libfemg_host.so (built here if missing, host compiler only)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("femg_build", os.path.join(ROOT, "fem-g_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_host()
    from oracle import build as ob
    ob.build_oracle()
    spec = importlib.util.spec_from_file_location("femg", os.path.join(ROOT, "fem-g_gb300", "femg.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["femg"] = mod
    spec.loader.exec_module(mod)
    return mod


def run_reference(args, ws, rank):
    """The reference's CPU implementation of the path on this host's cores.
    Where the reference's own library was built (oracle/_ref/ref_assemble:
    its sources with the gmsh stand-in), its Formulation::assemble is timed
    on the whole workload (kind "reference"); elsewhere the oracle's C
    restatement of it, pinned to the reference at 1e-13 (kind "port"), on a
    bounded sample of the workload's elements. The process never loads the
    GPU library: problem set-up comes from the host-only library."""
    if rank != 0:
        return
    femg = load_femg_host()
    cfg, wname = workload_config(femg, args.workload if args.workload not in ("c4", "c5mf") else "c3", args.m)
    from oracle import reference as R
    from oracle import oracle as O
    base = {"impl": "reference", "metric": METRIC, "unit": "element matrices/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex128",
            "data": "synthetic (seeded, reference configuration shapes)"}
    if R.available() and args.ref_kind in ("auto", "reference"):
        runs = max(1, min(args.steps, 3))
        r = R.run(cfg, threads=0, repeats=runs + 1)
        prob = femg.Problem(cfg, host_only=True)
        E = prob.E
        rate = E / r["assemble_seconds"]
        line = dict(base, value=rate, ms_per_step=1000.0 * r["assemble_seconds"],
                    config={"workload": wname, "elements": E, "nnz": r["nnz"], "sample_elements": E},
                    nnz_per_s=r["nnz"] / r["assemble_seconds"],
                    cpu_baseline={"value": rate, "unit": "element matrices/s", "cores": r["threads"], "kind": "reference",
                                  "sample": "the whole workload: the reference's Formulation::assemble (its sources, gmsh "
                                            "stand-in), median of %d runs after one" % r["timed_runs"]},
                    e2e={"value": rate, "unit": "element matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    pre_seconds=r["pre_seconds"])
        print(json.dumps(line), flush=True)
        return
    prob = femg.Problem(cfg, host_only=True)
    a = prob.arrays()
    t, nt = prob.terms()
    S = min(a["E"], args.ref_sample)
    b = sub_arrays(a, S)
    for _ in range(args.warmup):
        O.assemble(b, t, nt)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.assemble(b, t, nt)
        times.append(time.perf_counter() - t0)
    ms = 1000.0 * float(np.mean(times))
    rate = S / (ms / 1000.0)
    line = dict(base, value=rate, ms_per_step=ms,
                config={"workload": wname, "elements": int(a["E"]), "nnz": prob.nnz, "sample_elements": S},
                nnz_per_s=rate * prob.nnz / a["E"],
                cpu_baseline={"value": rate, "unit": "element matrices/s", "cores": O.num_threads(), "kind": "port",
                              "sample": "first %d of %d elements per step, the oracle's C restatement of "
                                        "Formulation::assemble (pinned to the reference's own assembly)" % (S, a["E"])},
                e2e={"value": rate, "unit": "element matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3")
    ap.add_argument("--m", type=int, default=0)
    ap.add_argument("--ref-sample", type=int, default=60000)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--c4-n", type=int, default=64)
    ap.add_argument("--c4-m-lo", type=int, default=8)
    ap.add_argument("--c4-m-hi", type=int, default=48)
    ap.add_argument("--n-freq", type=int, default=16)
    ap.add_argument("--c5-m", type=int, default=60)
    ap.add_argument("--no-c4", action="store_true", help="leave the batched workload out of the default line")
    ap.add_argument("--no-c5", action="store_true", help="leave the multi-frequency workload out of the default line")
    ap.add_argument("--ref-kind", default="auto", choices=["auto", "reference", "port"])
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    femg = load_femg()
    if args.workload in ("c4", "c5mf"):
        if ws > 1:
            raise SystemExit("the batched and multi-frequency workloads run on one GPU")
        sub = (bench_batch if args.workload == "c4" else bench_multi_freq)(args, femg, torch)
        line = dict(sub, n_gpus=1, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="fp32-tf32x3/fp64",
                    data="synthetic (seeded, reference configuration shapes)")
        line["config"] = dict(sub["config"], parallelism="single")
        print(json.dumps(line), flush=True)
        return
    line = bench_headline(args, femg, torch, ws, rank, local, dist)
    # the batched (c4) and multi-frequency (c5) workloads of the target, one
    # GPU each, after the headline's buffers are released. Each runs in a child
    # process of its own: the batch alone holds about 120 GB of host memory
    # (64 problems' patterns, and 78 GB of host outputs for its end-to-end
    # figure), which a process that ran the headline before does not give
    # back to the system in full.
    if rank == 0 and ws == 1 and args.workload == "c3":
        torch.cuda.empty_cache()
        if not args.no_c4:
            line["c4"] = run_child(args, "c4")
        if not args.no_c5:
            line["c5mf"] = run_child(args, "c5mf")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_child(args, workload):
    """bench.py --workload <workload> in a child process: its JSON line."""
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", workload, "--steps", str(args.steps), "--warmup",
           str(args.warmup), "--cpu-seconds", str(args.cpu_seconds), "--c4-n", str(args.c4_n), "--c4-m-lo",
           str(args.c4_m_lo), "--c4-m-hi", str(args.c4_m_hi), "--n-freq", str(args.n_freq), "--c5-m", str(args.c5_m)]
    if args.no_cpu:
        cmd.append("--no-cpu")
    r = subprocess.run(cmd, capture_output=True, text=True)
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"error": "bench.py --workload %s exited %d: %s" % (workload, r.returncode, (r.stderr or "")[-500:])}
    return json.loads(lines[-1])


def bench_headline(args, femg, torch, ws, rank, local, dist):
    """The headline workload (default: 384,000 order-3 tets with per-tet
    coefficients), timed on every rank; returns rank 0's line (None elsewhere)."""
    cfg, wname = workload_config(femg, args.workload, args.m)
    t0 = time.perf_counter()
    prob = femg.Problem(cfg)
    pre_s = prob.pre_seconds()
    t1 = time.perf_counter()
    plan = prob.plan()
    plan_s = time.perf_counter() - t1
    plan.bind_terms()
    a_info = plan.info()
    E, nnz, nrows = a_info["E"], a_info["nnz"], int(prob.sys.n_rows)
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    dv = torch.empty(2 * nnz, dtype=torch.float64, device="cuda")
    db = torch.empty(2 * nrows, dtype=torch.float64, device="cuda")
    dv64 = torch.empty_like(dv)

    precisions = ["mixed", "fp64"]
    try:
        plan.assemble("mixed", values=dv.data_ptr(), rhs=db.data_ptr(), bound=True, stream=sptr)
    except femg.FgError as e:
        if e.status != femg.FG_ERR_UNSUPPORTED:
            raise
        precisions = ["fp64"]

    def step(prec, out):
        plan.assemble(prec, values=out.data_ptr(), rhs=db.data_ptr(), bound=True, stream=sptr)

    def barrier():
        if ws > 1:
            dist.barrier()

    def timed(prec, out, steps, profile=False):
        for _ in range(args.warmup):
            step(prec, out)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        if profile:
            femg.profile_read()
            femg.profile_enable(True)
        l0 = femg.lib().fg_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(prec, out)
        e1.record(stream)
        torch.cuda.synchronize()
        launches = femg.lib().fg_launch_count() - l0
        prof = None
        if profile:
            femg.profile_enable(False)
            prof = femg.profile_read()
        barrier()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        if ws > 1:
            ms = max_over_ranks(ms, dist, "cuda")
        return ms, launches, prof

    # clocks are sampled over both timed regions (the mixed one alone lasts
    # only milliseconds)
    clocks = ClockSampler(local)
    clocks.start()
    head = precisions[0]
    ms_head, launches, prof = timed(head, dv, args.steps, profile=True)
    fp64_steps = max(3, min(args.steps, 5)) if head == "mixed" else args.steps
    ms_fp64 = ms_head if head == "fp64" else timed("fp64", dv64, fp64_steps)[0]
    # beside the plain FP64 method (the quadrature loop), FP64 with the exact
    # factorization of the affine element matrices: what the algorithm alone gives
    plan.set_fp64_method(femg.FG_FP64_FACTORED)
    ms_fp64_fact = timed("fp64", dv64, 5)[0]
    plan.set_fp64_method(femg.FG_FP64_QUADRATURE)
    # the fused mixed kernel (contraction and reduction in one launch, opt-in)
    fused = None
    if head == "mixed":
        finfo = plan.fused_info()
        if finfo["applies"]:
            plan.set_mixed_fused(True)
            ms_fused, _, fprof = timed("mixed", dv64, 5, profile=True)
            plan.set_mixed_fused(False)
            fused = {"ms_per_step": ms_fused, "value": ws * E / (ms_fused / 1000.0), "blocks": finfo["blocks"],
                     "elements_per_block": finfo["elems_per_block"],
                     "contractions_per_element": finfo["contractions_per_element"],
                     "kernels": {k: {"launches": v[0], "total_ms": v[1]} for k, v in (fprof or {}).items()}}
        else:
            fused = {"applies": False, "why": finfo["why"]}
    clk = clocks.stop()
    if head == "mixed":
        step("fp64", dv64)
        torch.cuda.synchronize()
        vm = dv.view(torch.complex128) if hasattr(dv, "view") else dv
        diff = torch.linalg.vector_norm(dv - dv64).item() / max(torch.linalg.vector_norm(dv64).item(), 1e-300)
    else:
        diff = 0.0

    # end to end through the C ABI: host coefficient arrays and host (pinned) outputs
    hv = torch.empty(2 * nnz, dtype=torch.float64, pin_memory=True)
    hb = torch.empty(2 * nrows, dtype=torch.float64, pin_memory=True)
    tt, nt = prob.terms()
    h2d = 0
    for k in range(nt):
        for ex in (tt[k].coef, tt[k].coef2):
            h2d += ex.n_arrays * E * 16
    h2d += int(prob.sys.n_fixed) * 16
    d2h = (nnz + nrows) * 16
    L = femg.lib()
    dptr = C.cast(prob.dir_ptr, C.c_void_p) if prob.sys.n_fixed else None
    fn = L.fg_assemble_mixed if head == "mixed" else L.fg_assemble_fp64
    extra = (None,) if head == "mixed" else ()

    def e2e_step():
        femg.check(fn(plan.ptr, tt, nt, 0.0, dptr, hv.data_ptr(), hb.data_ptr(), sptr, *extra))

    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    w0 = time.perf_counter()
    e2e_calls = []
    for _ in range(e2e_steps):
        c0 = time.perf_counter()
        e2e_step()
        e2e_calls.append(1000.0 * (time.perf_counter() - c0))
    torch.cuda.synchronize()
    e2e_ms = 1000.0 * (time.perf_counter() - w0) / e2e_steps
    if ws > 1:
        e2e_ms = max_over_ranks(e2e_ms, dist, "cuda")
    # the same into ordinary (pageable) host memory: the reference's module
    # array is a std::vector, which a drop-in writes unless it registers it
    pv = np.empty(nnz, np.complex128)
    pb = np.empty(nrows, np.complex128)

    def e2e_pageable_step():
        femg.check(fn(plan.ptr, tt, nt, 0.0, dptr, pv.ctypes.data, pb.ctypes.data, sptr, *extra))

    e2e_pageable_step()  # first touch of the pages
    p_calls = []
    for _ in range(e2e_steps):
        c0 = time.perf_counter()
        e2e_pageable_step()
        p_calls.append(1000.0 * (time.perf_counter() - c0))
    e2e_pageable_ms = float(np.mean(p_calls))
    del pv, pb

    # roofline of the dominant kernel (algorithmic bytes of the fused minimum
    # per launch / measured average launch time)
    pk, pk_kind = peaks()
    dom, (dcount, dms) = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (1, 0.0))
    n_el = plan.info()["n"]
    nv_nodes = 4
    coef_bytes = 16  # per-element complex coefficient
    alg_bytes = E * (nv_nodes * 3 * 8 + nv_nodes * 4 + coef_bytes + n_el * n_el * 4) + nnz * 16 + nrows * 16
    avg_ms = dms / max(dcount, 1)
    achieved = alg_bytes / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else 0.0
    traffic, traffic_src = None, None
    if dom in GATHER_TRAFFIC_PER_NNZ_P3 and args.workload in ("c2", "c3") and head == "mixed":
        traffic = GATHER_TRAFFIC_PER_NNZ_P3[dom] * nnz
        traffic_src = "ncu dram bytes of %s on the 30^3 x 6 P3 mesh, scaled by nonzeros" % dom
    step_gbs = alg_bytes / (ms_head / 1000.0) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": traffic, "traffic_source": traffic_src, "kernel": dom,
            "kernel_avg_ms": avg_ms, "algorithmic_bytes": alg_bytes, "peak_source": pk_kind,
            "kernels": {k: {"launches": v[0], "total_ms": v[1]} for k, v in (prof or {}).items()},
            "step": {"achieved": step_gbs, "frac": step_gbs / pk["hbm_gbs"],
                     "note": "the same fused-minimum bytes over the whole step (all kernels)"}}

    if rank == 0:
        cpu = None
        if not args.no_cpu:
            a = prob.arrays()
            rate, S, dt, cores = cpu_rate(prob, a, args.cpu_seconds)
            cpu = {"value": rate, "unit": "element matrices/s", "cores": cores, "kind": "port",
                   "sample": "first %d of %d elements, %.1f s, oracle restatement of Formulation::assemble" % (S, E, dt),
                   "quadrature_points": plan.info()["nq"]}
        value = replica_value(E, ms_head, ws)
        line = {"metric": METRIC, "value": value, "unit": "element matrices/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_head, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "fp32-tf32x3/fp64" if head == "mixed" else "fp64",
                "data": "synthetic (seeded, reference configuration shapes)",
                "config": {"workload": wname, "elements": E, "nnz": nnz, "unknowns": nrows, "dofs_per_element": n_el,
                           "quadrature_points": plan.info()["nq"], "precision": head, "l2": "CSR output larger than L2, no flush",
                           "parallelism": "replicas" if ws > 1 else "single"},
                "nnz_per_s": ws * nnz / (ms_head / 1000.0),
                "fp64": {"value": ws * E / (ms_fp64 / 1000.0), "ms_per_step": ms_fp64, "nnz_per_s": ws * nnz / (ms_fp64 / 1000.0),
                         "method": "plain: quadrature loop of BilinearTerm::evaluate in FP64",
                         "quadrature_points": plan.info()["nq"],
                         "fp64_pipe_active": (ELEMENT_FP64_PIPE_ACTIVE_P3 if args.workload in ("c2", "c3") else None),
                         "note": ("the quadrature loop's work is proportional to the points of the rule; the stand-in "
                                  "Gauss%d rule has %d points (Grundmann-Moeller), a published degree-6 tetrahedral rule "
                                  "(Keast) has 24" % (cfg.gauss, plan.info()["nq"]) if cfg.dim == 3 and cfg.gauss == 6 else
                                  "the quadrature loop's work is proportional to the points of the rule")},
                "fp64_factored": {"value": ws * E / (ms_fp64_fact / 1000.0), "ms_per_step": ms_fp64_fact,
                                  "method": "exact factorization of the affine element matrices, FP64 on the CUDA cores"},
                "speedup_mixed_vs_fp64_factored": ms_fp64_fact / ms_head,
                "mixed_fused": fused,
                "mixed_vs_fp64_rel_fro": diff,
                "speedup_mixed_vs_fp64": ms_fp64 / ms_head,
                "pre_seconds": pre_s, "plan_seconds": plan_s,
                "e2e": {"value": replica_value(E, e2e_ms, ws), "unit": "element matrices/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "host_memory": "page-locked",
                        "ms_per_call": {"median": float(np.median(e2e_calls)), "min": min(e2e_calls), "max": max(e2e_calls)}},
                "e2e_pageable": {"value": replica_value(E, e2e_pageable_ms, ws), "unit": "element matrices/s",
                                 "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_pageable_ms,
                                 "host_memory": "pageable (as the reference's std::vector module array)",
                                 "ms_per_call": {"median": float(np.median(p_calls)), "min": min(p_calls), "max": max(p_calls)}},
                "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "clocks": clk}
        return line
    return None


if __name__ == "__main__":
    main()
