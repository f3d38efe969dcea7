"""The multi-GPU path is replicas only: every rank assembles its own copy of
the workload and the benchmark reports all ranks' element matrices over the
slowest rank's time. Two gloo ranks on the CPU check that the replicas agree
(CSR of the oracle on each rank) and the max-over-ranks timing."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "fem-g_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import femg
    from oracle import oracle
    prob = femg.Problem(femg.config_c3(m=2))
    a = prob.arrays()
    t, nt = prob.terms()
    v, _ = oracle.assemble(a, t, nt)
    mine = torch.from_numpy(v.view(np.float64).copy())
    gathered = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine)
    # the oracle adds with OpenMP atomics like the reference: equal to rounding
    same = all(float(torch.linalg.vector_norm(g - gathered[0]) / torch.linalg.vector_norm(gathered[0])) <= 1e-13
               for g in gathered)
    ms = 1.0 + rank  # this rank's step time
    ms_max = bench.max_over_ranks(ms, dist, "cpu")
    value = bench.replica_value(int(a["E"]), ms_max, world)
    out.put((rank, same, ms_max, value, int(a["E"])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_agree_and_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, same, ms_max, value, E in res:
        assert same
        assert ms_max == 2.0
        assert value == pytest.approx(2 * E / 0.002)
