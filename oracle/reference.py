"""The reference's own assembly (GmshFEM's Formulation::pre and assemble,
compiled from its sources with the gmsh stand-in of oracle/gmsh_shim/) —
TEST INFRASTRUCTURE ONLY.

``run(cfg)`` runs ``oracle/_ref/ref_assemble`` (built by oracle/build.py
where the reference tree is present) on one problem in a child process and
returns what the reference produced: its CSR pattern and values, right-hand
side, and DOF dictionary with the numbering. ``available()`` says whether the
program was built here.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "_ref", "ref_assemble")
MAGIC = 0x46454D4752454631

FIELDS = ["kind", "dim", "m", "mesh_order", "space", "order", "gauss", "jitter", "seed", "k", "coef_mode", "dirichlet",
          "dirichlet_value", "source", "omega", "lame_sigma", "upper", "order2"]


def available():
    return os.path.exists(EXE)


def _args(cfg):
    out = []
    for f in FIELDS:
        v = getattr(cfg, f) if not isinstance(cfg, dict) else cfg[f]
        out.append(repr(float(v)) if isinstance(v, float) else str(int(v)))
    return out


def write_programs(path, programs):
    """programs: {"grad" | "mass" | "source": [(op, arg, re, im), ...]}"""
    with open(path, "w") as f:
        for term, code in programs.items():
            f.write("%s %d\n" % (term, len(code)))
            for op, arg, re, im in code:
                f.write("%d %d %r %r\n" % (op, arg, float(re), float(im)))


def run(cfg, threads=0, repeats=1, timeout=3600, programs=None):
    """Reference pre() + assemble() of the problem `cfg` (an
    fg_problem_config, from femg.config*). threads = 0: all host threads.
    repeats > 1: assemble() that many times (setSystemToZero in between) and
    report the median wall time of the repeats after the first. programs:
    coefficient programs that replace the terms of a scalar problem
    (write_programs)."""
    if not available():
        raise RuntimeError("the reference program is not built (oracle/build.py, needs the reference tree)")
    threads = threads or os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "out.bin")
        extra = []
        if programs:
            extra = [os.path.join(tmp, "programs.txt")]
            write_programs(extra[0], programs)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        r = subprocess.run([EXE, path, str(threads), str(repeats)] + _args(cfg) + extra, capture_output=True, text=True,
                           timeout=timeout, env=env)
        if r.returncode != 0:
            raise RuntimeError("ref_assemble failed (%d): %s%s" % (r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
        raw = open(path, "rb").read()
    pos = 0

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos).copy()
        pos += a.nbytes
        return a

    assert int(take(np.uint64, 1)[0]) == MAGIC
    n, nnz = (int(x) for x in take(np.uint64, 2))
    out = {"n_rows": n, "nnz": nnz}
    out["ai"] = take(np.uint64, n + 1)
    out["aj"] = take(np.uint64, nnz)
    out["values"] = take(np.complex128, nnz)
    out["rhs"] = take(np.complex128, n)
    # every field's DOF dictionary in its iteration order, field after field
    parts = {"dof_num_type": [], "dof_entity": [], "dof_num_dof": [], "dof_assemble_type": []}
    nf = int(take(np.uint64, 1)[0])
    for _ in range(nf):
        nd = int(take(np.uint64, 1)[0])
        parts["dof_num_type"].append(take(np.uint64, nd))
        parts["dof_entity"].append(take(np.uint64, nd))
        parts["dof_num_dof"].append(take(np.uint64, nd))
        parts["dof_assemble_type"].append(take(np.int32, nd))
    for k, v in parts.items():
        out[k] = np.concatenate(v)
    out["fields"] = nf
    out["pre_seconds"] = float(take(np.float64, 1)[0])
    out["assemble_seconds"] = float(take(np.float64, 1)[0])
    out["timed_runs"] = int(take(np.uint64, 1)[0])
    out["threads"] = threads
    assert pos == len(raw)
    return out
