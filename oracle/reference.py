"""The reference's own assembly (GmshFEM's Formulation::pre and assemble,
compiled from its sources with the gmsh stand-in of oracle/gmsh_shim/) —
TEST INFRASTRUCTURE ONLY.

``run(cfg)`` runs ``oracle/_ref/ref_assemble`` (built by oracle/build.py
where the reference tree is present) on one problem in a child process and
returns what the reference produced: its CSR pattern and values, right-hand
side, and DOF dictionary with the numbering. ``available()`` says whether the
program was built here. ``run(cfg, dropin=True)`` runs ``ref_dropin``
instead: the same program whose formulation is the GpuFormulation binding,
its C ABI calls recorded (``read_record``) and assembled by the oracle.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "_ref", "ref_assemble")
DROPIN_EXE = os.path.join(HERE, "_ref", "ref_dropin")
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


def dropin_available():
    return os.path.exists(DROPIN_EXE)


def run(cfg, threads=0, repeats=1, timeout=3600, programs=None, dropin=False):
    """Reference pre() + assemble() of the problem `cfg` (an
    fg_problem_config, from femg.config*). threads = 0: all host threads.
    repeats > 1: assemble() that many times (setSystemToZero in between) and
    report the median wall time of the repeats after the first. programs:
    coefficient programs that replace the terms of a scalar problem
    (write_programs). dropin: the drop-in program; the result then also
    holds "record", its C ABI calls (read_record)."""
    exe = DROPIN_EXE if dropin else EXE
    if not os.path.exists(exe):
        raise RuntimeError("the reference program is not built (oracle/build.py, needs the reference tree)")
    threads = threads or os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "out.bin")
        extra = []
        if programs:
            extra = [os.path.join(tmp, "programs.txt")]
            write_programs(extra[0], programs)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        if dropin:
            env["FEMG_RECORD"] = os.path.join(tmp, "record.bin")
        r = subprocess.run([exe, path, str(threads), str(repeats)] + _args(cfg) + extra, capture_output=True, text=True,
                           timeout=timeout, env=env)
        if r.returncode != 0:
            raise RuntimeError("%s failed (%d): %s%s" % (os.path.basename(exe), r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
        raw = open(path, "rb").read()
        record = read_record(env["FEMG_RECORD"]) if dropin and os.path.exists(env["FEMG_RECORD"]) else None
        log = r.stdout + r.stderr
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
    out["log"] = log
    nsep = int(take(np.uint64, 1)[0])
    if nsep:  # assemble(separate = true): values are K, then C and M
        out["K"] = out["values"]
        out["C"] = take(np.complex128, nnz)
        out["M"] = take(np.complex128, nnz)
    if dropin:
        out["record"] = record or []
    assert pos == len(raw)
    return out


def read_record(path):
    """The C ABI calls of the drop-in program (the record format of
    fg_record.cpp): a list of dicts, one per fg_assemble_fp64 call, with the
    arrays of oracle.assemble's bucket dictionaries and the terms as
    (kind, dt, [(op, arg, re, im)], [arrays], [(code, arrays)] of the
    term's vector or tensor programs, (code, arrays) of its second
    coefficient))."""
    raw = open(path, "rb").read()
    assert raw[:8] == b"FEMGREC1"
    pos = 8

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos).copy()
        pos += a.nbytes
        return a

    def one(dtype):
        return take(dtype, 1)[0].item()

    calls = []
    while pos < len(raw):
        c = {}
        c["entry"] = one(np.int32)  # 0: fg_assemble_fp64, 1: fg_assemble_separate
        c["dim"], c["nn"] = one(np.int32), one(np.int32)
        nodes = one(np.int64)
        c["xyz"] = take(np.float64, 3 * nodes).reshape(nodes, 3)
        E = one(np.int64)
        c["E"] = E
        c["enodes"] = take(np.int64, E * c["nn"]).reshape(E, c["nn"])
        nq = one(np.int32)
        c["nq"] = nq
        c["w"] = take(np.float64, nq)
        c["geo_val"] = take(np.float64, nq * c["nn"]).reshape(nq, c["nn"])
        c["geo_grad"] = take(np.float64, nq * c["nn"] * 3).reshape(nq, c["nn"], 3)
        c["nb"], c["mult"], c["n_orient"], c["form"] = (one(np.int32) for _ in range(4))
        comp = 3 if c["form"] == 1 else 1
        c["bval"] = take(np.float64, c["n_orient"] * nq * c["nb"] * comp)
        c["bgrad"] = take(np.float64, c["n_orient"] * nq * c["nb"] * 3)
        c["orient"] = take(np.int32, E) if one(np.int32) else np.zeros(E, np.int32)
        n_rows = one(np.uint64)
        c["n_rows"] = n_rows
        c["ai"] = take(np.uint64, n_rows + 1)
        c["aj"] = take(np.uint64, int(c["ai"][-1]))
        n = c["nb"] * c["mult"]
        c["edof"] = take(np.uint64, E * n).reshape(E, n)
        c["etype"] = take(np.int32, E * n).reshape(E, n)
        c["n_fixed"] = one(np.uint64)
        c["upper"] = one(np.int32)
        c["coupled"] = one(np.int32)
        if c["coupled"]:
            nbu, nou, formu = one(np.int32), one(np.int32), one(np.int32)
            u = {"nb": nbu, "n_orient": nou, "form": formu}
            u["bval"] = take(np.float64, nou * nq * nbu * (3 if formu == 1 else 1))
            u["bgrad"] = take(np.float64, nou * nq * nbu * 3)
            u["orient"] = take(np.int32, E) if one(np.int32) else np.zeros(E, np.int32)
            u["edof"] = take(np.uint64, E * nbu).reshape(E, nbu)
            u["etype"] = take(np.int32, E * nbu).reshape(E, nbu)
            c["unknown"] = u
        c["frequency"] = one(np.float64)
        c["dirichlet"] = take(np.complex128, c["n_fixed"])
        def program():
            code = []
            for _ in range(one(np.int32)):
                op, arg = one(np.int32), one(np.int32)
                re, im = one(np.float64), one(np.float64)
                code.append((op, arg, re, im))
            arrays = [take(np.float64, one(np.uint64)) for _ in range(one(np.int32))]
            return code, arrays

        terms = []
        for _ in range(one(np.int32)):
            kind, dt = one(np.int32), one(np.int32)
            code, arrays = program()
            code2, arrays2 = program()
            tensor = [program() for _ in range(one(np.int32))]
            terms.append((kind, dt, code, arrays, tensor, (code2, arrays2)))
        c["terms"] = terms
        calls.append(c)
    return calls
