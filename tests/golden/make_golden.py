"""Generates tests/golden/golden_small.npz: golden vectors for the numbering
and assembly path, from the reference's own code where it builds here.

- hilbert_{2,3}d: seeded float32 points (with ties) and the permutation that
  the reference's Hilbert sort (src/reorder/Hilbert.cpp:174-288, compiled
  into oracle/_ref/libref.so from the reference tree) gives them.
- robin_<case>: the DOF dictionary iteration order that the reference's
  robin_hood 3.8.0 map (robin_hood.h as vendored in the reference tree, in
  libref.so) gives for the case's DOF creation and reserve() script.
- csr_<case>: ai, aj, CSR values and right-hand side that the reference's
  own Formulation::pre() and assemble() produce (oracle/_ref/ref_assemble:
  the reference library compiled with the gmsh stand-in), and dof_<case>:
  the reference's DOF dictionary in iteration order (keys, assemble types,
  numbering).

Run from the repository root after oracle/build.py has built liboracle.so,
libref.so and ref_assemble:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fem-g_gb300"))

CASES = {
    "c1_m8": dict(cfg="config_c1", kw=dict(m=8)),
    "c1_m8_dirichlet1": dict(cfg="config_c1", kw=dict(m=8), set=dict(dirichlet_value=1.0)),
    "c2_m2": dict(cfg="config_c2", kw=dict(m=2)),
    "c2_m1_p4": dict(cfg="config_c2", kw=dict(m=1, order=4)),
    "c3_m2": dict(cfg="config_c3", kw=dict(m=2)),
    "c3_m4": dict(cfg="config_c3", kw=dict(m=4)),
    "c5_m1": dict(cfg="config_c5", kw=dict(m=1)),
    "c5_m2": dict(cfg="config_c5", kw=dict(m=2)),
    "maxwell_3d_m2": dict(cfg="config", kw=dict(kind=2, dim=3, m=2, mesh_order=1, space=2, order=0, gauss=2, jitter=0.15,
                                                seed=7, k=3.0, coef_mode=1)),
    "upper_c3_m2": dict(cfg="config_c3", kw=dict(m=2), set=dict(upper=1)),
}


def build_config(femg, name):
    spec = CASES[name]
    cfg = getattr(femg, spec["cfg"])(**spec["kw"])
    for k, v in spec.get("set", {}).items():
        setattr(cfg, k, v)
    return cfg


def build_case(femg, name):
    return femg.Problem(build_config(femg, name))


def dictionary_script(oracle, prob):
    cr = prob.created_dofs()
    at, arg = prob.reserve_log()
    kinds, args = oracle.robin_script(len(cr["num_type"]), at, arg)
    return cr, kinds, args


def main():
    import femg
    from oracle import oracle, reference

    if oracle.ref() is None:
        raise SystemExit("oracle/_ref/libref.so is not built (the reference tree is needed to make the fixtures)")
    if not reference.available():
        raise SystemExit("oracle/_ref/ref_assemble is not built (the reference tree is needed to make the fixtures)")
    out = {}
    for dim in (2, 3):
        rng = np.random.default_rng(100 + dim)
        pts = rng.random((4000, dim), dtype=np.float32)
        pts[50:120] = pts[0]  # ties: stable order
        mn = np.full(dim, -1e-6, np.float32)
        mx = np.full(dim, 1 + 1e-6, np.float32)
        out["hilbert_%dd_pts" % dim] = pts
        out["hilbert_%dd_perm" % dim] = oracle.ref_hilbert_order(dim, pts, mn, mx)
    for name in CASES:
        prob = build_case(femg, name)
        cr, kinds, args = dictionary_script(oracle, prob)
        out["robin_%s" % name] = oracle.robin_order(kinds, args, cr["num_type"], cr["entity"], use_ref=True)
        ref = reference.run(build_config(femg, name), threads=4)
        out["csr_%s_ai" % name] = ref["ai"]
        out["csr_%s_aj" % name] = ref["aj"]
        out["csr_%s_values" % name] = ref["values"]
        out["csr_%s_rhs" % name] = ref["rhs"]
        for k in ("num_type", "entity", "num_dof", "assemble_type"):
            out["dof_%s_%s" % (name, k)] = ref["dof_" + k]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
