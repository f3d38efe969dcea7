"""Generates tests/golden/dropin.npz: the C ABI calls that the drop-in binding
(fem-g_gb300/binding/GpuFormulation.h, compiled against the reference's
headers into oracle/_ref/ref_dropin) makes for the cases of
tests/dropin_cases.py, and what the reference's own Formulation::assemble
(oracle/_ref/ref_assemble) produces for the same problems: CSR values and
right-hand side. The GPU tests replay the calls through libfemg.so and set
the result against the reference's; the reference tree does not exist where
they run.

Run from the repository root after oracle/build.py has built ref_assemble and
ref_dropin:  python tests/golden/make_dropin.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fem-g_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import femg  # noqa: E402
from dropin_cases import cases, to_fixture  # noqa: E402
from oracle import reference  # noqa: E402


def main():
    out = {}
    names = []
    for name, (cfg, progs) in cases(femg).items():
        ref = reference.run(cfg, threads=2, programs=progs)
        drop = reference.run(cfg, threads=2, programs=progs, dropin=True)
        assert len(drop["record"]) >= 1, name
        out.update(to_fixture(name + "/", drop["record"], ref))
        names.append(name)
    out["cases"] = np.array(names)
    path = os.path.join(ROOT, "tests", "golden", "dropin.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
