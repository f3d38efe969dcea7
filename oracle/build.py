"""Build recipe of the oracle — TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/liboracle.so``: the plain-C restatement (oracle.c), built
  with gcc on any machine (here and on the GPU machine).
* ``oracle/_ref/libref.so``: the reference's own numbering code compiled from
  its sources where they lie (fem-master/src/reorder/Hilbert.cpp and the
  vendored fem-master/contrib/robin-hood-hashing/robin_hood.h) around
  ref_driver.cpp. Built only where the reference tree is present; the rest
  of the reference needs gmsh (absent) and cmake-generated headers, so it is
  not built.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(REF_OUT, "libref.so")
REFERENCE = "/root/reference/fem-master"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    _run(["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", LIB, "-lm"])
    return LIB


def build_ref():
    """Compile the reference's numbering sources (only where they exist)."""
    if not os.path.isdir(REFERENCE):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(REFERENCE, "src/reorder/Hilbert.cpp")]
    deps = srcs + [os.path.join(HERE, "ref_shim", "OmpInterface.h")]
    if os.path.exists(REF_LIB) and os.path.getmtime(REF_LIB) >= max(os.path.getmtime(p) for p in deps):
        return REF_LIB
    _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared",
          "-I" + os.path.join(HERE, "ref_shim"),
          "-I" + os.path.join(REFERENCE, "src/reorder"),
          "-I" + os.path.join(REFERENCE, "contrib/robin-hood-hashing")] + srcs + ["-o", REF_LIB])
    return REF_LIB


def build():
    build_oracle()
    build_ref()


if __name__ == "__main__":
    build()
    print(LIB, REF_LIB if os.path.exists(REF_LIB) else "(no reference build)")
