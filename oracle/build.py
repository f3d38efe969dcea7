"""Build recipes of the oracle — TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/liboracle.so``: the plain-C restatement (oracle.c), built
  with gcc on any machine (here and on the GPU machine).
* ``oracle/_ref/libref.so``: the reference's own numbering code compiled from
  its sources where they lie (fem-master/src/reorder/Hilbert.cpp and the
  vendored fem-master/contrib/robin-hood-hashing/robin_hood.h) around
  ref_driver.cpp.
* ``oracle/_ref/ref_assemble``: the reference's whole library (every
  fem-master/src/**/*.cpp but the analytics, which need Boost) compiled where
  it lies with g++ -O3 (its cmake Release flags), OpenMP on, PETSc, SLEPc,
  Boost and Bessel off, the vendored Eigen 3.4.0 and robin-hood 3.8.0,
  against the hand-written configuration header and the gmsh stand-in of
  gmsh_shim/ (with this project's meshes and reference-element tables from
  fem-g_gb300/host/), linked with ref_assemble.cpp into a program that runs
  the reference's Formulation::pre() and assemble() on one problem.
* ``oracle/_ref/ref_dropin``: the same program built with FEMG_DROPIN, its
  formulations being the GpuFormulation of fem-g_gb300/binding/ (compiled
  against the reference's headers), linked with fg_record.cpp, a stand-in of
  the C ABI that records the binding's calls and assembles them with the
  oracle (oracle.c).

The last two are built only where the reference tree is present: the
directory ``$FEMG_REFERENCE_DIR``, by default the reference checkout of this
machine. Nothing is copied out of it; objects go to ``oracle/_ref/obj``.
"""
import concurrent.futures
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(REF_OUT, "libref.so")
REF_EXE = os.path.join(REF_OUT, "ref_assemble")
DROPIN_EXE = os.path.join(REF_OUT, "ref_dropin")
REFERENCE = os.environ.get("FEMG_REFERENCE_DIR", "/root/reference/fem-master")

# reference source directories (include paths), as its CMakeLists.txt lists them
REF_DIRS = ["algebra", "analytics", "common", "common/io", "equation", "dofs", "domain", "field", "function",
            "function/executionTree", "post", "post/mesh", "problem", "reorder", "system", "term", "term/evaluator"]
HOST_SOURCES = ["mesh.cpp", "refelem.cpp", "dofs.cpp", "formulation.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout[-4000:], r.stderr[-4000:]))


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


def _compile_obj(src, obj, flags, deps_time):
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), deps_time):
        return obj
    _run(["g++"] + flags + ["-c", src, "-o", obj])
    return obj


def build_gmshfem_ref(jobs=None):
    """Compile the reference library with the gmsh stand-in and link the
    reference-assembly program (only where the reference tree exists)."""
    if not os.path.isdir(REFERENCE):
        return None
    objdir = os.path.join(REF_OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    shim = os.path.join(HERE, "gmsh_shim")
    host = os.path.join(ROOT, "fem-g_gb300", "host")
    inc = ["-I" + shim] + ["-I" + os.path.join(REFERENCE, "src", d) for d in REF_DIRS]
    inc += ["-I" + os.path.join(REFERENCE, "contrib/eigen"), "-I" + os.path.join(REFERENCE, "contrib/robin-hood-hashing")]
    ref_flags = ["-std=c++17", "-O3", "-DNDEBUG", "-fPIC", "-fopenmp", "-w"] + inc
    own_flags = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off"]
    shim_time = max(os.path.getmtime(p) for p in glob.glob(os.path.join(shim, "*")))
    host_hdr = max(os.path.getmtime(p) for p in glob.glob(os.path.join(host, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h")))
    jobsl = []
    for path in sorted(glob.glob(os.path.join(REFERENCE, "src", "**", "*.cpp"), recursive=True)):
        rel = os.path.relpath(path, os.path.join(REFERENCE, "src"))
        if rel.startswith("analytics"):
            continue  # needs Boost
        jobsl.append((path, os.path.join(objdir, "ref_" + rel.replace("/", "_") + ".o"), ref_flags, shim_time))
    jobsl.append((os.path.join(shim, "gmsh_shim.cpp"), os.path.join(objdir, "gmsh_shim.o"), own_flags, max(shim_time, host_hdr)))
    for h in HOST_SOURCES:
        jobsl.append((os.path.join(host, h), os.path.join(objdir, "host_" + h + ".o"), own_flags, host_hdr))
    jobsl.append((os.path.join(HERE, "ref_assemble.cpp"), os.path.join(objdir, "ref_assemble.o"),
                  ref_flags + ["-I" + HERE], max(shim_time, host_hdr)))
    binding = os.path.join(ROOT, "fem-g_gb300", "binding")
    bind_time = max([host_hdr] + [os.path.getmtime(p) for p in glob.glob(os.path.join(binding, "*.h"))])
    jobsl.append((os.path.join(HERE, "ref_assemble.cpp"), os.path.join(objdir, "ref_dropin.o"),
                  ref_flags + ["-I" + HERE, "-I" + binding, "-I" + os.path.join(ROOT, "include"), "-DFEMG_DROPIN"],
                  max(shim_time, bind_time)))
    jobsl.append((os.path.join(HERE, "fg_record.cpp"), os.path.join(objdir, "fg_record.o"), own_flags, host_hdr))
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(lambda j: _compile_obj(*j), jobsl))
    oracle_obj = os.path.join(objdir, "oracle.o")
    src = os.path.join(HERE, "oracle.c")
    if not os.path.exists(oracle_obj) or os.path.getmtime(oracle_obj) < os.path.getmtime(src):
        _run(["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-c", src, "-o", oracle_obj])
    common = [o for o in objs if not o.endswith(("ref_assemble.o", "ref_dropin.o", "fg_record.o"))]
    for exe, own in ((REF_EXE, ["ref_assemble.o"]), (DROPIN_EXE, ["ref_dropin.o", "fg_record.o", "oracle.o"])):
        parts = common + [os.path.join(objdir, o) for o in own]
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(o) for o in parts):
            continue
        _run(["g++", "-fopenmp", "-o", exe] + parts + ["-lm"])
    return REF_EXE


def build():
    build_oracle()
    build_ref()
    build_gmshfem_ref()


if __name__ == "__main__":
    build()
    print(LIB, REF_LIB if os.path.exists(REF_LIB) else "(no reference build)",
          REF_EXE if os.path.exists(REF_EXE) else "(no reference program)")
