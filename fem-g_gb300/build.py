"""Build the in-tree shared library libfemg.so (CUDA kernels for sm_103a, the
C ABI and the host-side mirror of the reference interface), and
libfemg_host.so: the host mirror alone (problem set-up and pre(), no CUDA),
which the CPU baseline loads so that its process never maps the GPU library.

Every translation unit is compiled in parallel into ``_build/`` next to this
file; nothing is installed. ``build()`` is idempotent: a unit is recompiled
only when its source or a header is newer than its object.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfemg.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = ["csrc/plan.cu", "csrc/assemble_fp64.cu", "csrc/assemble_fp64f.cu", "csrc/assemble_mixed.cu", "csrc/gather.cu", "csrc/assemble_static.cu", "csrc/multi_freq.cu", "csrc/batch.cu", "csrc/pattern.cu", "csrc/numbering.cu", "csrc/fused.cu"]
HOST_ONLY_SOURCES = ["host/errors.cpp", "host/mesh.cpp", "host/refelem.cpp", "host/dofs.cpp", "host/formulation.cpp",
                     "host/problems.cpp"]
HOST_SOURCES = HOST_ONLY_SOURCES + ["host/problem_assemble.cpp"]
HEADERS = ["csrc/common.cuh", "csrc/tc_ptx.cuh", "host/mesh.h", "host/refelem.h", "host/dofs.h", "host/formulation.h", "host/problem_internal.h"]
HOST_LIB = os.path.join(BUILD, "libfemg_host.so")


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _newest_header():
    paths = [os.path.join(HERE, h) for h in HEADERS]
    paths += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, hdr_time):
    path = os.path.join(HERE, src)
    obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), hdr_time):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off",
               "-I" + os.path.join(_cuda_home(), "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def _cuda_home():
    nv = _nvcc()
    return os.path.dirname(os.path.dirname(os.path.realpath(nv)))


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdr = _newest_header()
    srcs = CUDA_SOURCES + HOST_SOURCES
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [_nvcc(), ARCH, "-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


def build_host(verbose=False):
    """libfemg_host.so: the host mirror's problem set-up without any GPU code."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = _newest_header()
    objs = [_compile(s, hdr) for s in HOST_ONLY_SOURCES]
    if os.path.exists(HOST_LIB) and os.path.getmtime(HOST_LIB) >= max(os.path.getmtime(o) for o in objs):
        return HOST_LIB
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-o", HOST_LIB] + objs + ["-Wl,--no-undefined"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", HOST_LIB)
    return HOST_LIB


if __name__ == "__main__":
    build(verbose=True)
    build_host(verbose=True)
