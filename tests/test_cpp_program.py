"""The C++ GmshFEM-style program tests/cpp/formulation_test.cpp, linked
against libfemg.so: pre() checks on the CPU, the assembled system on a GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "formulation_test.cpp")


@pytest.fixture(scope="module")
def program(femg, tmp_path_factory):
    lib_dir = os.path.dirname(femg.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("cpp") / "formulation_test")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", SRC, "-I" + os.path.join(ROOT, "include"), "-L" + lib_dir,
           "-lfemg", "-Wl,-rpath," + lib_dir, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_program_pre_on_cpu(program):
    r = subprocess.run([program, "--cpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_program_assembles_on_gpu(program, cuda):
    r = subprocess.run([program], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
