"""The C++ drop-in header (include/mptg_planner.hpp): compiles against the C
ABI on the CPU; on the GPU the program solves a grid and checks the reference
acceptance conditions (test/planner_integration_test.hpp:219-291)."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(out):
    from mpt_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "planner_api.cpp"), "-L", libdir, "-lmptg",
           "-Wl,-rpath," + libdir, "-o", out]
    subprocess.check_call(cmd)


def test_cpp_header_compiles():
    with tempfile.TemporaryDirectory() as td:
        _compile(os.path.join(td, "planner_api"))


@pytest.mark.gpu
def test_cpp_planner_solves():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "planner_api")
        _compile(exe)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "C++ Planner OK" in r.stdout
