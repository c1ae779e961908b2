"""The C++ drop-in header (include/mptg_planner.hpp): compiles against the C
ABI on the CPU; its host logic runs on the CPU against a scripted stand-in of
the planner calls (tests/cpp/fake_mptg_planner.cpp: forwarded parameters,
solve loops, exceptions, path and graph reads), plainly and under
AddressSanitizer + UndefinedBehaviorSanitizer; on the GPU the program solves a
grid and checks the reference acceptance conditions
(test/planner_integration_test.hpp:219-291)."""
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


@pytest.mark.parametrize("sanitize", [False, True])
def test_cpp_header_host_logic(tmp_path, sanitize):
    exe = str(tmp_path / "planner_header_check")
    cmd = ["g++", "-std=c++17", "-O1" if sanitize else "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "planner_header_check.cpp"),
           os.path.join(ROOT, "tests", "cpp", "fake_mptg_planner.cpp"), "-o", exe]
    if sanitize:
        cmd[4:4] = ["-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"]
    subprocess.check_call(cmd)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "planner header OK" in r.stdout


@pytest.mark.gpu
def test_cpp_planner_solves():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "planner_api")
        _compile(exe)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "C++ Planner OK" in r.stdout
