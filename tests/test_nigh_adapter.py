"""CPU: the nigh adapter (include/mptg_nigh.hpp) under the reference's own
PRRT, PRRT* and PPRM, compiled in place (skipped where the reference sources
are absent).  The program runs against the CPU stand-in of the C ABI's
nearest-neighbour calls (tests/cpp/fake_mptg_nn.cpp), which checks the
adapter's bookkeeping; a second build links the same program against the real
libmptg to check the adapter's calls against the ABI it ships with."""
import os
import subprocess

import pytest

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("reference sources not present", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAGS = ["g++", "-std=c++17", "-O2", "-Wall", "-fopenmp", "-DNDEBUG", "-DMPT_LOG_LEVEL=WARN", "-Wno-attributes",
         "-Wno-unused-variable", "-I", os.path.join(ROOT, "include"),
         "-I", os.path.join(ROOT, "oracle", "ref", "shim"), "-I", ref.REFERENCE_SRC,
         os.path.join(ROOT, "tests", "cpp", "nigh_adapter.cpp")]


def test_nigh_adapter_under_reference_planners(tmp_path):
    exe = str(tmp_path / "nigh_adapter")
    subprocess.check_call(FLAGS + [os.path.join(ROOT, "tests", "cpp", "fake_mptg_nn.cpp"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "nigh adapter OK" in r.stdout
    for name in ("PRRT:", "PRRT, OpenMP workers:", "PRRT*:", "PPRM:"):
        assert name in r.stdout


def test_nigh_adapter_links_against_libmptg(tmp_path):
    from mpt_gb300 import build
    libdir = os.path.dirname(build.build())
    subprocess.check_call(FLAGS + ["-L", libdir, "-lmptg", "-Wl,-rpath," + libdir, "-o", str(tmp_path / "na_gpu")])


def test_nigh_adapter_under_sanitizers(tmp_path):
    """The same program built with AddressSanitizer and UndefinedBehaviorSanitizer
    (aborting on the first report): the adapter, the reference planners over it
    and the CPU stand-in stay inside their buffers."""
    exe = str(tmp_path / "nigh_adapter_san")
    try:
        subprocess.check_call(FLAGS + ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                                       "-fno-omit-frame-pointer", "-g",
                                       os.path.join(ROOT, "tests", "cpp", "fake_mptg_nn.cpp"), "-o", exe])
    except subprocess.CalledProcessError:
        pytest.skip("sanitizer runtimes not available to g++")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, ASAN_OPTIONS="detect_leaks=0"))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "nigh adapter OK" in r.stdout and "runtime error" not in r.stderr
