"""The nigh adapter (include/mptg_nigh.hpp) under the reference's own PRRT,
PRRT* and PPRM, compiled from the reference headers (staged into
oracle/_ref/src; skipped where they are absent).  On the CPU the program runs
against the CPU stand-in of the C ABI's nearest-neighbour calls
(tests/cpp/fake_mptg_nn.cpp), which checks the adapter's bookkeeping, and a
second build links it against the real libmptg; on the GPU that second build
runs, with the device kd-tree answering every query."""
import os
import subprocess

import pytest

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("reference sources not present", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# -ffp-contract=off: the brute-force distances the program checks against must
# round like the library's (g++ contracts a*b+c into FMA on Arm by default)
FLAGS = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-fopenmp", "-DNDEBUG", "-DMPT_LOG_LEVEL=WARN", "-Wno-attributes",
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


@pytest.mark.gpu
def test_nigh_adapter_on_gpu(tmp_path):
    """MPT's own PRRT (single-threaded and with its OpenMP workers), PRRT* and
    PPRM over PRRT<mpt_gb300::GpuKDTree> and friends, with every nearest and
    k-nearest call answered by the device kd-tree of the real libmptg: the
    container checks against brute force and the planners' acceptance rules
    (test/planner_integration_test.hpp:219-291) pass."""
    from mpt_gb300 import build
    libdir = os.path.dirname(build.build())
    exe = str(tmp_path / "na_gpu")
    subprocess.check_call(FLAGS + ["-L", libdir, "-lmptg", "-Wl,-rpath," + libdir, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "nigh adapter OK" in r.stdout
    for name in ("PRRT:", "PRRT, OpenMP workers:", "PRRT*:", "PPRM:"):
        assert name in r.stdout


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
