"""CPU: the oracle's own tests again, against a build of oracle.c with
AddressSanitizer and UndefinedBehaviorSanitizer (MPTG_ORACLE_SANITIZE=1,
aborting on the first report), in a child process that preloads the sanitizer
runtimes: the checker itself reads and writes only inside its buffers."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _runtime(name):
    try:
        path = subprocess.check_output(["gcc", "-print-file-name=" + name], text=True).strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_oracle_tests_under_asan_and_ubsan():
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not asan or not ubsan:
        pytest.skip("gcc sanitizer runtimes not installed")
    env = dict(os.environ, LD_PRELOAD=asan + " " + ubsan, ASAN_OPTIONS="detect_leaks=0",
               MPTG_ORACLE_SANITIZE="1")
    files = [os.path.join(ROOT, "tests", f) for f in
             ("test_oracle_kats.py", "test_oracle_planners.py", "test_oracle_prm.py")]
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", *files], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=1200)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-4000:]
    assert "AddressSanitizer" not in out and "runtime error" not in out
    assert os.path.exists(os.path.join(ROOT, "oracle", "_build", "liborc_san.so"))
