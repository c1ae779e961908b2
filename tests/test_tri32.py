"""CPU: the certified FP32 triangle-pair verdicts of the mesh kernels
(mpt_gb300/csrc/tri32.cuh) never disagree with the oracle's FP64 Moller test
(orc_tri_tri), on random pairs with touching, vertex-sharing and 1e-7-offset
cases; compiled twice, with and without FMA contraction (the device code may
be contracted)."""
import os
import platform
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("contract", ["off", "fast"])
def test_fp32_triangle_verdicts_agree_with_fp64(tmp_path, contract):
    obj = str(tmp_path / "oracle.o")
    exe = str(tmp_path / "tri32_check")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-c", os.path.join(ROOT, "oracle", "oracle.c"),
                           "-o", obj])
    flags = ["-ffp-contract=" + contract]
    if contract == "fast" and platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    subprocess.check_call(["g++", "-O2", "-std=c++17"] + flags +
                          [os.path.join(ROOT, "tests", "cpp", "tri32_check.cpp"), obj, "-o", exe, "-fopenmp", "-lm"])
    r = subprocess.run([exe, "400000"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "wrong 0" in r.stdout
