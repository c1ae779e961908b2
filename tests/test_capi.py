"""CPU: the C-ABI library builds, loads without a GPU and exports every
function include/mptg.h declares; error paths that need no GPU."""
import ctypes
import subprocess

import pytest


def test_library_exports_declared_symbols():
    from mpt_gb300 import _lib, build
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = _lib.declared_symbols()
    assert "mptg_nearest" in declared and "mptg_valid_edges" in declared
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.check_output(["nm", "-D", "--defined-only", path], text=True)
    for s in declared:
        assert " " + s + "\n" in out or out.endswith(" " + s), s


def test_null_arguments_rejected_without_gpu():
    import mpt_gb300 as m
    lib = m.load()
    assert lib.mptg_create(None, 0) == 1  # INVALID_ARG
    assert lib.mptg_tree_destroy(None) == 1
    assert lib.mptg_nearest(None, None, 0, None, None, None) == 1
    assert lib.mptg_last_error(None) == b"null context"


def test_create_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import mpt_gb300 as m
    h = ctypes.c_void_p()
    st = m.load().mptg_create(ctypes.byref(h), 0)
    assert st == 3  # CUDA_ERROR: no device
    assert not h.value
