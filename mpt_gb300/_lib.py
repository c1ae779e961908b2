"""ctypes binding of libmptg.so (the C ABI declared in include/mptg.h).

The library is loaded from mpt_gb300/_build/libmptg.so; a missing library is
an error (there is no CPU fallback).  Buffers may be numpy arrays (host) or
CUDA tensors (anything with ``data_ptr()``), passed through as raw pointers.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None

OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "QUEUE_OVERFLOW",
                6: "UNSUPPORTED_METRIC", 7: "CAPACITY", 8: "NO_START", 9: "ALREADY_SOLVING"}


class MptgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, str(status)), msg))
        self.status = status


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("grid", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("nlinks", ctypes.c_int), ("link_len", ctypes.c_void_p), ("ndiscs", ctypes.c_int),
        ("discs", ctypes.c_void_p), ("robot_radius", ctypes.c_double), ("self_collision", ctypes.c_int),
        ("nrobot", ctypes.c_int64), ("robot_tris", ctypes.c_void_p), ("nenv", ctypes.c_int64),
        ("env_tris", ctypes.c_void_p), ("w_rot", ctypes.c_double), ("w_pos", ctypes.c_double),
    ]


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libmptg.so (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libmptg.so is not built (run __graft_entry__.build()); no CPU fallback exists")
    L = ctypes.CDLL(path)
    P, S, I, D = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_double
    St = ctypes.c_int
    sig = {
        "mptg_create": (St, [ctypes.POINTER(P), I]),
        "mptg_destroy": (St, [P]),
        "mptg_last_error": (ctypes.c_char_p, [P]),
        "mptg_kernel_launches": (ctypes.c_uint64, [P]),
        "mptg_tree_create": (St, [P, I, I, P, S, ctypes.POINTER(P)]),
        "mptg_tree_destroy": (St, [P]),
        "mptg_tree_insert": (St, [P, P, S, P]),
        "mptg_tree_size": (St, [P, ctypes.POINTER(S)]),
        "mptg_tree_set_strategy": (St, [P, I]),
        "mptg_tree_states": (St, [P, S, S, P, P]),
        "mptg_nearest": (St, [P, P, S, P, P, P]),
        "mptg_nearest_k": (St, [P, P, S, I, D, P, P, P]),
        "mptg_nearest_linear": (St, [P, P, S, P, P, P]),
        "mptg_tree_counters": (St, [P, P, I]),
        "mptg_scene_create": (St, [P, P, ctypes.POINTER(P)]),
        "mptg_scene_destroy": (St, [P]),
        "mptg_scene_space": (St, [P, P, P, P]),
        "mptg_valid_states": (St, [P, P, S, P, P]),
        "mptg_valid_edges": (St, [P, P, P, S, D, I, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def declared_symbols() -> list[str]:
    """Function names declared in include/mptg.h (parsed from the header)."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mptg.h")
    text = open(hdr).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mptg_[a-z0-9_]+)\s*\(", text)))


def ptr(x):
    """Raw address of a numpy array or a tensor-like object (data_ptr)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(type(x))
