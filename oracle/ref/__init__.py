"""Reference-built checker -- TEST INFRASTRUCTURE ONLY.

Compiles the MPT reference's own headers (from the reference source tree,
read in place; nothing is copied) through ref_driver.cpp against the
project-written nigh/Eigen stand-ins in shim/, together with the oracle, into
oracle/_ref/libref.so.  Only possible where the reference sources exist; the
tests that use it skip otherwise.  Recipe (what build() runs):

  gcc -O2 -ffp-contract=off -fPIC -c oracle/oracle.c -o oracle/_ref/oracle.o
  g++ -O2 -ffp-contract=off -std=c++17 -DNDEBUG -fPIC -shared \
      -I oracle/ref/shim -I <reference>/src oracle/ref/ref_driver.cpp \
      oracle/_ref/oracle.o -o oracle/_ref/libref.so
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libref.so")
REFERENCE_SRC = os.environ.get("MPT_REFERENCE_SRC", "/root/reference/src")


def available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_SRC, "mpt"))


def build_if_available(force: bool = False):
    if not available():
        return None
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(ORACLE, "oracle.c"), os.path.join(ORACLE, "oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    obj = os.path.join(OUT, "oracle.o")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-std=c11", "-c",
                           os.path.join(ORACLE, "oracle.c"), "-o", obj])
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-DNDEBUG", "-fPIC", "-shared",
                           "-fopenmp", "-I", os.path.join(HERE, "shim"), "-I", REFERENCE_SRC,
                           os.path.join(HERE, "ref_driver.cpp"), obj, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_if_available()
        if path is None:
            raise FileNotFoundError("reference sources not present")
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.ref_dmv_edges.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_longlong, ctypes.c_double, P, P]
        L.ref_interpolate.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_double, P]
        L.ref_goal_l2.argtypes = [P, ctypes.c_double, P, P]
        _lib = L
    return _lib
