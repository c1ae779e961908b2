"""Reference-built checker -- TEST INFRASTRUCTURE ONLY.

Compiles the MPT reference's own headers through ref_driver.cpp against the
project-written nigh/Eigen stand-ins in shim/, together with the oracle, into
oracle/_ref/libref.so.  The headers come from MPT_REFERENCE_SRC when that is
set, else from the git-ignored copy that oracle/ref/stage.py writes into
oracle/_ref/src (the copy travels with oracle/_ref to hosts without a
reference tree, so the checker builds there too).  The tests that use it skip
where neither exists.  Recipe (what build_if_available() runs):

  gcc -O2 -ffp-contract=off -fPIC -c oracle/oracle.c -o oracle/_ref/oracle.o
  g++ -O2 -ffp-contract=off -std=c++17 -DNDEBUG -DMPT_LOG_LEVEL=WARN -Wno-attributes -fPIC -shared -fopenmp \
      -I oracle/ref/shim -I <reference src> oracle/ref/ref_driver.cpp \
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
REFERENCE_SRC = os.environ.get("MPT_REFERENCE_SRC") or os.path.join(OUT, "src")


def available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_SRC, "mpt"))


def build_if_available(force: bool = False):
    if not available():
        return None
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(ORACLE, "oracle.c"), os.path.join(ORACLE, "oracle.h")]
    for d, _, files in os.walk(os.path.join(HERE, "shim")):
        srcs += [os.path.join(d, f) for f in files]
    marker = os.path.join(REFERENCE_SRC, "STAGED_FILES")
    if os.path.exists(marker):
        srcs.append(marker)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    obj = os.path.join(OUT, "oracle.o")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-std=c11", "-c",
                           os.path.join(ORACLE, "oracle.c"), "-o", obj])
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-DNDEBUG", "-DMPT_LOG_LEVEL=WARN",
                           "-Wno-attributes", "-fPIC", "-shared",
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
        L.ref_dmv_edges_mt.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_longlong, ctypes.c_double, P, P,
                                       ctypes.c_int]
        L.ref_interpolate.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_double, P]
        L.ref_goal_l2.argtypes = [P, ctypes.c_double, P, P]
        D = ctypes.c_double
        L.ref_stream_graph.restype = ctypes.c_int
        L.ref_stream_graph.argtypes = [ctypes.c_int, P, P, P, P, P, P, P, ctypes.c_longlong, P, ctypes.c_longlong, P,
                                       P, ctypes.c_longlong, P, P, ctypes.c_longlong, P]
        L.ref_plan_solve.restype = ctypes.c_int
        L.ref_plan_solve.argtypes = [ctypes.c_int, P, P, P, P, P, P, D, D, D, D, ctypes.c_int, ctypes.c_ulonglong,
                                     ctypes.c_int, D, P, ctypes.c_int, P, P, P, P]
        _lib = L
    return _lib


PLANNERS = {"prrt": 0, "prrt_star": 1, "pprm": 2}


def dmv_edges(desc: dict, a, b, step: float, threads: int = 0):
    """The reference's DiscreteMotionValidator (discrete_motion_validator.hpp:
    71-130) over the oracle's valid(), per edge on `threads` OpenMP threads
    (0 = all): (booleans uint8 [n], valid() calls int64 [n]).  Grid (L2, 2-D),
    planar arm (SO(2)^10) and SE(3) (weights 2/1, the reference's slerp with
    glibc acos/sin) scenes."""
    import numpy as np

    from oracle import _ptr, make_scene

    L = lib()
    sc, keep = make_scene(desc)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = a.shape[0]
    out = np.empty(n, np.uint8)
    cnt = np.empty(n, np.int64)
    r = L.ref_dmv_edges_mt(ctypes.byref(sc), int(desc["metric"]), int(desc["dim"]), _ptr(a), _ptr(b), n, float(step),
                           _ptr(out), _ptr(cnt), int(threads))
    if r != 0:
        raise ValueError("no reference DMV instantiation for metric %s dim %s" % (desc["metric"], desc["dim"]))
    return out, cnt


def plan_solve(desc: dict, seed: int, algo: str = "prrt", threads: int = 1, time_limit_s: float = 30.0,
               goal_bias: float = 0.01, path_cap: int = 100000):
    """One of the reference's own planners -- PRRT (src/mpt/prrt.hpp), PRRT*
    with k-nearest rewiring (src/mpt/prrt_star.hpp) or PPRM (src/mpt/pprm.hpp)
    -- on a scene dict of mpt_gb300.scenes (grid, planar arm or rigid mesh):
    the oracle's valid(), the reference's DMV (or the joint-step edge check of
    arm scenes) as link(), GoalState, setRange(range) and setGoalBias (PRRT and
    PRRT*), uniform samples in [lo, hi] (uniform rotations for SE(3)), the goal
    added with addGoal (PPRM).  Until the first solution or the time limit;
    threads 1 runs the single_threaded variant, 0 the OpenMP worker pool.

    Returns dict(solved, path [m][D], nodes, solve_s, cost)."""
    import numpy as np

    from oracle import _ptr, make_scene, make_space

    L = lib()
    sc, keep = make_scene(desc)
    sp = make_space(int(desc["metric"]), int(desc["dim"]), desc.get("weights", (1.0, 1.0)))
    D = int(desc["dim"])
    arrs = [np.ascontiguousarray(desc[k], dtype=np.float64) for k in ("lo", "hi", "start", "goal")]
    path = np.empty((path_cap, D), dtype=np.float64)
    plen = ctypes.c_int(0)
    nodes = ctypes.c_longlong(0)
    secs = ctypes.c_double(0)
    cost = ctypes.c_double(0)
    r = L.ref_plan_solve(PLANNERS[algo], ctypes.byref(sc), ctypes.byref(sp), *[_ptr(a) for a in arrs],
                         float(desc["goal_radius"]), float(desc["range"]), float(goal_bias), float(desc["edge_step"]),
                         int(desc["resolution"]), int(seed), int(threads), float(time_limit_s), _ptr(path), path_cap,
                         ctypes.byref(plen), ctypes.byref(nodes), ctypes.byref(secs), ctypes.byref(cost))
    if r < 0:
        raise ValueError("no reference planner instantiation for metric %s dim %d" % (desc["metric"], D))
    return {"solved": bool(r), "path": path[:min(plen.value, path_cap)].copy(), "nodes": nodes.value,
            "solve_s": secs.value, "cost": cost.value}


def stream_graph(desc: dict, params: dict, algo: str, nsamples: int, vcap: int = 1 << 20, ecap: int = 1 << 22):
    """The reference's own PRRT, PRRT* or PPRM, single-threaded, fed nsamples
    states of the planners' sample stream (params["seed"], wavefront size
    params["wavefront"]) instead of its RNG: PRRT and PRRT* from the scene's
    start with setRange(params["range"]) and no goal bias; PPRM with the start and the goal
    added first.  The graph through visitGraph: (vertex states [nv][D], edges
    [ne][2][D] as (from, to) state pairs -- PRRT node -> parent, PPRM every edge
    from both ends, path [m][D]) where path is PPRM's solution() when solved
    (empty otherwise and for PRRT / PRRT*)."""
    import numpy as np

    from oracle import PlanParams, _ptr, make_scene, make_space

    L = lib()
    sc, keep = make_scene(desc)
    sp = make_space(int(desc["metric"]), int(desc["dim"]), desc.get("weights", (1.0, 1.0)))
    pp = PlanParams()
    for k in ("range", "goal_bias", "goal_radius", "edge_step"):
        setattr(pp, k, float(params[k]))
    pp.resolution = int(params["resolution"])
    pp.wavefront = int(params["wavefront"])
    pp.seed = int(params["seed"])
    pp.max_nodes = int(params["max_nodes"])
    D = int(desc["dim"])
    arrs = [np.ascontiguousarray(desc[k], dtype=np.float64) for k in ("lo", "hi", "start", "goal")]
    v = np.empty((vcap, D), dtype=np.float64)
    e = np.empty((ecap, 2, D), dtype=np.float64)
    nv = ctypes.c_longlong(0)
    ne = ctypes.c_longlong(0)
    pcap = 1 << 16
    path = np.empty((pcap, D), dtype=np.float64)
    plen = ctypes.c_longlong(0)
    r = L.ref_stream_graph(PLANNERS[algo], ctypes.byref(sc), ctypes.byref(sp), ctypes.byref(pp),
                           *[_ptr(a) for a in arrs], int(nsamples), _ptr(v), vcap, ctypes.byref(nv), _ptr(e), ecap,
                           ctypes.byref(ne), _ptr(path), pcap, ctypes.byref(plen))
    if r == -1:
        raise ValueError("no reference stream instantiation for %s on metric %s dim %d" % (algo, desc["metric"], D))
    if r == -2:
        raise ValueError("vcap/ecap too small (%d vertices, %d edges)" % (nv.value, ne.value))
    return v[:nv.value].copy(), e[:ne.value].copy(), path[:plen.value].copy()
