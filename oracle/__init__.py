"""CPU oracle for the MPT planner hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference legs may import it; the ``mpt_gb300``
product never imports, links or calls anything here.

``oracle.c`` restates the reference algorithms in plain C (each function cites
the reference file:line it follows) and is built into ``oracle/_build/liborc.so``
with ``-O2 -ffp-contract=off -fopenmp``.  ``ref/`` builds the reference's own
DiscreteMotionValidator / GoalState headers against a project-written nigh
stand-in into ``oracle/_ref/`` (only where the reference sources are present).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liborc.so")
ROOT = os.path.dirname(HERE)

L2, SO2, SO3, SE3, L1 = 0, 1, 2, 3, 4


# MPTG_ORACLE_SANITIZE=1 selects a second build with AddressSanitizer and
# UndefinedBehaviorSanitizer (aborting on the first report), for running the
# oracle's tests under the sanitizers; the process must preload libasan.
SANITIZE = bool(os.environ.get("MPTG_ORACLE_SANITIZE"))
SANITIZE_FLAGS = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer", "-g"]
if SANITIZE:
    LIB_PATH = os.path.join(BUILD_DIR, "liborc_san.so")


def build(force: bool = False) -> str:
    """Compile oracle.c into _build/liborc.so (gcc, OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "oracle.c")
    hdrs = [os.path.join(HERE, "oracle.h"), os.path.join(ROOT, "include", "mptg_detmath.h")]
    if not force and os.path.exists(LIB_PATH):
        mt = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(p) <= mt for p in [src] + hdrs):
            return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=c11", "-o", tmp, src, "-lm"]
    if SANITIZE:
        cmd[1:1] = SANITIZE_FLAGS
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Space(ctypes.Structure):
    _fields_ = [("metric", ctypes.c_int), ("dim", ctypes.c_int), ("w", ctypes.c_double * 2)]


class Scene(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("grid", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("nlinks", ctypes.c_int), ("link_len", ctypes.c_void_p), ("ndiscs", ctypes.c_int),
        ("discs", ctypes.c_void_p), ("robot_radius", ctypes.c_double), ("self_collision", ctypes.c_int),
        ("nrobot", ctypes.c_int64), ("robot_tris", ctypes.c_void_p), ("nenv", ctypes.c_int64),
        ("env_tris", ctypes.c_void_p),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.orc_distance.restype = ctypes.c_double
        L.orc_distance.argtypes = [P, P, P]
        L.orc_interpolate.argtypes = [P, P, P, ctypes.c_double, P]
        L.orc_so2_ccw.restype = ctypes.c_double
        L.orc_so2_ccw.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_so2_bound.restype = ctypes.c_double
        L.orc_so2_bound.argtypes = [ctypes.c_double]
        L.orc_nn_brute.argtypes = [P, P, ctypes.c_int64, P, ctypes.c_int64, P, P, ctypes.c_int]
        L.orc_knn_brute.argtypes = [P, P, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_kd_build.restype = P
        L.orc_kd_build.argtypes = [P, P, ctypes.c_int64, ctypes.c_int]
        L.orc_kd_nearest.argtypes = [P, P, ctypes.c_int64, P, P, ctypes.c_int, P]
        L.orc_kd_free.argtypes = [P]
        L.orc_valid_states.argtypes = [P, P, P, ctypes.c_int64, P, ctypes.c_int]
        L.orc_valid_edges.argtypes = [P, P, P, P, ctypes.c_int64, ctypes.c_double, ctypes.c_int, P, P,
                                      ctypes.c_int]
        L.orc_tri_tri.restype = ctypes.c_int
        L.orc_tri_tri.argtypes = [P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_space(metric: int, dim: int, w=(1.0, 1.0)) -> Space:
    s = Space()
    s.metric = metric
    s.dim = dim
    s.w[0] = float(w[0])
    s.w[1] = float(w[1])
    return s


def distance(space: Space, a, b) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().orc_distance(ctypes.byref(space), _ptr(a), _ptr(b))


def interpolate(space: Space, a, b, t: float) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(space.dim, dtype=np.float64)
    lib().orc_interpolate(ctypes.byref(space), _ptr(a), _ptr(b), float(t), _ptr(out))
    return out


def nn_brute(space: Space, pts: np.ndarray, q: np.ndarray, nthreads: int = 0):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    nq = q.shape[0]
    idx = np.empty(nq, dtype=np.int32)
    dist = np.empty(nq, dtype=np.float64)
    lib().orc_nn_brute(ctypes.byref(space), _ptr(pts), pts.shape[0], _ptr(q), nq, _ptr(idx), _ptr(dist),
                       nthreads or os.cpu_count())
    return idx, dist


def knn_brute(space: Space, pts: np.ndarray, q: np.ndarray, k: int, nthreads: int = 0):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    nq = q.shape[0]
    idx = np.empty((nq, k), dtype=np.int32)
    dist = np.empty((nq, k), dtype=np.float64)
    lib().orc_knn_brute(ctypes.byref(space), _ptr(pts), pts.shape[0], _ptr(q), nq, k, _ptr(idx), _ptr(dist),
                        nthreads or os.cpu_count())
    return idx, dist


class KDTree:
    """The CPU kd-tree that stands in for nigh's KDTreeBatch in the baseline."""

    def __init__(self, space: Space, pts: np.ndarray, leaf: int = 8):
        self.space = space
        self.pts = np.ascontiguousarray(pts, dtype=np.float64)
        self.h = lib().orc_kd_build(ctypes.byref(space), _ptr(self.pts), self.pts.shape[0], leaf)

    def nearest(self, q: np.ndarray, nthreads: int = 0):
        q = np.ascontiguousarray(q, dtype=np.float64)
        nq = q.shape[0]
        idx = np.empty(nq, dtype=np.int32)
        dist = np.empty(nq, dtype=np.float64)
        ev = ctypes.c_int64(0)
        lib().orc_kd_nearest(self.h, _ptr(q), nq, _ptr(idx), _ptr(dist), nthreads or os.cpu_count(),
                             ctypes.byref(ev))
        self.last_evals = ev.value
        return idx, dist

    def __del__(self):
        try:
            if self.h:
                lib().orc_kd_free(self.h)
                self.h = None
        except Exception:
            pass


def make_scene(desc: dict):
    """Build an oracle Scene from a scene dict produced by mpt_gb300.scenes.

    Returns (Scene, keepalive) -- keep the second value alive while using it."""
    sc = Scene()
    keep = []
    kind = desc["kind"]
    if kind == "grid":
        g = np.ascontiguousarray(desc["grid"], dtype=np.uint8)
        keep.append(g)
        sc.kind = 0
        sc.grid = g.ctypes.data
        sc.height, sc.width = g.shape
    elif kind == "arm":
        lens = np.ascontiguousarray(desc["link_len"], dtype=np.float64)
        discs = np.ascontiguousarray(desc["discs"], dtype=np.float64)
        keep += [lens, discs]
        sc.kind = 1
        sc.nlinks = lens.shape[0]
        sc.link_len = lens.ctypes.data
        sc.ndiscs = discs.shape[0]
        sc.discs = discs.ctypes.data
        sc.robot_radius = float(desc.get("robot_radius", 0.0))
        sc.self_collision = int(desc.get("self_collision", 1))
    elif kind == "mesh":
        rt = np.ascontiguousarray(desc["robot_tris"], dtype=np.float64)
        et = np.ascontiguousarray(desc["env_tris"], dtype=np.float64)
        keep += [rt, et]
        sc.kind = 2
        sc.nrobot = rt.shape[0]
        sc.robot_tris = rt.ctypes.data
        sc.nenv = et.shape[0]
        sc.env_tris = et.ctypes.data
    else:
        raise ValueError(kind)
    return sc, keep


def valid_states(desc: dict, space: Space, q: np.ndarray, nthreads: int = 0) -> np.ndarray:
    sc, keep = make_scene(desc)
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = np.empty(q.shape[0], dtype=np.uint8)
    lib().orc_valid_states(ctypes.byref(sc), ctypes.byref(space), _ptr(q), q.shape[0], _ptr(out),
                           nthreads or os.cpu_count())
    return out


def valid_edges(desc: dict, space: Space, a: np.ndarray, b: np.ndarray, step: float, resolution: int = 0,
                nthreads: int = 0):
    sc, keep = make_scene(desc)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(a.shape[0], dtype=np.uint8)
    ns = ctypes.c_int64(0)
    lib().orc_valid_edges(ctypes.byref(sc), ctypes.byref(space), _ptr(a), _ptr(b), a.shape[0], float(step),
                          int(resolution), _ptr(out), ctypes.byref(ns), nthreads or os.cpu_count())
    return out, ns.value


class PlanParams(ctypes.Structure):
    _fields_ = [("range", ctypes.c_double), ("goal_bias", ctypes.c_double), ("goal_radius", ctypes.c_double),
                ("edge_step", ctypes.c_double), ("resolution", ctypes.c_int), ("wavefront", ctypes.c_int),
                ("seed", ctypes.c_uint64), ("max_nodes", ctypes.c_int64)]


def plan(desc: dict, space: Space, params: dict, lo, hi, start, goal, max_waves: int, stop_when_solved: bool,
         nthreads: int = 0):
    """Replay of the wavefront planner: (states, parents, goal ids)."""
    L = lib()
    if not getattr(L, "_plan_sig", False):
        P = ctypes.c_void_p
        L.orc_plan.restype = ctypes.c_int64
        L.orc_plan.argtypes = [P, P, P, P, P, P, P, ctypes.c_int, ctypes.c_int, P, P, P, P, ctypes.c_int]
        L.orc_uniform.restype = ctypes.c_double
        L.orc_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        L._plan_sig = True
    sc, keep = make_scene(desc)
    pp = PlanParams()
    for k in ("range", "goal_bias", "goal_radius", "edge_step"):
        setattr(pp, k, float(params[k]))
    pp.resolution = int(params["resolution"])
    pp.wavefront = int(params["wavefront"])
    pp.seed = int(params["seed"])
    pp.max_nodes = int(params["max_nodes"])
    D = space.dim
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    start = np.ascontiguousarray(start, dtype=np.float64)
    g = None if goal is None else np.ascontiguousarray(goal, dtype=np.float64)
    states = np.empty((pp.max_nodes, D), dtype=np.float64)
    parents = np.empty(pp.max_nodes, dtype=np.int32)
    goals = np.empty(pp.max_nodes, dtype=np.int32)
    ng = ctypes.c_int64(0)
    n = L.orc_plan(ctypes.byref(sc), ctypes.byref(space), ctypes.byref(pp), _ptr(lo), _ptr(hi), _ptr(start),
                   None if g is None else _ptr(g), int(max_waves), int(stop_when_solved), _ptr(states), _ptr(parents),
                   _ptr(goals), ctypes.byref(ng), nthreads or os.cpu_count())
    return states[:n].copy(), parents[:n].copy(), goals[:ng.value].copy()


def set_plan_nn(mode):
    """Nearest-neighbour search of the planner replays: "brute" (or False; the
    definition, the default), "kdtree" (or True; the exact kd-tree, same
    answers) or "auto" (the kd-tree up to 7 dimensions), for CPU timing runs."""
    code = {False: 0, True: 1, "brute": 0, "kdtree": 1, "auto": 2}[mode]
    L = lib()
    L.orc_set_plan_nn.restype = None
    L.orc_set_plan_nn.argtypes = [ctypes.c_int]
    L.orc_set_plan_nn(code)


def plan_star(desc: dict, space: Space, params: dict, lo, hi, start, goal, max_waves: int, rewire_factor: float = 1.1,
              nthreads: int = 0):
    """Replay of the wavefront PRRT* planner: (states, parents, costs, goal ids, rewires)."""
    L = lib()
    if not getattr(L, "_plan_star_sig", False):
        P = ctypes.c_void_p
        L.orc_plan_star.restype = ctypes.c_int64
        L.orc_plan_star.argtypes = [P, P, P, P, P, P, P, ctypes.c_int, ctypes.c_double, P, P, P, P, P, P,
                                    ctypes.c_int]
        L._plan_star_sig = True
    sc, keep = make_scene(desc)
    pp = PlanParams()
    for k in ("range", "goal_bias", "goal_radius", "edge_step"):
        setattr(pp, k, float(params[k]))
    pp.resolution = int(params["resolution"])
    pp.wavefront = int(params["wavefront"])
    pp.seed = int(params["seed"])
    pp.max_nodes = int(params["max_nodes"])
    D = space.dim
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    start = np.ascontiguousarray(start, dtype=np.float64)
    g = None if goal is None else np.ascontiguousarray(goal, dtype=np.float64)
    states = np.empty((pp.max_nodes, D), dtype=np.float64)
    parents = np.empty(pp.max_nodes, dtype=np.int32)
    costs = np.empty(pp.max_nodes, dtype=np.float64)
    goals = np.empty(pp.max_nodes, dtype=np.int32)
    ng = ctypes.c_int64(0)
    nrw = ctypes.c_int64(0)
    n = L.orc_plan_star(ctypes.byref(sc), ctypes.byref(space), ctypes.byref(pp), _ptr(lo), _ptr(hi), _ptr(start),
                        None if g is None else _ptr(g), int(max_waves), float(rewire_factor), _ptr(states),
                        _ptr(parents), _ptr(costs), _ptr(goals), ctypes.byref(ng), ctypes.byref(nrw),
                        nthreads or os.cpu_count())
    del keep
    return states[:n].copy(), parents[:n].copy(), costs[:n].copy(), goals[:ng.value].copy(), nrw.value


def prm(desc: dict, space: Space, params: dict, lo, hi, goal, starts, goals, max_waves: int,
        stop_when_solved: bool = False, edge_cap: int = 1 << 22):
    """Replay of the wavefront PPRM roadmap: dict(states, flags, edges (from, to,
    dist) sorted by (from, to), stats[8], path node ids, cost)."""
    L = lib()
    if not getattr(L, "_prm_sig", False):
        P = ctypes.c_void_p
        L.orc_prm.restype = ctypes.c_int64
        L.orc_prm.argtypes = [P, P, P, P, P, P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P,
                              P, P, P, P, ctypes.c_int64, P]
        L.orc_prm_dijkstra.restype = ctypes.c_int64
        L.orc_prm_dijkstra.argtypes = [ctypes.c_int64, P, ctypes.c_int64, P, P, P, P, P]
        L.orc_prm_k.restype = ctypes.c_int
        L.orc_prm_k.argtypes = [ctypes.c_int64, ctypes.c_int]
        L._prm_sig = True
    sc, keep = make_scene(desc)
    pp = PlanParams()
    pp.range = 0.0
    pp.goal_bias = 0.0
    pp.goal_radius = float(params["goal_radius"])
    pp.edge_step = float(params["edge_step"])
    pp.resolution = int(params["resolution"])
    pp.wavefront = int(params["wavefront"])
    pp.seed = int(params["seed"])
    pp.max_nodes = int(params["max_nodes"])
    D = space.dim
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    lo, hi = f64(lo), f64(hi)
    g = None if goal is None else f64(goal)
    S = f64(starts).reshape(-1, D)
    G = f64(goals).reshape(-1, D)
    states = np.empty((pp.max_nodes, D), dtype=np.float64)
    flags = np.empty(pp.max_nodes, dtype=np.uint8)
    ef = np.empty(edge_cap, dtype=np.int32)
    et = np.empty(edge_cap, dtype=np.int32)
    ed = np.empty(edge_cap, dtype=np.float64)
    ne = ctypes.c_int64(0)
    stats = np.zeros(8, dtype=np.int64)
    n = L.orc_prm(ctypes.byref(sc), ctypes.byref(space), ctypes.byref(pp), _ptr(lo), _ptr(hi),
                  None if g is None else _ptr(g), _ptr(S), len(S), _ptr(G), len(G), int(max_waves),
                  int(stop_when_solved), _ptr(states), _ptr(flags), ctypes.byref(ne), _ptr(ef), _ptr(et), _ptr(ed),
                  edge_cap, _ptr(stats))
    del keep
    m = ne.value
    assert m <= edge_cap, "edge_cap too small"
    order = np.lexsort((et[:m], ef[:m]))
    ef, et, ed = ef[:m][order].copy(), et[:m][order].copy(), ed[:m][order].copy()
    path = np.empty(max(n, 1), dtype=np.int32)
    cost = ctypes.c_double(0.0)
    plen = L.orc_prm_dijkstra(n, _ptr(flags), m, _ptr(ef), _ptr(et), _ptr(ed), _ptr(path), ctypes.byref(cost))
    return {"states": states[:n].copy(), "flags": flags[:n].copy(), "edges": (ef, et, ed), "stats": stats,
            "path": path[:plen].copy(), "cost": cost.value}


def prm_k(n: int, dim: int) -> int:
    """k of the PPRM neighbourhood for a roadmap of n nodes."""
    L = lib()
    L.orc_prm_k.restype = ctypes.c_int
    L.orc_prm_k.argtypes = [ctypes.c_int64, ctypes.c_int]
    return int(L.orc_prm_k(int(n), int(dim)))


def uniform(seed: int, i: int, w: int, j: int) -> float:
    lib()
    if not getattr(_lib, "_plan_sig", False):
        plan  # signatures are set on first plan(); set the one needed here
        _lib.orc_uniform.restype = ctypes.c_double
        _lib.orc_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
    return _lib.orc_uniform(seed, i, w, j)


def tri_tri(t1, t2) -> bool:
    t1 = np.ascontiguousarray(t1, dtype=np.float64).reshape(9)
    t2 = np.ascontiguousarray(t2, dtype=np.float64).reshape(9)
    return bool(lib().orc_tri_tri(_ptr(t1), _ptr(t2)))


def sample_states(space: Space, seed: int, lo, hi, n: int, wavefront: int = 4096) -> np.ndarray:
    """The first n states of the planners' sample stream: state c is sample
    c % wavefront of wavefront c / wavefront (orc_sample_state, no goal bias)."""
    L = lib()
    if not getattr(L, "_sample_sig", False):
        P = ctypes.c_void_p
        L.orc_sample_state.argtypes = [P, P, P, P, ctypes.c_uint32, ctypes.c_uint32, P]
        L._sample_sig = True
    pp = PlanParams()
    pp.wavefront = int(wavefront)
    pp.seed = int(seed)
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    out = np.empty((n, space.dim), dtype=np.float64)
    W = int(wavefront)
    for c in range(n):
        L.orc_sample_state(ctypes.byref(space), ctypes.byref(pp), _ptr(lo), _ptr(hi), c % W, c // W,
                           out[c:].ctypes.data_as(ctypes.c_void_p))
    return out


def prm_dijkstra(n: int, flags, efrom, eto, edist):
    """Shortest roadmap path (orc_prm_dijkstra) over undirected edges from any
    node with flag bit 1 to the nearest node with flag bit 2: (node ids, cost)."""
    L = lib()
    P = ctypes.c_void_p
    L.orc_prm_dijkstra.restype = ctypes.c_int64
    L.orc_prm_dijkstra.argtypes = [ctypes.c_int64, P, ctypes.c_int64, P, P, P, P, P]
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    ef = np.ascontiguousarray(efrom, dtype=np.int32)
    et = np.ascontiguousarray(eto, dtype=np.int32)
    ed = np.ascontiguousarray(edist, dtype=np.float64)
    path = np.empty(max(int(n), 1), dtype=np.int32)
    cost = ctypes.c_double(0.0)
    m = L.orc_prm_dijkstra(int(n), _ptr(flags), len(ef), _ptr(ef), _ptr(et), _ptr(ed), _ptr(path), ctypes.byref(cost))
    return path[:m].copy(), cost.value
