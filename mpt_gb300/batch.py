"""Batched multi-query serving: many independent planning queries over shared
scenes in one call (mptg_plan_batch in include/mptg.h).

The reference serves one query per Planner object
(src/mpt/impl/prrt/prrt.hpp:149-157, one solve per planner); here a batch of
queries runs on host workers that each own a CUDA stream and reuse one planner
per scene, so the wavefronts of different queries overlap on the GPU.  A
query's result is exactly that of a single Planner with the same seed and
parameters.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import Context, Scene, _check, load
from .planner import Scenario, _Params


class _Query(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("start", ctypes.c_void_p), ("goal", ctypes.c_void_p),
                ("goal_radius", ctypes.c_double), ("params", _Params), ("lo", ctypes.c_void_p),
                ("hi", ctypes.c_void_p), ("time_limit_s", ctypes.c_double), ("surrogate", ctypes.c_void_p),
                ("surrogate_threshold", ctypes.c_double), ("surrogate_points", ctypes.c_int),
                ("path", ctypes.c_void_p), ("path_cap", ctypes.c_size_t), ("surrogate_candidates", ctypes.c_int)]


class _Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("solved", ctypes.c_int), ("nodes", ctypes.c_size_t),
                ("wavefronts", ctypes.c_size_t), ("solve_s", ctypes.c_double), ("finish_s", ctypes.c_double),
                ("cost", ctypes.c_double), ("path_len", ctypes.c_size_t)]


def _sig(L):
    if getattr(L, "_batch_sig", False):
        return
    L.mptg_plan_batch.restype = ctypes.c_int
    L.mptg_plan_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Query), ctypes.c_size_t, ctypes.c_int,
                                  ctypes.POINTER(_Result)]
    L.mptg_planner_reset.restype = ctypes.c_int
    L.mptg_planner_reset.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.mptg_tree_clear.restype = ctypes.c_int
    L.mptg_tree_clear.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L._batch_sig = True


@dataclass
class Query:
    """One planning query: a Scenario (scene + goal + bounds + link
    resolution), a start, a seed and a node budget."""
    scenario: Scenario
    start: np.ndarray
    seed: int
    max_nodes: int
    wavefront: int = 4096
    range: float | None = None        # None: the scenario's default steer range
    goal_bias: float = 0.01
    time_limit: float = 0.0           # seconds, <= 0: none
    surrogate: object | None = None   # mpt_gb300.surrogate.Surrogate
    threshold: float = 0.0
    surrogate_points: int = 1         # states scored per candidate edge
    surrogate_candidates: int = 1     # candidate edges per wavefront slot (surrogate-biased sampling)
    path_cap: int = 4096


def plan_batch(ctx: Context, queries: list[Query], concurrency: int = 8) -> list[dict]:
    """Runs every query; returns per query: solved, nodes, wavefronts, solve_s
    (first wavefront to end), finish_s (batch start to end), cost and path."""
    L = load()
    _sig(L)
    scenes = {}
    keep = []
    qs = (_Query * len(queries))()
    paths = []
    for i, q in enumerate(queries):
        sc = q.scenario
        key = id(sc.desc)
        if key not in scenes:
            scenes[key] = Scene(ctx, sc.desc)
        g = scenes[key]
        start = np.ascontiguousarray(q.start, dtype=np.float64)
        goal = np.ascontiguousarray(sc.goal.state, dtype=np.float64)
        lo = np.ascontiguousarray(sc.lo, dtype=np.float64)
        hi = np.ascontiguousarray(sc.hi, dtype=np.float64)
        path = np.empty((q.path_cap, g.dim), dtype=np.float64)
        keep += [start, goal, lo, hi]
        paths.append(path)
        rng = sc.default_range if q.range is None else float(q.range)
        p = qs[i]
        p.scene = g.h.value if isinstance(g.h, ctypes.c_void_p) else g.h
        p.start, p.goal = start.ctypes.data, goal.ctypes.data
        p.goal_radius = sc.goal.radius
        p.params.range = rng if math.isfinite(rng) else 0.0
        p.params.goal_bias = q.goal_bias
        p.params.goal_radius = sc.goal.radius
        p.params.edge_step = sc.edge_step
        p.params.resolution = sc.resolution
        p.params.wavefront = int(q.wavefront)
        p.params.seed = int(q.seed) & ((1 << 64) - 1)
        p.params.max_nodes = int(q.max_nodes)
        p.lo, p.hi = lo.ctypes.data, hi.ctypes.data
        p.time_limit_s = float(q.time_limit)
        if q.surrogate is not None:
            from . import surrogate as S
            S._sig(L)
            h = q.surrogate.h
            p.surrogate = h.value if isinstance(h, ctypes.c_void_p) else h
            p.surrogate_threshold = float(q.threshold)
            p.surrogate_points = int(q.surrogate_points)
            p.surrogate_candidates = int(q.surrogate_candidates)
        p.path, p.path_cap = path.ctypes.data, q.path_cap
    out = (_Result * len(queries))()
    _check(ctx.h, L.mptg_plan_batch(ctx.h, qs, len(queries), int(concurrency), out))
    res = []
    for i, r in enumerate(out):
        n = r.path_len if r.path_len <= queries[i].path_cap else 0
        res.append({"status": r.status, "solved": bool(r.solved), "nodes": r.nodes, "wavefronts": r.wavefronts,
                    "solve_s": r.solve_s, "finish_s": r.finish_s, "cost": r.cost, "path_len": r.path_len,
                    "path": paths[i][:n].copy() if r.solved and n else None})
    del keep
    return res


__all__ = ["Query", "plan_batch"]
