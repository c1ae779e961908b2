"""mpt_gb300 - GB300-native hot path of MPT's parallel planners.

Python host mirror of the C ABI in include/mptg.h:

* ``Context``  -- one per GPU (mptg_create)
* ``Tree``     -- the device kd-tree standing in for nigh::Nigh (insert,
  nearest, nearest_k, linear scan)
* ``Scene``    -- a scenario's collision world: ``valid(states)`` batches
  Scenario::valid, ``link(a, b)`` batches Scenario::link through the
  DiscreteMotionValidator
* ``planner``  -- Planner / PRRT with the reference's option names

All compute runs in libmptg.so's CUDA kernels; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import MptgError, load, ptr

L2, SO2, SO3, SE3, L1 = 0, 1, 2, 3, 4
SCENE_GRID, SCENE_PLANAR_ARM, SCENE_RIGID_MESH = 0, 1, 2


def _check(ctx_handle, st: int):
    if st != 0:
        msg = load().mptg_last_error(ctx_handle)
        raise MptgError(st, msg.decode() if msg else "")


def _is_host(x) -> bool:
    return isinstance(x, np.ndarray)


class Context:
    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        st = self.lib.mptg_create(ctypes.byref(h), device)
        if st != 0:
            raise MptgError(st, "mptg_create(device=%d) failed" % device)
        self.h = h
        self.device = device

    def kernel_launches(self) -> int:
        return int(self.lib.mptg_kernel_launches(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.mptg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream_ptr(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


class Tree:
    """Device kd-tree over one metric space (nigh::Nigh stand-in)."""

    def __init__(self, ctx: Context, metric: int, dim: int, capacity: int, weights=(1.0, 1.0)):
        self.ctx = ctx
        self.lib = ctx.lib
        self.metric, self.dim = metric, dim
        w = np.asarray(weights, dtype=np.float64)
        self._w = w
        h = ctypes.c_void_p()
        _check(ctx.h, self.lib.mptg_tree_create(ctx.h, metric, dim, w.ctypes.data, capacity, ctypes.byref(h)))
        self.h = h

    @classmethod
    def borrow(cls, ctx: Context, handle, metric: int, dim: int, weights=(1.0, 1.0), owner=None):
        """A Tree view of a handle another object owns (mptg_planner_tree):
        queries only; closing it does not destroy the tree."""
        t = cls.__new__(cls)
        t.ctx, t.lib = ctx, ctx.lib
        t.metric, t.dim = metric, dim
        t._w = np.asarray(weights, dtype=np.float64)
        t.h = handle
        t._owner = owner
        return t

    # nearest-neighbour strategies (mptg_nn_strategy)
    AUTO, KDTREE, EXHAUSTIVE = 0, 1, 2

    def set_strategy(self, strategy: int):
        _check(self.ctx.h, self.lib.mptg_tree_set_strategy(self.h, int(strategy)))

    def __len__(self):
        n = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_tree_size(self.h, ctypes.byref(n)))
        return n.value

    def insert(self, states, stream=None):
        if _is_host(states):
            states = np.ascontiguousarray(states, dtype=np.float64).reshape(-1, self.dim)
            n = states.shape[0]
        else:
            n = states.shape[0]
        _check(self.ctx.h, self.lib.mptg_tree_insert(self.h, ptr(states), n, _stream_ptr(stream)))

    def states(self, first: int = 0, n: int | None = None) -> np.ndarray:
        if n is None:
            n = len(self) - first
        out = np.empty((n, self.dim), dtype=np.float64)
        _check(self.ctx.h, self.lib.mptg_tree_states(self.h, first, n, out.ctypes.data, None))
        return out

    def nearest(self, queries, idx_out=None, dist_out=None, stream=None, linear=False):
        """Exact 1-NN of every query: (ids int32, distances float64).

        numpy queries -> numpy results (synchronous); device tensors need
        device ``idx_out``/``dist_out`` and run asynchronously on ``stream``."""
        fn = self.lib.mptg_nearest_linear if linear else self.lib.mptg_nearest
        if _is_host(queries):
            q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, self.dim)
            nq = q.shape[0]
            idx = np.empty(nq, dtype=np.int32)
            dist = np.empty(nq, dtype=np.float64)
            _check(self.ctx.h, fn(self.h, q.ctypes.data, nq, idx.ctypes.data, dist.ctypes.data, None))
            return idx, dist
        nq = queries.shape[0]
        _check(self.ctx.h, fn(self.h, ptr(queries), nq, ptr(idx_out), ptr(dist_out), _stream_ptr(stream)))
        return idx_out, dist_out

    def nearest_k(self, queries, k: int, radius: float = float("inf")):
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, self.dim)
        nq = q.shape[0]
        idx = np.empty((nq, k), dtype=np.int32)
        dist = np.empty((nq, k), dtype=np.float64)
        _check(self.ctx.h, self.lib.mptg_nearest_k(self.h, q.ctypes.data, nq, k, float(radius), idx.ctypes.data,
                                                   dist.ctypes.data, None))
        return idx, dist

    def counters(self, reset: bool = False) -> dict:
        out = (ctypes.c_uint64 * 5)()
        _check(self.ctx.h, self.lib.mptg_tree_counters(self.h, out, int(reset)))
        keys = ["queries", "internal_visited", "leaves_visited", "points_evaluated", "reranked"]
        return dict(zip(keys, [int(v) for v in out]))

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owner", None) is None:
                self.lib.mptg_tree_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """A scenario's collision world on the device."""

    def __init__(self, ctx: Context, desc: dict):
        self.ctx = ctx
        self.lib = ctx.lib
        d = _lib.SceneDesc()
        self._keep = []
        kind = desc["kind"]
        if kind == "grid":
            g = np.ascontiguousarray(desc["grid"], dtype=np.uint8)
            self._keep.append(g)
            d.kind = SCENE_GRID
            d.grid = g.ctypes.data
            d.height, d.width = g.shape
        elif kind == "arm":
            ll = np.ascontiguousarray(desc["link_len"], dtype=np.float64)
            dc = np.ascontiguousarray(desc["discs"], dtype=np.float64)
            self._keep += [ll, dc]
            d.kind = SCENE_PLANAR_ARM
            d.nlinks = ll.shape[0]
            d.link_len = ll.ctypes.data
            d.ndiscs = dc.shape[0]
            d.discs = dc.ctypes.data
            d.robot_radius = float(desc.get("robot_radius", 0.0))
            d.self_collision = int(desc.get("self_collision", 1))
        elif kind == "mesh":
            rt = np.ascontiguousarray(desc["robot_tris"], dtype=np.float64)
            et = np.ascontiguousarray(desc["env_tris"], dtype=np.float64)
            self._keep += [rt, et]
            d.kind = SCENE_RIGID_MESH
            d.nrobot = rt.shape[0]
            d.robot_tris = rt.ctypes.data
            d.nenv = et.shape[0]
            d.env_tris = et.ctypes.data
            w = desc.get("weights", (1.0, 1.0))
            d.w_rot, d.w_pos = float(w[0]), float(w[1])
        else:
            raise ValueError(kind)
        h = ctypes.c_void_p()
        _check(ctx.h, self.lib.mptg_scene_create(ctx.h, ctypes.byref(d), ctypes.byref(h)))
        self.h = h
        dim = ctypes.c_int()
        met = ctypes.c_int()
        w = (ctypes.c_double * 2)()
        _check(ctx.h, self.lib.mptg_scene_space(h, ctypes.byref(dim), ctypes.byref(met), w))
        self.dim, self.metric, self.weights = dim.value, met.value, (w[0], w[1])

    def valid(self, states, out=None, stream=None):
        if _is_host(states):
            q = np.ascontiguousarray(states, dtype=np.float64).reshape(-1, self.dim)
            res = np.empty(q.shape[0], dtype=np.uint8)
            _check(self.ctx.h, self.lib.mptg_valid_states(self.h, q.ctypes.data, q.shape[0], res.ctypes.data, None))
            return res
        _check(self.ctx.h, self.lib.mptg_valid_states(self.h, ptr(states), states.shape[0], ptr(out),
                                                      _stream_ptr(stream)))
        return out

    def link(self, a, b, step: float, resolution: int = 0, out=None, stream=None):
        if _is_host(a):
            a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, self.dim)
            b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1, self.dim)
            res = np.empty(a.shape[0], dtype=np.uint8)
            _check(self.ctx.h, self.lib.mptg_valid_edges(self.h, a.ctypes.data, b.ctypes.data, a.shape[0], float(step),
                                                         int(resolution), res.ctypes.data, None))
            return res
        _check(self.ctx.h, self.lib.mptg_valid_edges(self.h, ptr(a), ptr(b), a.shape[0], float(step), int(resolution),
                                                     ptr(out), _stream_ptr(stream)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.mptg_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
