"""Learned collision surrogate (host mirror of mptg_surrogate_*).

Trained on states labelled by the exact checker; used by the planner only to
order and cull candidate edges -- the exact check still decides every edge
that enters the tree.  See mpt_gb300/csrc/surrogate.cu for the network.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import Context, _check, load


def _sig(L):
    if getattr(L, "_sg_sig", False):
        return
    P, S = ctypes.c_void_p, ctypes.c_size_t
    for name, args in [
        ("mptg_surrogate_create", [P, ctypes.c_int, P, P, ctypes.c_uint64, ctypes.POINTER(P)]),
        ("mptg_surrogate_destroy", [P]),
        ("mptg_surrogate_num_params", [P, ctypes.POINTER(S)]),
        ("mptg_surrogate_get", [P, ctypes.c_int, P, S]),
        ("mptg_surrogate_set", [P, P, S]),
        ("mptg_surrogate_train_step", [P, P, P, S, ctypes.c_double, ctypes.POINTER(ctypes.c_float), P]),
        ("mptg_surrogate_score", [P, P, S, P, P]),
        ("mptg_planner_set_surrogate", [P, P, ctypes.c_double]),
        ("mptg_planner_set_surrogate_points", [P, ctypes.c_int]),
        ("mptg_planner_set_surrogate_bias", [P, ctypes.c_int]),
    ]:
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = args
    L._sg_sig = True


def se3_normalisation(lo, hi, pos_gain: float = 10.0):
    """Feature map for SE(3) states: position to [-pos_gain, pos_gain],
    quaternion unchanged.  A gain of 10 lets the first SiLU layer resolve
    obstacles about 1/20 of the workspace across (held-out accuracy on the
    400-box scene: 0.76 at gain 1, 0.86 at gain 10, 1M states, 5 epochs)."""
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    scale = np.ones(7)
    shift = np.zeros(7)
    scale[4:] = 2.0 * pos_gain / (hi[4:] - lo[4:])
    shift[4:] = 0.5 * (hi[4:] + lo[4:])
    return scale, shift


class Surrogate:
    def __init__(self, ctx: Context, in_dim: int, scale=None, shift=None, seed: int = 1):
        self.ctx = ctx
        self.lib = load()
        _sig(self.lib)
        self.in_dim = in_dim
        sc = np.ascontiguousarray(scale if scale is not None else np.ones(in_dim), dtype=np.float64)
        sh = np.ascontiguousarray(shift if shift is not None else np.zeros(in_dim), dtype=np.float64)
        h = ctypes.c_void_p()
        _check(ctx.h, self.lib.mptg_surrogate_create(ctx.h, in_dim, sc.ctypes.data, sh.ctypes.data, seed,
                                                     ctypes.byref(h)))
        self.h = h
        n = ctypes.c_size_t()
        _check(ctx.h, self.lib.mptg_surrogate_num_params(h, ctypes.byref(n)))
        self.nparam = n.value

    def params(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        _check(self.ctx.h, self.lib.mptg_surrogate_get(self.h, 0, out.ctypes.data, self.nparam))
        return out

    def grads(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        _check(self.ctx.h, self.lib.mptg_surrogate_get(self.h, 1, out.ctypes.data, self.nparam))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(self.ctx.h, self.lib.mptg_surrogate_set(self.h, p.ctypes.data, self.nparam))

    def train_step(self, states, labels, lr: float = 1e-3) -> float:
        s = np.ascontiguousarray(states, dtype=np.float64)
        y = np.ascontiguousarray(labels, dtype=np.uint8)
        loss = ctypes.c_float()
        _check(self.ctx.h, self.lib.mptg_surrogate_train_step(self.h, s.ctypes.data, y.ctypes.data, len(y), float(lr),
                                                              ctypes.byref(loss), None))
        return float(loss.value)

    def score(self, states) -> np.ndarray:
        s = np.ascontiguousarray(states, dtype=np.float64)
        out = np.empty(len(s), dtype=np.float32)
        _check(self.ctx.h, self.lib.mptg_surrogate_score(self.h, s.ctypes.data, len(s), out.ctypes.data, None))
        return out

    def fit(self, states, labels, epochs: int = 1, batch: int = 8192, lr: float = 1e-3, seed: int = 0):
        """Adam over shuffled mini-batches; returns the per-epoch mean loss."""
        rng = np.random.default_rng(seed)
        n = (len(states) // batch) * batch
        hist = []
        for _ in range(epochs):
            perm = rng.permutation(len(states))[:n]
            losses = [self.train_step(states[perm[i:i + batch]], labels[perm[i:i + batch]], lr)
                      for i in range(0, n, batch)]
            hist.append(float(np.mean(losses)))
        return hist

    def close(self):
        if getattr(self, "h", None):
            self.lib.mptg_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
