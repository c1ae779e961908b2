"""GPU: mptg_nearest_linear_noalloc, the nearest-neighbour entry point that
allocates no device memory, for callers that cannot allocate while they run
(real-time control loops that must not call cudaMalloc after start-up, and
plugins whose host framework owns all device memory).

Called through the C ABI and checked, bit for bit as every NN test here is,
against the existing allocating entry point (mptg_nearest_linear on a tree
holding the same points) and against the oracle's exact FP64 brute force, on
calls in a row over five metrics.  This file is collected last so that a
failing run stops only after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_fn(lib):
    f = lib.mptg_nearest_linear_noalloc
    P = ctypes.c_void_p
    f.restype = ctypes.c_int
    f.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_size_t, P, ctypes.c_size_t, P, P, P]
    return f


def _existing(ctx, metric, dim, w, pts, q):
    import mpt_gb300 as m
    tree = m.Tree(ctx, metric, dim, max(1, len(pts)), w)
    tree.insert(pts)
    return tree.nearest(q, linear=True)


def _call(fn, ctx, torch, sc, pts, q):
    n, nq = len(pts), len(q)
    w = np.asarray(sc["weights"], dtype=np.float64)
    dp = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    dq = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    di = torch.full((nq,), -7, dtype=torch.int32, device="cuda")
    dd = torch.zeros(nq, dtype=torch.float64, device="cuda")
    st = fn(ctx.h, sc["metric"], sc["dim"], w.ctypes.data, dp.data_ptr(), n, dq.data_ptr(), nq, di.data_ptr(),
            dd.data_ptr(), None)
    torch.cuda.synchronize()
    return st, di.cpu().numpy(), dd.cpu().numpy()


def test_noalloc_matches_existing_entry_point_twice(ctx, orc):
    torch = pytest.importorskip("torch")
    import mpt_gb300 as m
    from mpt_gb300 import scenes
    fn = _noalloc_fn(m.load())
    se3 = {"metric": 3, "dim": 7, "lo": np.array([-1, -1, -1, -1, 0, 0, 0.0]),
           "hi": np.array([1, 1, 1, 1, 20, 20, 20.0]), "weights": (2.0, 1.0)}
    so3 = {"metric": 2, "dim": 4, "weights": (1.0, 1.0)}
    l1 = {"metric": 4, "dim": 3, "lo": np.full(3, -50.0), "hi": np.full(3, 50.0), "weights": (1.0, 1.0)}
    calls = [(scenes.grid_scene(), 40000, 3000, 11),   # first call: large L2 coordinates
             (scenes.arm_scene(), 20000, 2000, 12),    # second call: fewer points, another metric
             (l1, 30000, 1500, 14),                    # L1 in 3-D (the kernel's 4-wide instance)
             (so3, 25000, 1500, 15),                   # SO(3): the chord sweep with FP64 acos re-rank
             (se3, 65536, 1000, 13)]                   # the maximum point count
    for sc, n, nq, seed in calls:
        pts = scenes.uniform_states(sc, n, seed)
        q = scenes.uniform_states(sc, nq, seed + 100)
        want_i, want_d = _existing(ctx, sc["metric"], sc["dim"], sc["weights"], pts, q)
        st, got_i, got_d = _call(fn, ctx, torch, sc, pts, q)
        assert st == 0, m.load().mptg_last_error(ctx.h)
        assert np.array_equal(got_i, want_i)
        assert np.array_equal(got_d.view(np.int64), want_d.view(np.int64))
        # and directly against the oracle's exact FP64 brute force (lowest id on ties)
        sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
        oi, od = orc.nn_brute(sp, pts, q[:300])
        assert np.array_equal(got_i[:300], oi)
        assert np.array_equal(got_d[:300].view(np.int64), od.view(np.int64))


def test_noalloc_invalid_call_does_not_leak_into_the_next(ctx):
    """A call with a NaN point answers id -1 and NaN for every query; the next
    call on the same scratch array answers exactly as the allocating entry
    point does (each call clears the error flag it shares)."""
    torch = pytest.importorskip("torch")
    import mpt_gb300 as m
    from mpt_gb300 import scenes
    fn = _noalloc_fn(m.load())
    sc = scenes.grid_scene()
    pts = scenes.uniform_states(sc, 5000, 31)
    q = scenes.uniform_states(sc, 700, 32)
    bad = pts.copy()
    bad[1234, 1] = np.nan
    st, gi, gd = _call(fn, ctx, torch, sc, bad, q)
    assert st == 0
    assert (gi == -1).all() and np.isnan(gd).all()
    want_i, want_d = _existing(ctx, sc["metric"], sc["dim"], sc["weights"], pts, q)
    st, gi, gd = _call(fn, ctx, torch, sc, pts, q)
    assert st == 0
    assert np.array_equal(gi, want_i) and np.array_equal(gd.view(np.int64), want_d.view(np.int64))


def test_noalloc_rejects_oversize_and_host_buffers(ctx):
    torch = pytest.importorskip("torch")
    import mpt_gb300 as m
    fn = _noalloc_fn(m.load())
    dq = torch.zeros((4, 2), dtype=torch.float64, device="cuda")
    di = torch.empty(4, dtype=torch.int32, device="cuda")
    dd = torch.empty(4, dtype=torch.float64, device="cuda")
    big = torch.zeros((65537, 2), dtype=torch.float64, device="cuda")
    st = fn(ctx.h, 0, 2, None, big.data_ptr(), 65537, dq.data_ptr(), 4, di.data_ptr(), dd.data_ptr(), None)
    assert st == 1 and b"at most 65536 points" in m.load().mptg_last_error(ctx.h)
    hq = np.zeros((4, 2))
    st = fn(ctx.h, 0, 2, None, big.data_ptr(), 10, hq.ctypes.data, 4, di.data_ptr(), dd.data_ptr(), None)
    assert st == 1
    # an empty point set answers -1 / +inf
    st = fn(ctx.h, 0, 2, None, None, 0, dq.data_ptr(), 4, di.data_ptr(), dd.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    assert (di.cpu().numpy() == -1).all() and np.isinf(dd.cpu().numpy()).all()
