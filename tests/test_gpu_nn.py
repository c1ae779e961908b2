"""GPU parity: kd-tree nearest / k-nearest / linear scan through the C ABI
against the oracle's exact FP64 brute force (bit-exact ids and distances)."""
import math

import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _se3_space():
    return {"metric": 3, "dim": 7, "lo": np.array([-1, -1, -1, -1, 0, 0, 0.0]),
            "hi": np.array([1, 1, 1, 1, 20, 20, 20.0]), "weights": (2.0, 1.0)}


SPACES = {
    "grid_l2": lambda: scenes.grid_scene(),
    "arm_so2x10": lambda: scenes.arm_scene(),
    "se3": _se3_space,
    "l1_3d": lambda: {"metric": 4, "dim": 3, "lo": np.zeros(3), "hi": np.full(3, 5.0), "weights": (1, 1)},
    "so3": lambda: {"metric": 2, "dim": 4, "lo": None, "hi": None, "weights": (1, 1)},
    "l2_16d": lambda: {"metric": 0, "dim": 16, "lo": np.full(16, -1.0), "hi": np.ones(16), "weights": (1, 1)},
}


def _make(ctx, sc, cap):
    import mpt_gb300 as m
    return m.Tree(ctx, sc["metric"], sc["dim"], cap, sc["weights"])


@pytest.mark.parametrize("name", list(SPACES))
def test_nearest_matches_oracle(ctx, orc, name):
    sc = SPACES[name]()
    n = 20000
    pts = scenes.uniform_states(sc, n, 101)
    q = scenes.uniform_states(sc, 2000, 102)
    tree = _make(ctx, sc, n)
    # batches of different sizes exercise leaf overflow splits
    for lo, hi in [(0, 1), (1, 40), (40, 1000), (1000, 1001), (1001, 8000), (8000, n)]:
        tree.insert(pts[lo:hi])
    assert len(tree) == n
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    oi, od = orc.nn_brute(sp, pts, q)
    q2 = np.concatenate([q, scenes.uniform_states(sc, 3001, 103)])
    oi2, od2 = orc.nn_brute(sp, pts, q2)
    for strategy in (tree.KDTREE, tree.EXHAUSTIVE, tree.AUTO):
        tree.set_strategy(strategy)
        gi, gd = tree.nearest(q)  # < 2048 queries: input order
        assert np.array_equal(gi, oi), (strategy, np.nonzero(gi != oi)[0][:10])
        assert np.array_equal(gd.view(np.int64), od.view(np.int64))
        # >= 2048 queries: spatially ordered search
        gi2, gd2 = tree.nearest(q2)
        assert np.array_equal(gi2, oi2), (strategy, np.nonzero(gi2 != oi2)[0][:10])
        assert np.array_equal(gd2.view(np.int64), od2.view(np.int64))
    li, ld = tree.nearest(q, linear=True)
    assert np.array_equal(li, oi) and np.array_equal(ld.view(np.int64), od.view(np.int64))
    # stored states come back unchanged
    assert np.array_equal(tree.states(), pts)


def test_nearest_ties_and_duplicates(ctx, orc):
    import mpt_gb300 as m
    sc = {"metric": 0, "dim": 2, "weights": (1, 1)}
    base = np.array([[1.0, 1.0], [3.0, 1.0]])
    # 100 copies of two points (degenerate splits), plus a lattice with exact ties
    pts = np.concatenate([np.repeat(base, 100, axis=0), np.stack(np.meshgrid(np.arange(10.0), np.arange(10.0)),
                                                                 -1).reshape(-1, 2)])
    tree = m.Tree(ctx, 0, 2, len(pts))
    tree.insert(pts[:150])
    tree.insert(pts[150:])
    q = np.array([[2.0, 1.0], [1.0, 1.0], [0.5, 0.5], [4.5, 4.5], [9.0, 9.0], [100.0, -3.0]])
    sp = orc.make_space(0, 2)
    oi, od = orc.nn_brute(sp, pts, q)
    for strategy in (tree.KDTREE, tree.EXHAUSTIVE):
        tree.set_strategy(strategy)
        gi, gd = tree.nearest(q)
        assert np.array_equal(gi, oi) and np.array_equal(gd, od)
        assert gi[1] == 0  # lowest id among 100 identical points at distance 0
    # more than 8 points within the FP32 band of the minimum: the exhaustive
    # sweep's second pass
    pts8 = np.concatenate([np.repeat(np.array([[0.25] * 8]), 20, axis=0),
                           scenes.uniform_states({"metric": 0, "dim": 8, "lo": np.zeros(8), "hi": np.ones(8)}, 500, 7)])
    t8 = m.Tree(ctx, 0, 8, len(pts8))
    t8.insert(pts8)
    q8 = np.concatenate([np.full((3, 8), 0.25), np.full((2, 8), 0.2500001), np.random.default_rng(1).random((50, 8))])
    oi8, od8 = orc.nn_brute(orc.make_space(0, 8), pts8, q8)
    for strategy in (t8.KDTREE, t8.EXHAUSTIVE):
        t8.set_strategy(strategy)
        gi8, gd8 = t8.nearest(q8)
        assert np.array_equal(gi8, oi8) and np.array_equal(gd8.view(np.int64), od8.view(np.int64))
        assert (gi8[:5] == 0).all()


def test_frontier_growth_rebuilds_and_stays_exact(ctx, orc):
    """A tree grown at one frontier (points along a line, in small batches)
    degenerates under leaf splits; the depth-triggered rebuild keeps it
    searchable and exact."""
    import mpt_gb300 as m
    rng = np.random.default_rng(3)
    t = np.linspace(0, 1000, 20000)
    pts = np.stack([t, 0.001 * np.sin(t)], 1) + rng.normal(0, 1e-3, (20000, 2))
    tree = m.Tree(ctx, 0, 2, len(pts))
    for lo in range(0, len(pts), 100):
        tree.insert(pts[lo:lo + 100])
    q = np.stack([rng.uniform(-10, 1010, 3000), rng.uniform(-5, 5, 3000)], 1)
    oi, od = orc.nn_brute(orc.make_space(0, 2), pts, q)
    gi, gd = tree.nearest(q)
    assert np.array_equal(gi, oi) and np.array_equal(gd, od)


def test_empty_and_single(ctx):
    import mpt_gb300 as m
    tree = m.Tree(ctx, 1, 3, 10)
    i, d = tree.nearest(np.zeros((3, 3)))
    assert (i == -1).all() and np.isinf(d).all()
    tree.insert(np.array([[0.5, -0.5, 3.0]]))
    i, d = tree.nearest(np.array([[0.5, -0.5, -3.0]]))
    assert i[0] == 0
    assert d[0] == abs(0.5 - 0.5) + 0.0 + (2 * math.pi - 6.0) or d[0] >= 0


def test_invalid_states_rejected(ctx):
    import mpt_gb300 as m
    tree = m.Tree(ctx, 1, 2, 10)
    with pytest.raises(m.MptgError):
        tree.insert(np.array([[4.0, 0.0]]))  # outside [-pi, pi]
    assert len(tree) == 0
    tq = m.Tree(ctx, 3, 7, 10, (2.0, 1.0))
    with pytest.raises(m.MptgError):
        tq.insert(np.array([[0.0, 0, 0, 0.9, 1, 2, 3]]))  # not a unit quaternion
    with pytest.raises(m.MptgError):
        m.Tree(ctx, 0, 17, 10)
    with pytest.raises(m.MptgError):
        tree.insert(np.zeros((11, 2)))  # capacity


@pytest.mark.parametrize("name,k,radius", [("grid_l2", 1, math.inf), ("grid_l2", 7, math.inf),
                                           ("arm_so2x10", 40, math.inf), ("arm_so2x10", 64, 6.0),
                                           ("se3", 33, math.inf), ("grid_l2", 20, 10.0)])
def test_nearest_k_matches_oracle(ctx, orc, name, k, radius):
    sc = SPACES[name]()
    n = 12000
    pts = scenes.uniform_states(sc, n, 201)
    q = scenes.uniform_states(sc, 500, 202)
    tree = _make(ctx, sc, n)
    tree.insert(pts[:5000])
    tree.insert(pts[5000:])
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    oi, od = orc.knn_brute(sp, pts, q, k)
    if math.isfinite(radius):
        far = od > radius
        oi[far] = -1
        od[far] = np.inf
    for strategy in (tree.KDTREE, tree.EXHAUSTIVE, tree.AUTO):
        tree.set_strategy(strategy)
        gi, gd = tree.nearest_k(q, k, radius)
        assert np.array_equal(gi, oi), strategy
        assert np.array_equal(gd, od)


@pytest.mark.parametrize("n,reps,k", [(40, 1, 32), (12000, 6, 32), (12000, 40, 20), (9000, 1, 48)])
def test_nearest_k_exhaustive_ties(ctx, orc, n, reps, k):
    """The exhaustive k-NN's FP32 selection: splits smaller than its 64-entry
    list, runs of duplicates longer than the list's slack (the exact second
    sweep) and k near the slack, against the oracle's (distance, id) order."""
    sc = SPACES["arm_so2x10"]()
    base = scenes.uniform_states(sc, max(1, n // reps), 211)
    pts = np.repeat(base, reps, axis=0)[:n]
    q = np.concatenate([scenes.uniform_states(sc, 300, 212), base[:20]])
    tree = _make(ctx, sc, n)
    tree.insert(pts)
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    oi, od = orc.knn_brute(sp, pts, q, k)
    for strategy in (tree.EXHAUSTIVE, tree.KDTREE):
        tree.set_strategy(strategy)
        gi, gd = tree.nearest_k(q, k)
        assert np.array_equal(gi, oi), strategy
        assert np.array_equal(gd, od)


def test_device_buffers_async(ctx, orc):
    torch = pytest.importorskip("torch")
    import mpt_gb300 as m
    sc = scenes.arm_scene()
    pts = scenes.uniform_states(sc, 30000, 301)
    q = scenes.uniform_states(sc, 4096, 302)
    tree = m.Tree(ctx, sc["metric"], sc["dim"], len(pts))
    dp = torch.from_numpy(pts).cuda()
    tree.insert(dp)
    dq = torch.from_numpy(q).cuda()
    di = torch.empty(len(q), dtype=torch.int32, device="cuda")
    dd = torch.empty(len(q), dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        tree.nearest(dq, di, dd, stream=s)
    s.synchronize()
    oi, od = orc.nn_brute(orc.make_space(1, 10), pts, q)
    assert np.array_equal(di.cpu().numpy(), oi)
    assert np.array_equal(dd.cpu().numpy(), od)
    c = tree.counters(reset=True)
    assert c["queries"] == len(q) and c["points_evaluated"] > 0
