"""GPU: batched multi-query serving (mptg_plan_batch) and planner reuse.

* every query of a concurrent batch gives bit-for-bit the result of a single
  Planner with the same seed and parameters (solved, tree size, wavefronts,
  cost, path), with and without the learned surrogate;
* a batch query's path is a parent chain of the oracle's replayed tree;
* mptg_planner_reset: capacity checks, and a reset planner replays a fresh one.
"""
import ctypes

import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def three():
    return {"grid": scenes.grid_scene(), "arm": scenes.arm_scene(), "mesh": scenes.mesh_scene()}


def _single(ctx, q):
    from mpt_gb300 import planner as P
    pl = P.Planner(q.scenario, P.PRRT(P.gpu_wavefront(q.wavefront)), seed=q.seed, ctx=ctx, max_nodes=q.max_nodes)
    pl.set_goal_bias(q.goal_bias)
    if q.surrogate is not None:
        pl.set_surrogate(q.surrogate, q.threshold, q.surrogate_points)
    pl.add_start(q.start)
    pl.run(0, 0.0, True)
    st = pl.stats()
    path = np.array(pl.solution()) if pl.solved() else None
    cost = pl.last_cost if pl.solved() else float("inf")
    out = {"solved": pl.solved(), "nodes": pl.size(), "wavefronts": int(st["wavefronts"]), "cost": cost,
           "path": path}
    pl.close()
    return out


def _queries(three, n, seed0, surrogate=None, points=1):
    from mpt_gb300 import planner as P
    from mpt_gb300.batch import Query
    sc = {k: P.Scenario(v) for k, v in three.items()}
    budgets = {"grid": [2000, 60000], "arm": [3000, 20000], "mesh": [2000, 12000]}
    waves = {"grid": 512, "arm": 1024, "mesh": 1024}
    kinds = ["grid", "arm", "mesh"]
    qs = []
    for i in range(n):
        k = kinds[i % 3]
        qs.append(Query(sc[k], three[k]["start"], seed=seed0 + i, max_nodes=budgets[k][(i // 3) % 2],
                        wavefront=waves[k], goal_bias=0.05, surrogate=surrogate if k == "mesh" else None,
                        threshold=0.0, surrogate_points=points))
    return qs


def _same(a, b):
    assert a["solved"] == b["solved"]
    assert a["nodes"] == b["nodes"]
    assert a["wavefronts"] == b["wavefronts"]
    if a["solved"]:
        assert a["cost"] == b["cost"]
        assert np.array_equal(a["path"].view(np.int64), b["path"].view(np.int64))


def test_batch_equals_single_planners(ctx, three):
    from mpt_gb300.batch import plan_batch
    qs = _queries(three, 12, 300)
    res = plan_batch(ctx, qs, concurrency=4)
    assert all(r["status"] == 0 for r in res)
    assert any(r["solved"] for r in res) and not all(r["solved"] for r in res)
    for q, r in zip(qs, res):
        _same(r, _single(ctx, q))
        assert r["nodes"] <= q.max_nodes
        assert 0 < r["solve_s"] <= r["finish_s"]


def test_batch_grid_queries_in_one_launch(ctx, three):
    """More grid queries than SMs, run as one persistent launch (one block per
    query): every one returns what a single planner returns, including the
    ones whose budget or whose block's 16,384 nodes run out first."""
    from mpt_gb300 import planner as P
    from mpt_gb300.batch import Query, plan_batch
    sc = three["grid"]
    scen = P.Scenario(sc)
    qs = []
    for i in range(170):
        W = (32, 48, 64, 128, 1000)[i % 5]
        budget = (400, 3000, 20000)[i % 3] if W < 1000 else 30000
        qs.append(Query(scen, sc["start"], seed=900 + i, max_nodes=budget, wavefront=W, goal_bias=0.05))
    res = plan_batch(ctx, qs, concurrency=4)
    assert all(r["status"] == 0 for r in res)
    assert sum(r["solved"] for r in res) > 50 and not all(r["solved"] for r in res)
    for q, r in zip(qs, res):
        _same(r, _single(ctx, q))
        assert r["nodes"] <= q.max_nodes
        assert 0 < r["solve_s"] <= r["finish_s"]


def test_batch_with_surrogate_equals_single(ctx, three):
    from mpt_gb300.batch import plan_batch
    from mpt_gb300.surrogate import Surrogate, se3_normalisation
    scale, shift = se3_normalisation(three["mesh"]["lo"], three["mesh"]["hi"])
    sg = Surrogate(ctx, 7, scale, shift, seed=3)
    for points in (1, 3):
        qs = _queries(three, 9, 500, surrogate=sg, points=points)
        res = plan_batch(ctx, qs, concurrency=6)
        for q, r in zip(qs, res):
            _same(r, _single(ctx, q))


def test_batch_path_is_a_chain_of_the_oracle_tree(ctx, orc, three):
    from mpt_gb300 import planner as P
    from mpt_gb300.batch import Query, plan_batch
    sc = three["grid"]
    q = Query(P.Scenario(sc), sc["start"], seed=77, max_nodes=60000, wavefront=1024, goal_bias=0.05)
    r = plan_batch(ctx, [q, q], concurrency=2)
    assert r[0]["solved"] and r[1]["solved"]
    _same(r[0], r[1])
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    params = {"range": sc["range"], "goal_bias": 0.05, "goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"],
              "resolution": sc["resolution"], "wavefront": 1024, "seed": 77, "max_nodes": 60000}
    ws, wp, wg = orc.plan(sc, sp, params, sc["lo"], sc["hi"], sc["start"], sc["goal"], 1 << 20, True)
    assert len(ws) == r[0]["nodes"]
    path = r[0]["path"]
    # the path's last state is one of the oracle's goal nodes; walking its
    # parents reproduces the path back to the start
    end = [g for g in wg if np.array_equal(ws[g].view(np.int64), path[-1].view(np.int64))]
    assert len(end) == 1
    chain, n = [], end[0]
    while n >= 0:
        chain.append(ws[n])
        n = wp[n]
    chain = np.array(chain[::-1])
    assert np.array_equal(chain.view(np.int64), path.view(np.int64))


def test_planner_reset(ctx, three):
    from mpt_gb300 import _check, load
    from mpt_gb300 import planner as P
    from mpt_gb300.batch import _sig
    L = load()
    _sig(L)
    sc = three["arm"]
    pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(512)), seed=11, ctx=ctx, max_nodes=20000)
    pl.add_start(sc["start"])
    pl.run(3)
    g1 = pl.graph()
    prm = P._Params()
    prm.range, prm.goal_bias, prm.goal_radius = sc["range"], 0.01, sc["goal_radius"]
    prm.edge_step, prm.resolution, prm.wavefront, prm.seed = sc["edge_step"], sc["resolution"], 512, 11
    prm.max_nodes = 40000
    assert L.mptg_planner_reset(pl.h, ctypes.byref(prm)) == 7  # CAPACITY: beyond the created budget
    prm.max_nodes = 20000
    prm.wavefront = 1024
    assert L.mptg_planner_reset(pl.h, ctypes.byref(prm)) == 7
    prm.wavefront = 512
    _check(ctx.h, L.mptg_planner_reset(pl.h, ctypes.byref(prm)))
    assert pl.size() == 0 and not pl.solved()
    assert pl.stats()["wavefronts"] == 0
    start = np.ascontiguousarray(sc["start"], dtype=np.float64)
    goal = np.ascontiguousarray(sc["goal"], dtype=np.float64)
    _check(ctx.h, L.mptg_planner_set_goal(pl.h, goal.ctypes.data, sc["goal_radius"]))
    _check(ctx.h, L.mptg_planner_add_start(pl.h, start.ctypes.data))
    pl.run(3)
    g2 = pl.graph()
    assert np.array_equal(g1[0].view(np.int64), g2[0].view(np.int64))
    assert np.array_equal(g1[1], g2[1])
    # NULL params keeps the parameters
    _check(ctx.h, L.mptg_planner_reset(pl.h, None))
    assert pl.size() == 0
    pl.close()


def test_batch_rejects_bad_queries(ctx, three):
    from mpt_gb300 import MptgError
    from mpt_gb300 import planner as P
    from mpt_gb300.batch import Query, plan_batch
    sc = three["grid"]
    with pytest.raises(MptgError):
        plan_batch(ctx, [Query(P.Scenario(sc), sc["start"], seed=1, max_nodes=1000, wavefront=0)])
    with pytest.raises(MptgError):
        plan_batch(ctx, [Query(P.Scenario(sc), sc["start"], seed=1, max_nodes=0)])
    assert plan_batch(ctx, []) == []
