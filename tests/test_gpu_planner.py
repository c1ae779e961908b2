"""GPU: the wavefront planner through the C ABI.

* bit-exact replay: the tree (states, parents, goal ids) after k wavefronts
  equals the oracle's CPU replay of the same wavefront algorithm;
* solving: every returned path is re-validated by the oracle (endpoints,
  each edge's DMV link, cost = summed oracle distances);
* the Planner mirror's API behaviour (reference: test/planner_integration_test.hpp:219-291)."""
import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _planner(ctx, sc, wavefront, seed, max_nodes, goal_bias=0.05, rng=None):
    from mpt_gb300 import planner as P
    pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(wavefront)), seed=seed, ctx=ctx, max_nodes=max_nodes)
    pl.set_goal_bias(goal_bias)
    if rng is not None:
        pl.set_range(rng)
    pl.add_start(sc["start"])
    return pl


def _oracle_plan(orc, sc, wavefront, seed, max_nodes, waves, stop, goal_bias=0.05):
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    params = {"range": sc["range"], "goal_bias": goal_bias, "goal_radius": sc["goal_radius"],
              "edge_step": sc["edge_step"], "resolution": sc["resolution"], "wavefront": wavefront, "seed": seed,
              "max_nodes": max_nodes}
    return orc.plan(sc, sp, params, sc["lo"], sc["hi"], sc["start"], sc["goal"], waves, stop)


@pytest.mark.parametrize("mk,wavefront,waves", [(scenes.grid_scene, 512, 8), (scenes.arm_scene, 256, 4),
                                                (scenes.mesh_scene, 256, 4)])
def test_wavefronts_replay_oracle_bit_exact(ctx, orc, mk, wavefront, waves):
    sc = mk()
    pl = _planner(ctx, sc, wavefront, 1234, 50000)
    pl.run(waves)
    states, parents = pl.graph()
    ws, wp, wg = _oracle_plan(orc, sc, wavefront, 1234, 50000, waves, False)
    assert len(states) == len(ws) and len(ws) > 50
    assert np.array_equal(states.view(np.int64), ws.view(np.int64))
    assert np.array_equal(parents, wp)
    st = pl.stats()
    assert st["goals"] == len(wg)
    pl.close()


def test_grid_solves_and_paths_revalidate(ctx, orc):
    sc = scenes.grid_scene()
    pl = _planner(ctx, sc, 2048, 99, 200000)
    t_end = 60.0
    pl.solve_for(t_end, lambda: pl.solved())
    assert pl.solved()
    path = np.array(pl.solution())
    assert len(path) > 2
    assert np.array_equal(path[0], sc["start"])
    sp = orc.make_space(0, 2)
    assert orc.distance(sp, path[-1], sc["goal"]) <= sc["goal_radius"]
    ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], 0)
    assert ok.all()
    assert orc.valid_states(sc, sp, path).all()
    cost = sum(orc.distance(sp, path[i + 1], path[i]) for i in range(len(path) - 1))
    assert pl.solution_cost() == pytest.approx(cost, rel=0, abs=1e-9)
    seen = []
    pl.solution(lambda q: seen.append(q))
    assert len(seen) == len(path) and all(np.array_equal(a, b) for a, b in zip(seen, path))
    # every tree edge is a valid link too
    states, parents = pl.graph()
    sel = np.nonzero(parents >= 0)[0][:3000]
    ok, _ = orc.valid_edges(sc, sp, states[parents[sel]], states[sel], sc["edge_step"], 0)
    assert ok.all()
    pl.close()


def test_arm_solves_and_paths_revalidate(ctx, orc):
    sc = scenes.arm_scene()
    pl = _planner(ctx, sc, 4096, 7, 400000, goal_bias=0.05)
    pl.solve_for(120.0, lambda: pl.solved())
    if not pl.solved():
        pytest.skip("not solved within the time budget (statistical)")
    path = np.array(pl.solution())
    sp = orc.make_space(1, 10)
    assert np.array_equal(path[0], sc["start"])
    assert orc.distance(sp, path[-1], sc["goal"]) <= sc["goal_radius"]
    ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], 1)
    assert ok.all()
    pl.close()


def test_planner_api_behaviour(ctx):
    from mpt_gb300 import planner as P
    sc = scenes.grid_scene()
    pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(64), P.report_stats(True)), seed=1, ctx=ctx,
                   max_nodes=1000)
    with pytest.raises(RuntimeError):
        pl.solve(lambda: True)  # reference: "there are no valid initial states"
    pl.set_range(16.0)
    assert pl.get_range() == 16.0 and pl.get_goal_bias() == 0.01
    pl.add_start(sc["start"])
    assert pl.size() == 1 and not pl.solved() and pl.solution() == []
    pl.solve(lambda: pl.size() >= 1000)  # node budget ends the run
    assert pl.size() == 1000
    with pytest.raises(RuntimeError):
        pl.set_range(8.0)
    # option packs resolve independent of order (prrt_integration_test.cpp:35-42)
    assert P.PRRT(P.gpu_wavefront(8), P.single_threaded) == P.PRRT(P.single_threaded, P.gpu_wavefront(8))
    seen = []

    class V:
        def vertex(self, q):
            seen.append(("v", tuple(q)))

        def edge(self, q):
            seen.append(("e", tuple(q)))
    pl.visit_graph(V())
    assert sum(1 for s in seen if s[0] == "v") == 1000
    assert sum(1 for s in seen if s[0] == "e") == 999
    pl.close()


def test_same_seed_same_tree(ctx):
    sc = scenes.arm_scene()
    a = _planner(ctx, sc, 1024, 5, 100000)
    b = _planner(ctx, sc, 1024, 5, 100000)
    a.run(3)
    b.run(3)
    sa, pa = a.graph()
    sb, pb = b.graph()
    assert np.array_equal(sa, sb) and np.array_equal(pa, pb)
    c = _planner(ctx, sc, 1024, 6, 100000)
    c.run(3)
    sc_, _ = c.graph()
    assert len(sc_) != len(sa) or not np.array_equal(sc_, sa)


def test_phase_timers_and_wavefront_autotuner(ctx):
    from mpt_gb300 import planner as P
    sc = scenes.grid_scene()
    pl = _planner(ctx, sc, 512, 3, 200000)
    pl.solve_for(20.0, lambda: pl.solved())
    t = pl.timers()
    st = pl.stats()
    assert set(t) == {"nearest", "surrogate", "valid_motion", "insert"}
    # phases are stream-timeline spans; without a surrogate its span is only
    # the gap between two event records
    assert all(v >= 0 for v in t.values()) and t["surrogate"] <= 0.05 * sum(t.values()) + 1e-3
    assert 0 < sum(t.values()) <= st["seconds"] * 1.05 + 1e-3
    pl.close()
    best, med = P.autotune_wavefront(ctx, P.Scenario(sc), sc["start"], candidates=(256, 2048), trials=1,
                                     time_limit=5.0, seed=9)
    assert best in (256, 2048) and set(med) == {256, 2048}
    assert med[best] == min(med.values()) and med[best] < 5.0
