"""GPU: the persistent block planner (mpt_gb300/csrc/bplan.cu).

On grid scenes with wavefronts of up to 1,024 samples, mptg_planner_run runs
its wavefronts inside one thread block.  It must build exactly the tree of
the multi-kernel wavefront (persistent mode off) and of the oracle's replay
(orc_plan): the same states bit for bit, the same parents and goals, through
the goal sample, the node budget, a stop at the first solution, and the
hand-over to the multi-kernel path past the block's 16,384-node capacity."""
import time

import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _planner(ctx, sc, W, seed, max_nodes, persistent=True, goal_bias=0.05):
    from mpt_gb300 import planner as P
    pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(W)), seed=seed, ctx=ctx, max_nodes=max_nodes)
    pl.set_goal_bias(goal_bias)
    pl.set_persistent(persistent)
    pl.add_start(sc["start"])
    return pl


def _oracle(orc, sc, W, seed, max_nodes, waves, stop, goal_bias=0.05):
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    params = {"range": sc["range"], "goal_bias": goal_bias, "goal_radius": sc["goal_radius"],
              "edge_step": sc["edge_step"], "resolution": sc["resolution"], "wavefront": W, "seed": seed,
              "max_nodes": max_nodes}
    return orc.plan(sc, sp, params, sc["lo"], sc["hi"], sc["start"], sc["goal"], waves, stop)


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("W,waves", [(64, 60), (256, 24), (1000, 8)])
def test_block_planner_replays_oracle(ctx, orc, W, waves):
    sc = scenes.grid_scene()
    pl = _planner(ctx, sc, W, 31, 1 << 20)
    pl.run(waves)
    states, parents = pl.graph()
    ws, wp, wg = _oracle(orc, sc, W, 31, 1 << 20, waves, False)
    assert len(ws) > 100
    assert _same(states, ws) and np.array_equal(parents, wp)
    assert pl.stats()["goals"] == len(wg)
    assert pl.stats()["wavefront_counter"] == waves
    pl.close()


@pytest.mark.parametrize("brute_pairs", [0, 1 << 40])
def test_block_planner_nearest_searches_agree(ctx, orc, brute_pairs):
    """The bucket-grid ring search (brute_pairs 0) and the exhaustive sweep
    (every wavefront) each build the oracle's tree."""
    sc = scenes.grid_scene()
    for W, waves in ((32, 50), (512, 10)):
        pl = _planner(ctx, sc, W, 41, 1 << 20)
        pl.set_block_search(brute_pairs)
        pl.run(waves)
        states, parents = pl.graph()
        ws, wp, wg = _oracle(orc, sc, W, 41, 1 << 20, waves, False)
        assert len(ws) > 100
        assert _same(states, ws) and np.array_equal(parents, wp)
        assert pl.stats()["goals"] == len(wg)
        pl.close()


def test_block_planner_equals_multi_kernel_until_solved(ctx):
    """Solved runs (stop at the first solution, goal sample on): the block
    planner and the multi-kernel path return the same tree, path, cost and
    motion-check sample count."""
    sc = scenes.grid_scene()
    for seed in (1000, 1001, 1002):
        out = []
        for persistent in (True, False):
            pl = _planner(ctx, sc, 256, seed, 1 << 20, persistent=persistent, goal_bias=0.01)
            pl.run(0, 30.0, True)
            assert pl.solved()
            states, parents = pl.graph()
            path = np.array(pl.solution())
            out.append((states, parents, path, pl.last_cost, pl.stats()["link_states_checked"]))
            pl.close()
        (s0, p0, q0, c0, k0), (s1, p1, q1, c1, k1) = out
        assert _same(s0, s1) and np.array_equal(p0, p1)
        assert _same(q0, q1) and c0 == c1
        assert k0 == k1


def test_block_planner_node_budget_and_capacity_hand_over(ctx, orc):
    """A node budget that cuts a wavefront short, and a run past the block's
    16,384-node capacity (the multi-kernel path takes over): both equal the
    oracle's replay."""
    sc = scenes.grid_scene()
    pl = _planner(ctx, sc, 512, 7, 3000)
    pl.run(40)
    states, parents = pl.graph()
    ws, wp, _ = _oracle(orc, sc, 512, 7, 3000, 40, False)
    assert len(states) == 3000 and _same(states, ws) and np.array_equal(parents, wp)
    pl.close()
    pl = _planner(ctx, sc, 1024, 8, 1 << 20, goal_bias=0.0)
    pl.run(40)
    states, parents = pl.graph()
    orc.set_plan_nn("auto")  # the replay's exact CPU kd-tree (same answers as its brute force)
    try:
        ws, wp, _ = _oracle(orc, sc, 1024, 8, 1 << 20, 40, False, goal_bias=0.0)
    finally:
        orc.set_plan_nn("brute")
    assert len(states) > 16384 and _same(states, ws) and np.array_equal(parents, wp)
    pl.close()


def test_block_planner_runs_replay_a_captured_graph(ctx, orc):
    """After its first run a planner replays the block planner through a CUDA
    graph captured on its stream; the tree is still the oracle's replay."""
    sc = scenes.grid_scene()
    pl = _planner(ctx, sc, 48, 52, 1 << 20)
    for _ in range(6):
        pl.run(5)
    assert pl.graph_runs() >= 5
    states, parents = pl.graph()
    ws, wp, _ = _oracle(orc, sc, 48, 52, 1 << 20, 30, False)
    assert _same(states, ws) and np.array_equal(parents, wp)
    pl.close()


def test_block_planner_solves_and_paths_revalidate(ctx, orc):
    """The grid's time to a first solution through the block planner, and the
    oracle's checker on every returned path."""
    sc = scenes.grid_scene()
    sp = orc.make_space(0, 2)
    times = []
    for seed in range(1000, 1010):
        pl = _planner(ctx, sc, 128, seed, 1 << 20, goal_bias=0.01)
        pl.prepare()
        t0 = time.perf_counter()
        pl.solve_for(20.0, lambda: pl.solved())
        times.append(time.perf_counter() - t0)
        assert pl.solved()
        path = np.array(pl.solution())
        assert np.array_equal(path[0], sc["start"])
        assert orc.distance(sp, path[-1], sc["goal"]) <= sc["goal_radius"]
        ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], 0)
        assert ok.all()
        pl.close()
    print("block planner grid time to solve (W=128): p50 %.2f ms, max %.2f ms"
          % (1e3 * float(np.median(times)), 1e3 * max(times)))
