"""GPU: the wavefront PRRT* (k-nearest rewiring) through the C ABI.

* bit-exact replay: states, parents, costs and the rewire count after k
  wavefronts equal the oracle's CPU replay (orc_plan_star);
* the rewired graph stays a tree whose edges pass the exact check and whose
  costs are the path lengths;
* the best solution's cost does not increase as the planner keeps running,
  and ends below the plain PRRT's on the same seed.
(reference: src/mpt/impl/prrt_star/prrt_star.hpp:505-657)"""
import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _star(ctx, sc, wavefront, seed, max_nodes, goal_bias=0.05, star=True):
    from mpt_gb300 import planner as P
    algo = P.PRRTStar(P.gpu_wavefront(wavefront)) if star else P.PRRT(P.gpu_wavefront(wavefront))
    pl = P.Planner(P.Scenario(sc), algo, seed=seed, ctx=ctx, max_nodes=max_nodes)
    pl.set_goal_bias(goal_bias)
    pl.add_start(sc["start"])
    return pl


@pytest.mark.parametrize("mk,wavefront,waves", [(scenes.grid_scene, 256, 10), (scenes.arm_scene, 256, 5),
                                                (scenes.mesh_scene, 256, 5)])
def test_prrt_star_replays_oracle_bit_exact(ctx, orc, mk, wavefront, waves):
    sc = mk()
    pl = _star(ctx, sc, wavefront, 4321, 20000)
    pl.run(waves)
    states, parents = pl.graph()
    costs = pl.costs()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    params = {"range": sc["range"], "goal_bias": 0.05, "goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"],
              "resolution": sc["resolution"], "wavefront": wavefront, "seed": 4321, "max_nodes": 20000}
    ws, wp, wc, wg, nrw = orc.plan_star(sc, sp, params, sc["lo"], sc["hi"], sc["start"], sc["goal"], waves)
    assert len(states) == len(ws) and len(ws) > 100
    assert np.array_equal(states.view(np.int64), ws.view(np.int64))
    assert np.array_equal(parents, wp)
    assert np.array_equal(costs.view(np.int64), wc.view(np.int64))
    assert pl.rewire_stats()["rewires"] == nrw
    assert pl.stats()["goals"] == len(wg)
    pl.close()


def test_prrt_star_graph_is_an_exact_tree(ctx, orc):
    sc = scenes.grid_scene()
    pl = _star(ctx, sc, 512, 7, 60000)
    pl.run(25)
    states, parents = pl.graph()
    costs = pl.costs()
    n = len(states)
    assert pl.rewire_stats()["rewires"] > 0
    # no cycles: every node reaches the start
    depth = np.zeros(n, dtype=np.int64)
    for x in range(n):
        y, d = x, 0
        while parents[y] >= 0:
            y = parents[y]
            d += 1
            assert d <= n
        assert y == 0
        depth[x] = d
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    sel = np.nonzero(parents >= 0)[0]
    ok, _ = orc.valid_edges(sc, sp, states[parents[sel]], states[sel], sc["edge_step"], sc["resolution"])
    assert ok.all()
    # costs are path lengths (summation order aside)
    for x in sel[:: max(1, len(sel) // 300)]:
        c, y = 0.0, x
        while parents[y] >= 0:
            c += orc.distance(sp, states[parents[y]], states[y])
            y = parents[y]
        assert abs(c - costs[x]) <= 1e-9 * max(1.0, c)
    pl.close()


def test_prrt_star_solution_improves(ctx, orc):
    sc = scenes.grid_scene()
    pl = _star(ctx, sc, 1024, 11, 400000)
    pl.solve_for(20.0, lambda: pl.solved())
    assert pl.solved()
    first = pl.solution_cost()
    hist = [first]
    for _ in range(8):
        pl.run(10)
        hist.append(pl.solution_cost())
    assert all(b <= a + 1e-9 for a, b in zip(hist, hist[1:]))
    path = np.array(pl.solution())
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], sc["resolution"])
    assert ok.all()
    assert np.array_equal(path[0], sc["start"])
    plain = _star(ctx, sc, 1024, 11, 400000, star=False)
    plain.run(int(pl.stats()["wavefronts"]))
    assert hist[-1] < plain.solution_cost()
    print("PRRT* cost %.2f -> %.2f; PRRT %.2f; rewires %s" % (first, hist[-1], plain.solution_cost(),
                                                            pl.rewire_stats()))
    pl.close()
    plain.close()


def test_set_rewire_after_first_wavefront_is_rejected(ctx):
    from mpt_gb300 import MptgError
    sc = scenes.grid_scene()
    pl = _star(ctx, sc, 256, 1, 10000, star=False)
    pl.run(1)
    with pytest.raises(MptgError):
        from mpt_gb300 import _check
        _check(ctx.h, pl.lib.mptg_planner_set_rewire(pl.h, 1, 1.1))
    pl.close()
