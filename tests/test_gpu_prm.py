"""GPU: the wavefront PPRM roadmap through the C ABI.

* bit-exact replay: nodes, the sorted edge list (from, to, distance), the
  counters (goal nodes included) and the Dijkstra path equal the oracle's
  one-sample-at-a-time replay (orc_prm) on the same sample stream;
* a solve on each scene: every edge passes the exact link check and the path
  is a chain of roadmap edges whose distances sum to the reported cost;
* the reference's error behaviour: no start or goal, invalid and duplicate
  starts.
(reference: src/mpt/impl/pprm/pprm.hpp:155-183,298-339)"""
import math

import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _prm(ctx, sc, wavefront, seed, max_nodes):
    from mpt_gb300 import planner as P
    pl = P.Planner(P.Scenario(sc), P.PPRM(P.gpu_wavefront(wavefront)), seed=seed, ctx=ctx, max_nodes=max_nodes)
    assert isinstance(pl, P.PPRMPlanner)
    return pl


def _params(sc, wavefront, seed, max_nodes):
    return {"goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"], "resolution": sc["resolution"],
            "wavefront": wavefront, "seed": seed, "max_nodes": max_nodes}


@pytest.mark.parametrize("mk,wavefront,waves", [(scenes.grid_scene, 256, 8), (scenes.arm_scene, 512, 8),
                                                (scenes.mesh_scene, 128, 4)])
def test_prm_replays_oracle_bit_exact(ctx, orc, mk, wavefront, waves):
    sc = mk()
    pl = _prm(ctx, sc, wavefront, 97, 20000)
    assert pl.add_start(sc["start"]) == 0
    assert pl.add_goal(sc["goal"]) == 1
    pl.run(waves)
    states, (ef, et, ed) = pl.graph()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    ref = orc.prm(sc, sp, _params(sc, wavefront, 97, 20000), sc["lo"], sc["hi"], sc["goal"], sc["start"],
                  sc["goal"], waves)
    assert len(states) == len(ref["states"]) and len(states) > 50
    assert np.array_equal(states.view(np.int64), ref["states"].view(np.int64))
    rf, rt, rd = ref["edges"]
    assert len(ef) == len(rf) and len(ef) > 0
    assert np.array_equal(ef, rf) and np.array_equal(et, rt)
    assert np.array_equal(ed.view(np.int64), rd.view(np.int64))
    st = pl.stats()
    keys = ["wavefronts", "samples", "valid_samples", "duplicates", "links_checked", "edges", "goal_nodes", "solved"]
    assert [st[k] for k in keys] == [int(v) for v in ref["stats"]]
    path = np.array(pl.solution())
    if ref["stats"][7]:
        assert pl.last_cost == ref["cost"]
        assert np.array_equal(path.view(np.int64), ref["states"][ref["path"]].view(np.int64))
    else:
        assert len(path) == 0 and math.isinf(pl.last_cost)
    pl.close()


@pytest.mark.parametrize("mk,wavefront", [(scenes.grid_scene, 1024), (scenes.arm_scene, 2048),
                                          (scenes.mesh_scene, 512)])
def test_prm_solves_with_exact_edges(ctx, orc, mk, wavefront):
    sc = mk()
    pl = _prm(ctx, sc, wavefront, 5, 1 << 18)
    pl.add_start(sc["start"])
    pl.add_goal(sc["goal"])
    pl.solve_for(30.0, lambda: pl.solved())
    assert pl.solved()
    states, (ef, et, ed) = pl.graph()
    assert (ef > et).all()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    sel = np.arange(len(ef))[:: max(1, len(ef) // 4000)]
    ok, _ = orc.valid_edges(sc, sp, states[ef[sel]], states[et[sel]], sc["edge_step"], sc["resolution"])
    assert ok.all()
    path = np.array(pl.solution())
    assert len(path) >= 2
    assert np.array_equal(path[0], sc["start"])
    assert orc.distance(sp, path[-1], sc["goal"]) <= sc["goal_radius"]
    ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], sc["resolution"])
    assert ok.all()
    c = sum(orc.distance(sp, path[i], path[i + 1]) for i in range(len(path) - 1))
    assert abs(c - pl.last_cost) <= 1e-9 * max(1.0, c)
    pl.close()


def test_prm_errors_and_duplicates(ctx):
    import mpt_gb300 as m
    sc = scenes.grid_scene()
    pl = _prm(ctx, sc, 64, 1, 1000)
    with pytest.raises(m.MptgError):
        pl.run(1)  # no start, no goal
    assert pl.add_start(sc["start"]) == 0
    assert pl.add_start(sc["start"]) == -1  # duplicate (pprm.hpp:306-308)
    with pytest.raises(m.MptgError):
        pl.run(1)  # no goal
    ys, xs = np.nonzero(sc["grid"])
    assert pl.add_goal(np.array([float(xs[0]), float(ys[0])])) == -1  # invalid state (pprm.hpp:299-300)
    with pytest.raises(m.MptgError):
        pl.add_goal(np.array([np.nan, 5.0]))  # outside the space: an error, nothing added
    assert pl.size() == 1
    assert pl.add_goal(sc["goal"]) == 1
    pl.run(2)
    assert pl.stats()["wavefronts"] == 2
    assert pl.stats()["duplicates"] >= 1
    pl.close()
