"""GPU: the wavefront PRRT and PRRT* at wavefront size 1 replay the oracle
bit for bit.  At that size the oracle's replays grow the same trees as MPT's
own PRRT and PRRT* fed the same sample stream (tests/test_oracle_vs_reference.py),
so these cases carry that equality onto the device."""
import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _params(sc, seed, max_nodes):
    return {"range": sc["range"], "goal_bias": 0.0, "goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"],
            "resolution": sc["resolution"], "wavefront": 1, "seed": seed, "max_nodes": max_nodes}


def _planner(ctx, sc, algo, seed, max_nodes):
    from mpt_gb300 import planner as P
    pl = P.Planner(P.Scenario(sc), algo(P.gpu_wavefront(1)), seed=seed, ctx=ctx, max_nodes=max_nodes)
    pl.set_goal_bias(0.0)
    pl.add_start(sc["start"])
    return pl


@pytest.mark.parametrize("mk,waves", [(scenes.grid_scene, 3000), (scenes.arm_scene, 1500), (scenes.mesh_scene, 300)])
def test_prrt_wavefront_one_replays_oracle(ctx, orc, mk, waves):
    from mpt_gb300 import planner as P
    sc = mk()
    pl = _planner(ctx, sc, P.PRRT, 11, waves + 1)
    pl.run(waves)
    states, parents = pl.graph()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    ws, wp, _ = orc.plan(sc, sp, _params(sc, 11, waves + 1), sc["lo"], sc["hi"], sc["start"], sc["goal"], waves, False)
    assert len(states) == len(ws) and len(ws) > 50
    assert np.array_equal(states.view(np.int64), ws.view(np.int64))
    assert np.array_equal(parents, wp)
    pl.close()


@pytest.mark.parametrize("mk,waves", [(scenes.grid_scene, 2000), (scenes.arm_scene, 1000)])
def test_prrt_star_wavefront_one_replays_oracle(ctx, orc, mk, waves):
    from mpt_gb300 import planner as P
    sc = mk()
    pl = _planner(ctx, sc, P.PRRTStar, 11, waves + 1)
    pl.run(waves)
    states, parents = pl.graph()
    costs = pl.costs()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    ws, wp, wc, _, nrw = orc.plan_star(sc, sp, _params(sc, 11, waves + 1), sc["lo"], sc["hi"], sc["start"],
                                       sc["goal"], waves)
    assert len(states) == len(ws) and len(ws) > 200
    assert np.array_equal(states.view(np.int64), ws.view(np.int64))
    assert np.array_equal(parents, wp)
    assert np.array_equal(costs.view(np.int64), wc.view(np.int64))
    assert pl.rewire_stats()["rewires"] == nrw
    pl.close()
