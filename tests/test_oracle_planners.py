"""CPU: the oracle's planner replays (test infrastructure the GPU planners are
checked against) hold the reference's invariants on their own -- PRRT's tree
(src/mpt/impl/prrt/prrt.hpp:411-452): every parent precedes its child, every
edge passes the DMV, goal nodes lie within the goal radius; PRRT*
(src/mpt/impl/prrt_star/prrt_star.hpp:505-657): the rewired graph stays a tree
whose costs are its path lengths, and its first solution is no costlier."""
import numpy as np

from mpt_gb300 import scenes


def _params(sc, W, seed, max_nodes=20000):
    return {"range": sc["range"], "goal_bias": 0.05, "goal_radius": sc["goal_radius"],
            "edge_step": sc["edge_step"], "resolution": sc["resolution"], "wavefront": W, "seed": seed,
            "max_nodes": max_nodes}


def test_prrt_replay_tree_invariants(orc):
    sc = scenes.grid_scene()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    st, par, goals = orc.plan(sc, sp, _params(sc, 256, 11), sc["lo"], sc["hi"], sc["start"], sc["goal"], 12, False)
    n = len(st)
    assert n > 500 and par[0] == -1 and (par[1:] >= 0).all() and (par[1:] < np.arange(1, n)).all()
    ok, _ = orc.valid_edges(sc, sp, st[par[1:]], st[1:], sc["edge_step"], sc["resolution"])
    assert ok.all()
    # steering: no new node is farther than the range from its parent
    d = np.array([orc.distance(sp, st[par[i]], st[i]) for i in range(1, n)])
    assert (d <= sc["range"] * (1 + 1e-12)).all() and (d > 0).all()
    for g in goals:
        assert orc.distance(sp, st[g], sc["goal"]) <= sc["goal_radius"]


def test_prrt_star_replay_costs_are_path_lengths(orc):
    sc = scenes.grid_scene()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    st, par, costs, goals, rewires = orc.plan_star(sc, sp, _params(sc, 256, 11), sc["lo"], sc["hi"], sc["start"],
                                                   sc["goal"], 12)
    n = len(st)
    assert n > 500 and rewires > 0
    sel = np.nonzero(par >= 0)[0]
    ok, _ = orc.valid_edges(sc, sp, st[par[sel]], st[sel], sc["edge_step"], sc["resolution"])
    assert ok.all()
    for x in sel[:: max(1, len(sel) // 200)]:
        c, y, hops = 0.0, x, 0
        while par[y] >= 0:
            c += orc.distance(sp, st[par[y]], st[y])
            y = par[y]
            hops += 1
            assert hops <= n
        assert y == 0
        assert abs(c - costs[x]) <= 1e-9 * max(1.0, c)
    # the same samples without rewiring reach the start by paths at least as long
    st0, par0, _ = orc.plan(sc, sp, _params(sc, 256, 11), sc["lo"], sc["hi"], sc["start"], sc["goal"], 12, False)
    assert len(st0) == n and np.array_equal(st0.view(np.int64), st.view(np.int64))

    def cost0(x):
        c = 0.0
        while par0[x] >= 0:
            c += orc.distance(sp, st0[par0[x]], st0[x])
            x = par0[x]
        return c

    for x in sel[:: max(1, len(sel) // 100)]:
        assert costs[x] <= cost0(x) * (1 + 1e-12)


def test_replay_kdtree_nn_equals_brute_force(orc):
    """The kd-tree option of the replays (used to time the CPU planner) builds
    the same trees as the brute-force definition."""
    for mk, W, waves in ((scenes.grid_scene, 512, 8), (scenes.arm_scene, 1024, 3), (scenes.mesh_scene, 128, 3)):
        sc = mk()
        sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
        p = _params(sc, W, 5)
        try:
            orc.set_plan_nn(True)
            a = orc.plan(sc, sp, p, sc["lo"], sc["hi"], sc["start"], sc["goal"], waves, False)
        finally:
            orc.set_plan_nn(False)
        b = orc.plan(sc, sp, p, sc["lo"], sc["hi"], sc["start"], sc["goal"], waves, False)
        assert len(a[0]) == len(b[0]) > 20
        assert np.array_equal(a[0].view(np.int64), b[0].view(np.int64))
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
