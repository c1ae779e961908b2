"""CPU: the oracle's PPRM restatement (orc_prm) against the reference's
addSample rules (src/mpt/impl/pprm/pprm.hpp:298-339): the neighbourhood size,
the one-at-a-time neighbourhoods, exact edges, components and the Dijkstra
path (src/mpt/impl/djikstras.hpp)."""
import math

import numpy as np

from mpt_gb300 import scenes


def test_prm_k_formula(orc):
    for dim in (2, 7, 10):
        for n in (1, 2, 10, 1000, 10 ** 6, 10 ** 9):
            e = math.e + math.e / dim
            want = min(64, n, max(1, math.ceil(e * math.log(n + 1))))
            assert orc.prm_k(n, dim) == want
    assert orc.prm_k(0, 2) == 0


def test_prm_roadmap_rules(orc):
    sc = scenes.grid_scene()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    params = {"goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"], "resolution": sc["resolution"],
              "wavefront": 128, "seed": 11, "max_nodes": 5000}
    r = orc.prm(sc, sp, params, sc["lo"], sc["hi"], sc["goal"], sc["start"], sc["goal"], 10)
    X = r["states"]
    ef, et, ed = r["edges"]
    n = len(X)
    assert n > 200 and len(ef) > n
    assert (ef > et).all()
    # each node's edges go to its k nearest among the nodes before it
    for i in range(2, n, max(1, n // 40)):
        d = np.array([orc.distance(sp, X[i], X[j]) for j in range(i)])
        k = orc.prm_k(i, 2)
        nb = np.lexsort((np.arange(i), d))[:k]
        mine = et[ef == i]
        assert set(mine.tolist()) <= set(nb.tolist())
        for j, dist in zip(et[ef == i], ed[ef == i]):
            assert dist == d[j]
    ok, _ = orc.valid_edges(sc, sp, X[ef], X[et], sc["edge_step"], sc["resolution"])
    assert ok.all()
    # solved iff the start (node 0) reaches a goal node; the path is a chain of edges
    adj = [[] for _ in range(n)]
    for a, b in zip(ef.tolist(), et.tolist()):
        adj[a].append(b)
        adj[b].append(a)
    seen, stack = {0}, [0]
    while stack:
        u = stack.pop()
        for v in adj[u]:
            if v not in seen:
                seen.add(v)
                stack.append(v)
    goals = {i for i in range(n) if orc.distance(sp, X[i], sc["goal"]) <= sc["goal_radius"]}
    assert bool(r["stats"][7]) == bool(seen & goals)
    assert r["stats"][6] == len(goals)
    if r["stats"][7]:
        p = r["path"]
        assert p[0] == 0 and p[-1] in goals
        edges = set(zip(ef.tolist(), et.tolist()))
        c = 0.0
        for a, b in zip(p[:-1], p[1:]):
            assert (max(a, b), min(a, b)) in edges
            c += orc.distance(sp, X[a], X[b])
        assert abs(c - r["cost"]) <= 1e-9 * c


def test_dijkstra_reference_known_answer(orc):
    """The graph of test/djikstras_test.cpp:55-101 (seven vertices, eleven
    undirected weighted edges, start 0, goal 4): the shortest path is
    0-1-3-2-4."""
    edges = [(0, 1, 1.0), (1, 3, 2.0), (0, 3, 3.1), (2, 4, 4.0), (0, 4, 10.3), (3, 2, 3.0), (0, 2, 6.2),
             (0, 5, 1.5), (5, 6, 9.5), (6, 4, 9.9), (1, 2, 7.0)]
    flags = [1, 0, 0, 0, 2, 0, 0]
    path, cost = orc.prm_dijkstra(7, flags, [e[0] for e in edges], [e[1] for e in edges], [e[2] for e in edges])
    assert list(path) == [0, 1, 3, 2, 4]
    assert cost == ((1.0 + 2.0) + 3.0) + 4.0
