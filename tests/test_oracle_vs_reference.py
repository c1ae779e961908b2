"""CPU: the oracle's restatement against the reference's OWN code, compiled
in place from the MPT headers (oracle/ref, skipped where the reference
sources are absent)."""
import ctypes

import numpy as np
import pytest

from mpt_gb300 import scenes

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("reference sources not present", allow_module_level=True)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.parametrize("metric,dim", [(0, 2), (0, 3), (1, 1), (1, 10)])
def test_interpolate_bit_exact(orc, metric, dim):
    L = ref.lib()
    rng = np.random.default_rng(metric * 100 + dim)
    sp = orc.make_space(metric, dim)
    lo, hi = (-np.pi, np.pi) if metric == 1 else (-50.0, 50.0)
    for _ in range(3000):
        a = rng.uniform(lo, hi, dim)
        b = rng.uniform(lo, hi, dim)
        t = float(rng.choice([rng.uniform(0, 1), rng.uniform(-3, 4), 0.0, 1.0]))
        want = np.empty(dim)
        assert L.ref_interpolate(metric, dim, _p(a), _p(b), t, _p(want)) == 0
        got = orc.interpolate(sp, a, b, t)
        assert np.array_equal(got.view(np.int64), want.view(np.int64)), (a, b, t, got, want)


def test_so3_slerp_against_glibc(orc):
    """The reference slerp calls std::acos/std::sin (glibc); the oracle and the
    device call the deterministic mptg_acos/mptg_sin.  They agree to a few ulp;
    the fraction of bit-identical results is reported."""
    L = ref.lib()
    sc = {"metric": 2, "dim": 4}
    qa = scenes.uniform_states(sc, 4000, 1)
    qb = scenes.uniform_states(sc, 4000, 2)
    sp = orc.make_space(2, 4)
    rng = np.random.default_rng(3)
    worst, same = 0.0, 0
    for i in range(len(qa)):
        t = float(rng.uniform(0, 1))
        want = np.empty(4)
        L.ref_interpolate(2, 4, _p(qa[i]), _p(qb[i]), t, _p(want))
        got = orc.interpolate(sp, qa[i], qb[i], t)
        worst = max(worst, float(np.abs(got - want).max()))
        same += int(np.array_equal(got, want))
    assert worst < 4e-15, worst
    assert same > 0.5 * len(qa), same


@pytest.mark.parametrize("mk", [scenes.grid_scene, scenes.arm_scene])
def test_dmv_bit_exact_with_sample_counts(orc, mk):
    """Booleans AND the number of valid() calls per edge match the reference's
    DiscreteMotionValidator (bisection ring queue, discrete_motion_validator.hpp:71-130)."""
    L = ref.lib()
    sc = mk()
    step = 1.0 if sc["kind"] == "grid" else 0.02
    a, b = scenes.steered_edges(sc, 400, 77)
    if sc["kind"] == "arm":
        # long edges in an obstacle-free arm scene: more than 256 interior
        # samples, all valid, exercise the queue's switch to sequential scanning
        sc = dict(sc, discs=np.zeros((0, 3)), self_collision=0)
        a = scenes.uniform_states(sc, 100, 78)
        b = scenes.uniform_states(sc, 100, 79)
        step = 0.005
    csc, keep = orc.make_scene(sc)
    n = len(a)
    out = np.empty(n, np.uint8)
    cnt = np.empty(n, np.int64)
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert L.ref_dmv_edges(ctypes.byref(csc), sc["metric"], sc["dim"], _p(a), _p(b), n, step, _p(out), _p(cnt)) == 0
    sp = orc.make_space(sc["metric"], sc["dim"])
    got = np.empty(n, np.uint8)
    gcnt = np.empty(n, np.int64)
    for i in range(n):
        g, c = orc.valid_edges(sc, sp, a[i:i + 1], b[i:i + 1], step, 0, nthreads=1)
        got[i], gcnt[i] = g[0], c
    assert np.array_equal(got, out)
    assert np.array_equal(gcnt, cnt)
    assert cnt.max() > 258 or sc["kind"] == "grid"


def test_goal_state(orc):
    L = ref.lib()
    g = np.array([1014.0, 1014.0])
    for q, r in [([1014.0, 1014.0], 8.0), ([1010.0, 1010.0], 8.0), ([1000.0, 1014.0], 8.0), ([1014.0, 1006.0], 8.0)]:
        q = np.array(q)
        d = ctypes.c_double()
        hit = L.ref_goal_l2(_p(g), r, _p(q), ctypes.byref(d))
        dist = orc.distance(orc.make_space(0, 2), q, g)
        assert hit == int(dist <= r)
        assert d.value == (0.0 if dist <= r else dist - r)


def _check_reference_solution(orc, sc, r, steered=True):
    """The acceptance rules of test/planner_integration_test.hpp:219-291 on a
    path from the reference's own planner, checked by the oracle's checker.
    steered: every edge within the range (PRRT; PRRT* rewiring and PPRM link
    k-nearest neighbours at any distance)."""
    path = r["path"]
    sp = orc.make_space(sc["metric"], sc["dim"])
    assert r["solved"] and len(path) >= 2
    assert np.array_equal(path[0], np.asarray(sc["start"], dtype=np.float64))  # the start, exactly
    assert orc.distance(sp, path[-1], sc["goal"]) <= sc["goal_radius"]
    assert orc.valid_states(sc, sp, path).all()
    ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], sc["resolution"])
    assert ok.all()
    steps = np.array([orc.distance(sp, path[i], path[i + 1]) for i in range(len(path) - 1)])
    assert not steered or (steps <= sc["range"] * (1 + 1e-12)).all()
    assert abs(steps.sum() - r["cost"]) <= 1e-9 * r["cost"]


@pytest.mark.parametrize("mk,seed,threads", [(scenes.grid_scene, 0, 1), (scenes.grid_scene, 1, 1),
                                             (scenes.grid_scene, 2, 0), (scenes.arm_scene, 0, 1)])
def test_reference_prrt_on_oracle_scenes(orc, mk, seed, threads):
    """The reference's PRRT planner (src/mpt/prrt.hpp, impl/prrt/prrt.hpp),
    compiled in place over the project-written nigh stand-in (exact brute-force
    NN), plans on the oracle's scene definitions -- valid() from the oracle,
    link() by the reference's DMV (grid) or the joint-step check (arm) -- and
    the oracle's checker accepts every path it returns.  threads 0 runs the
    reference's OpenMP worker pool with the concurrent NN container."""
    sc = mk()
    r = ref.plan_solve(sc, seed, threads=threads, time_limit_s=60.0)
    _check_reference_solution(orc, sc, r)
    assert r["nodes"] >= len(r["path"])


@pytest.mark.parametrize("mk,algo", [(scenes.grid_scene, "prrt_star"), (scenes.grid_scene, "pprm"),
                                     (scenes.arm_scene, "prrt_star"), (scenes.arm_scene, "pprm")])
def test_reference_prrt_star_and_pprm_on_oracle_scenes(orc, mk, algo):
    """The reference's PRRT* (src/mpt/prrt_star.hpp, k-nearest rewiring through
    the stand-in's nearest(nbh, q, k)) and PPRM (src/mpt/pprm.hpp: start and
    goal added, k-nearest roadmap, Dijkstra solution), single-threaded, on the
    oracle's scene definitions: the oracle's checker accepts their paths."""
    sc = mk()
    r = ref.plan_solve(sc, 1000, algo=algo, threads=1, time_limit_s=60.0)
    _check_reference_solution(orc, sc, r, steered=False)
    if algo == "pprm":
        sp = orc.make_space(sc["metric"], sc["dim"])
        assert orc.distance(sp, r["path"][-1], sc["goal"]) == 0.0  # the goal added with addGoal


def _stream_params(sc, W, seed, max_nodes=1 << 16):
    return {"range": sc["range"], "goal_bias": 0.0, "goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"],
            "resolution": sc["resolution"], "wavefront": W, "seed": seed, "max_nodes": max_nodes}


def _ids(states):
    ids = {s.tobytes(): i for i, s in enumerate(states)}
    assert len(ids) == len(states)
    return ids


@pytest.mark.parametrize("mk,nsamples", [(scenes.grid_scene, 3000), (scenes.arm_scene, 1500),
                                         (scenes.mesh_scene, 300)])
def test_reference_prrt_on_the_sample_stream_equals_the_replay(orc, mk, nsamples):
    """Fed the planners' sample stream one state at a time (goal bias 0), the
    reference's own PRRT (impl/prrt/prrt.hpp:411-452) grows exactly the tree of
    the oracle's replay at wavefront size 1: the same states bit for bit, each
    with the same parent.  (SE(3) interpolation in the reference build is the
    oracle's: MPT's Cartesian interpolate needs Eigen.)"""
    sc = mk()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    p = _stream_params(sc, 1, 11, nsamples + 1)
    st, par, _ = orc.plan(sc, sp, p, sc["lo"], sc["hi"], sc["start"], sc["goal"], nsamples, False)
    V, E, _ = ref.stream_graph(sc, p, "prrt", nsamples)
    ids = _ids(st)
    assert len(st) > 50
    assert {v.tobytes() for v in V} == set(ids) and len(V) == len(st)
    assert {(ids[a.tobytes()], ids[b.tobytes()]) for a, b in E} == {(i, int(par[i])) for i in range(1, len(st))}


@pytest.mark.parametrize("mk,nsamples", [(scenes.grid_scene, 2000), (scenes.arm_scene, 1000),
                                         (scenes.mesh_scene, 300)])
def test_reference_prrt_star_on_the_sample_stream_equals_the_replay(orc, mk, nsamples):
    """The reference's PRRT* (impl/prrt_star/prrt_star.hpp:505-657, k-nearest
    rewiring, factor 1.1) on the sample stream against the oracle's PRRT* replay
    at wavefront size 1: the same states, and on the grid and SE(3) the same
    parent for every node.  Parents may differ only where two candidates give the same
    cost: the reference orders candidates with std::sort, which is not stable,
    while the replay breaks such ties by (distance, id).  Such ties are common
    under the arm's summed SO(2) distance; there every node's cost along the
    reference's parent chain still equals the replay's (to 1e-12: the replay
    sums path costs by pointer jumping, in another order)."""
    sc = mk()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    p = _stream_params(sc, 1, 11, nsamples + 1)
    st, par, costs, _, rewires = orc.plan_star(sc, sp, p, sc["lo"], sc["hi"], sc["start"], sc["goal"], nsamples, 1.1)
    V, E, _ = ref.stream_graph(sc, p, "prrt_star", nsamples)
    ids = _ids(st)
    assert {v.tobytes() for v in V} == set(ids) and len(V) == len(st)
    rpar = np.full(len(st), -1, dtype=np.int64)
    for a, b in E:
        rpar[ids[a.tobytes()]] = ids[b.tobytes()]
    rcost = np.full(len(st), np.nan)

    def cost(i):
        chain = []
        while np.isnan(rcost[i]):
            if rpar[i] < 0:
                rcost[i] = 0.0
                break
            chain.append(i)
            i = rpar[i]
        for j in reversed(chain):
            rcost[j] = rcost[rpar[j]] + orc.distance(sp, st[rpar[j]], st[j])
        return rcost

    for i in range(len(st)):
        cost(i)
    assert np.allclose(rcost, costs, rtol=1e-12, atol=0)
    differ = np.nonzero(rpar != par)[0]
    if mk is not scenes.arm_scene:
        assert len(differ) == 0
    if mk is scenes.grid_scene:
        assert rewires > 50
    for i in differ:
        c0 = costs[par[i]] + orc.distance(sp, st[par[i]], st[i])
        c1 = costs[rpar[i]] + orc.distance(sp, st[rpar[i]], st[i])
        assert abs(c0 - c1) <= 1e-12 * c0


@pytest.mark.parametrize("mk,nsamples", [(scenes.grid_scene, 1920), (scenes.arm_scene, 6400),
                                         (scenes.mesh_scene, 128)])
def test_reference_pprm_on_the_sample_stream_equals_the_replay(orc, mk, nsamples):
    """The reference's PPRM (impl/pprm/pprm.hpp:141-371: start and goal added,
    then one sample at a time, k = ceil((e + e/dim) ln(n+1)) nearest, an edge to
    every neighbour the link accepts) fed the planners' sample stream builds
    exactly the oracle's replay roadmap -- the roadmap the GPU PPRM is tested
    equal to: the same nodes bit for bit and the same undirected edges, each
    visited from both ends -- and returns the same solution path."""
    sc = mk()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    W = 64
    p = _stream_params(sc, W, 12, 1 << 20)
    r = orc.prm(sc, sp, p, sc["lo"], sc["hi"], sc["goal"], sc["start"], sc["goal"], nsamples // W, False)
    V, E, path = ref.stream_graph(sc, p, "pprm", nsamples)
    ids = _ids(r["states"])
    ef, et, _ = r["edges"]
    assert len(ef) > 10
    assert {v.tobytes() for v in V} == set(ids) and len(V) == len(ids)
    got = [frozenset((ids[a.tobytes()], ids[b.tobytes()])) for a, b in E]
    assert len(got) == 2 * len(ef)
    assert set(got) == {frozenset((int(a), int(b))) for a, b in zip(ef, et)}
    # solution(): the reference's Dijkstra (src/mpt/impl/djikstras.hpp) and the
    # replay's (orc_prm_dijkstra) return the same path
    want = r["states"][r["path"]]
    assert len(want) > 0 or mk is scenes.mesh_scene
    assert len(path) == len(want) and np.array_equal(path.view(np.int64), want.view(np.int64))


def _near_contact_edges(sc, n, seed):
    """SE(3) edges that start near a box face (scenes.near_contact_states) and
    end within the steer range: translation toward a random state, rotation a
    fraction of the way toward a random orientation."""
    a = scenes.near_contact_states(sc, n, seed)
    c = scenes.uniform_states(sc, n, seed + 1)
    rng = np.random.default_rng(seed + 2)
    b = np.empty_like(a)
    for i in range(n):
        frac = rng.uniform(0.2, 1.0)
        dp = c[i, 4:] - a[i, 4:]
        t = min(1.0, sc["range"] * frac / max(np.linalg.norm(dp), 1e-12))
        qa, qc = a[i, :4], c[i, :4]
        if np.dot(qa, qc) < 0:
            qc = -qc
        q = qa + (qc - qa) * min(1.0, 0.5 * frac)
        b[i] = np.concatenate([q / np.linalg.norm(q), a[i, 4:] + dp * t])
    return a, b


def test_se3_dmv_with_glibc_slerp_agrees(orc):
    """The SE(3) motion check of the reference's own code -- its
    DiscreteMotionValidator over its SO(3) slerp (so3_space.hpp:44-83) and L2
    interpolate, with glibc's acos/sin and a glibc-acos metric for the step
    count -- against the oracle's, which uses the deterministic mptg_acos /
    mptg_sin (the functions the device shares).  On 1,500 edges starting at
    free states near box faces (where a last-ulp change of a sample state is most likely to flip
    a collision test), every boolean and every count of valid() calls agree:
    the two transcendental implementations do not change a single SE(3) edge
    decision on this set."""
    L = ref.lib()
    sc = scenes.mesh_scene()
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    a, b = _near_contact_edges(sc, 16000, 4242)
    free = np.nonzero(orc.valid_states(sc, sp, a) == 1)[0][:1500]  # the edge's outcome rests on its samples
    a = np.ascontiguousarray(a[free])
    b = np.ascontiguousarray(b[free])
    csc, keep = orc.make_scene(sc)
    n = len(a)
    out = np.empty(n, np.uint8)
    cnt = np.empty(n, np.int64)
    assert L.ref_dmv_edges(ctypes.byref(csc), 3, 7, _p(a), _p(b), n, sc["edge_step"], _p(out), _p(cnt)) == 0
    got = np.empty(n, np.uint8)
    gcnt = np.empty(n, np.int64)
    for i in range(n):
        g, c = orc.valid_edges(sc, sp, a[i:i + 1], b[i:i + 1], sc["edge_step"], 0, nthreads=1)
        got[i], gcnt[i] = g[0], c
    # a mixed set: both outcomes present, and edges long enough to need many samples
    assert n == 1500 and 0.1 < out.mean() < 0.9 and cnt.max() > 20
    disagree = np.nonzero((got != out) | (gcnt != cnt))[0]
    assert len(disagree) == 0, [(int(i), int(got[i]), int(out[i]), int(gcnt[i]), int(cnt[i])) for i in disagree[:10]]
