"""GPU parity: batched Scenario::valid and DiscreteMotionValidator edges
through the C ABI against the oracle (bit-exact booleans)."""
import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scene(ctx, sc):
    import mpt_gb300 as m
    return m.Scene(ctx, sc)


@pytest.mark.parametrize("mk", [scenes.grid_scene, scenes.arm_scene])
def test_states_match_oracle(ctx, orc, mk):
    sc = mk()
    q = scenes.uniform_states(sc, 20000, 401)
    if sc["kind"] == "grid":
        # include cell boundaries (x.5), the grid border and outside points
        extra = np.array([[0.5, 0.5], [1023.5, 10.0], [1023.49, 10.0], [-0.5, 3.0], [-1.0, 3.0], [1024.0, 1024.0],
                          [-0.99, -0.99], [511.5, 511.5], [np.nan, 3.0], [1e300, 2.0]])
        q = np.concatenate([q, extra])
    g = _scene(ctx, sc)
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    want = orc.valid_states(sc, sp, q)
    got = g.valid(q)
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    assert 0.01 < want.mean() < 0.99


@pytest.mark.parametrize("mk", [scenes.grid_scene, scenes.arm_scene])
def test_edges_match_oracle(ctx, orc, mk):
    sc = mk()
    a, b = scenes.steered_edges(sc, 4000, 402)
    g = _scene(ctx, sc)
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    want, _ = orc.valid_edges(sc, sp, a, b, sc["edge_step"], sc["resolution"])
    got = g.link(a, b, sc["edge_step"], sc["resolution"])
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    assert 0.01 < want.mean() < 0.99


def test_arm_states_on_the_collision_boundary(ctx, orc):
    """States bisected to within ~1e-10 rad of the collision boundary: the FP32
    filter must defer them to FP64, and the answers must equal the oracle's."""
    sc = scenes.arm_scene()
    sp = orc.make_space(1, 10)
    rng = np.random.default_rng(5)
    q = scenes.uniform_states(sc, 4000, 601)
    v = orc.valid_states(sc, sp, q)
    good, bad = q[v == 1][:150], q[v == 0][:150]
    lo, hi = good.copy(), bad.copy()  # lo valid, hi invalid
    for _ in range(34):
        mid = lo + 0.5 * (hi - lo)
        mv = orc.valid_states(sc, sp, mid).astype(bool)
        lo[mv] = mid[mv]
        hi[~mv] = mid[~mv]
    pts = np.concatenate([lo, hi, lo + 1e-12 * rng.normal(size=lo.shape), hi + 1e-12 * rng.normal(size=hi.shape)])
    pts = np.clip(pts, -np.pi, np.pi)
    g = _scene(ctx, sc)
    want = orc.valid_states(sc, sp, pts)
    got = g.valid(pts)
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    # edges ending on the boundary take the same exact path
    a = np.repeat(good[:1], len(pts), axis=0)
    wante, _ = orc.valid_edges(sc, sp, a, pts, 0.01, 1)
    gote = g.link(a, pts, 0.01, 1)
    assert np.array_equal(gote, wante)


def _near_contact_states(sc, n, seed):
    """SE(3) states whose robot sits within about one bounding radius of a box face."""
    rng = np.random.default_rng(seed)
    boxes = sc["boxes"]
    out = scenes.uniform_states(sc, n, seed + 1)
    for i in range(n):
        lo, hi = boxes[rng.integers(len(boxes))]
        p = rng.uniform(lo, hi)
        ax = rng.integers(3)
        side = rng.integers(2)
        p[ax] = (hi if side else lo)[ax] + (1 if side else -1) * rng.uniform(0.3, 1.2) * sc["robot_bound"]
        out[i, 4:] = p
    return out


def test_mesh_states_match_oracle(ctx, orc):
    sc = scenes.mesh_scene()
    q = np.concatenate([scenes.uniform_states(sc, 3000, 501), _near_contact_states(sc, 3000, 502)])
    g = _scene(ctx, sc)
    sp = orc.make_space(3, 7, sc["weights"])
    want = orc.valid_states(sc, sp, q)
    got = g.valid(q)
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    assert 0.05 < want.mean() < 0.95


def test_mesh_edges_match_oracle(ctx, orc):
    sc = scenes.mesh_scene()
    a, b = scenes.steered_edges(sc, 1500, 503)
    near = _near_contact_states(sc, 500, 504)
    a = np.concatenate([a, near])
    b = np.concatenate([b, near + np.concatenate([np.zeros((500, 4)), np.full((500, 3), 0.4)], 1)])
    g = _scene(ctx, sc)
    sp = orc.make_space(3, 7, sc["weights"])
    want, _ = orc.valid_edges(sc, sp, a, b, sc["edge_step"], 0)
    got = g.link(a, b, sc["edge_step"], 0)
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    assert 0.05 < want.mean() < 0.95


def test_edges_degenerate(ctx, orc):
    sc = scenes.grid_scene()
    g = _scene(ctx, sc)
    sp = orc.make_space(0, 2)
    a = np.array([[10.0, 10.0], [10.0, 10.0], [10.0, 10.0], [100.0, 500.0]])
    b = np.array([[10.0, 10.0], [10.5, 10.0], [10.0, 200.0], [100.0, 500.0 + 1e-9]])
    want, _ = orc.valid_edges(sc, sp, a, b, 1.0)
    got = g.link(a, b, 1.0)
    assert np.array_equal(got, want)


def test_arm_long_edges(ctx, orc):
    """Edges up to pi per joint (hundreds of samples, several warp rounds)."""
    sc = scenes.arm_scene()
    rng = np.random.default_rng(7)
    a = scenes.uniform_states(sc, 600, 403)
    b = scenes.uniform_states(sc, 600, 404)
    g = _scene(ctx, sc)
    sp = orc.make_space(1, 10)
    want, _ = orc.valid_edges(sc, sp, a, b, 0.01, 1)
    got = g.link(a, b, 0.01, 1)
    assert np.array_equal(got, want)
    # also the space-metric resolution (reference DMV semantics)
    want0, _ = orc.valid_edges(sc, sp, a, b, 0.05, 0)
    got0 = g.link(a, b, 0.05, 0)
    assert np.array_equal(got0, want0)
    assert rng is not None
