"""GPU: the learned collision surrogate.

* forward logits and backward gradients of the device kernels against the
  CPU reference MLP (oracle/mlp.py, FP64 with the same BF16 rounding points).
  Tolerance: relative L2 error of the gradient vector < 3e-2 and cosine
  > 0.999; logits within 0.02 + 0.02|z| (BF16 operands round at 2^-8
  relative, and a rounding flip of one activation moves sums at that scale);
* training on exact-checker labels learns the SE(3) scene (held-out accuracy,
  false-positive / false-negative rates reported);
* the surrogate-culled planner returns only exact-validated paths and spends
  fewer exact checks than the plain planner for the same wavefronts; with
  surrogate-biased sampling (lowest-risk of 4 candidate edges per slot) its
  tree grows faster per wavefront and stays deterministic."""
import numpy as np
import pytest

from mpt_gb300 import scenes

pytestmark = pytest.mark.gpu


def _labelled(ctx, sc, n, seed):
    import mpt_gb300 as m
    q = np.concatenate([scenes.uniform_states(sc, n // 2, seed), scenes.near_contact_states(sc, n - n // 2, seed + 7)])
    valid = m.Scene(ctx, sc).valid(q)
    return q, (1 - valid).astype(np.uint8)  # label 1 = in collision


def test_forward_and_gradients_match_reference(ctx):
    from mpt_gb300.surrogate import Surrogate, se3_normalisation
    from oracle import mlp
    sc = scenes.mesh_scene()
    scale, shift = se3_normalisation(sc["lo"], sc["hi"])
    sg = Surrogate(ctx, 7, scale, shift, seed=3)
    rng = np.random.default_rng(0)
    x = scenes.uniform_states(sc, 512, 11)
    y = rng.integers(0, 2, 512).astype(np.uint8)
    feats = (x - shift) * scale
    p = sg.params().astype(np.float64)
    z = sg.score(x)
    zr, _ = mlp.forward(p, feats, 7)
    assert np.all(np.abs(z - zr) <= 0.02 + 0.02 * np.abs(zr)), np.abs(z - zr).max()
    loss = sg.train_step(x, y, lr=0.0)
    g = sg.grads().astype(np.float64)
    lr_, gr, _ = mlp.loss_and_grad(p, feats, y, 7)
    assert abs(loss - lr_) < 1e-3 * max(1.0, abs(lr_))
    rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
    cos = float(g @ gr / (np.linalg.norm(g) * np.linalg.norm(gr)))
    assert rel < 3e-2 and cos > 0.999, (rel, cos)
    # a step with lr > 0 moves the parameters and leaves them finite
    sg.train_step(x, y, lr=1e-3)
    p2 = sg.params()
    assert np.isfinite(p2).all() and not np.array_equal(p2, p.astype(np.float32))


def test_fused_scorer_on_ragged_batches(ctx):
    """The one-launch scorer (k_sg_score_fused: every layer on the SM, several
    128-row tiles per CTA, a partial last tile): each row's logit is the same
    bits whatever batch it is scored in, repeated calls agree, and rows from
    the start, middle and end of a 50,001-state batch match the reference MLP."""
    from mpt_gb300.surrogate import Surrogate, se3_normalisation
    from oracle import mlp
    sc = scenes.mesh_scene()
    scale, shift = se3_normalisation(sc["lo"], sc["hi"])
    sg = Surrogate(ctx, 7, scale, shift, seed=4)
    x = scenes.uniform_states(sc, 50001, 23)
    z = sg.score(x)
    assert z.shape == (50001,) and np.isfinite(z).all()
    assert np.array_equal(sg.score(x).view(np.int32), z.view(np.int32))
    for lo, hi in ((0, 1000), (20000, 20129), (49990, 50001)):
        assert np.array_equal(sg.score(x[lo:hi]).view(np.int32), z[lo:hi].view(np.int32))
    p = sg.params().astype(np.float64)
    idx = np.r_[0:200, 25000:25200, 49801:50001]
    zr, _ = mlp.forward(p, (x[idx] - shift) * scale, 7)
    assert np.all(np.abs(z[idx] - zr) <= 0.02 + 0.02 * np.abs(zr)), np.abs(z[idx] - zr).max()


@pytest.fixture(scope="module")
def trained(ctx):
    from mpt_gb300.surrogate import Surrogate, se3_normalisation
    sc = scenes.mesh_scene()
    scale, shift = se3_normalisation(sc["lo"], sc["hi"])
    q, y = _labelled(ctx, sc, 1 << 20, 21)
    sg = Surrogate(ctx, 7, scale, shift, seed=5)
    hist = sg.fit(q, y, epochs=10, batch=8192, lr=1e-3)
    return sc, sg, hist


def test_training_learns_the_scene(ctx, trained):
    sc, sg, hist = trained
    assert hist[-1] < hist[0]
    qt, yt = _labelled(ctx, sc, 32768, 99)
    pred = (sg.score(qt) > 0).astype(np.uint8)
    acc = float((pred == yt).mean())
    fp = float(((pred == 1) & (yt == 0)).sum() / max(1, (yt == 0).sum()))  # free predicted in collision
    fn = float(((pred == 0) & (yt == 1)).sum() / max(1, (yt == 1).sum()))  # collision predicted free
    print("surrogate held-out accuracy %.4f  FP %.4f  FN %.4f  loss %s" % (acc, fp, fn, hist))
    assert acc > 0.85, (acc, fp, fn)


def test_surrogate_planner_exact_paths_and_fewer_checks(ctx, orc, trained):
    from mpt_gb300 import planner as P
    sc, sg, _ = trained
    waves = 6
    stats = {}
    for mode in ("plain", "surrogate", "biased"):
        pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(4096)), seed=17, ctx=ctx, max_nodes=1 << 20)
        pl.add_start(sc["start"])
        if mode == "surrogate":
            pl.set_surrogate(sg, threshold=2.0)
        elif mode == "biased":
            pl.set_surrogate(sg, threshold=2.0, candidates=4)
        pl.run(waves)
        st = pl.stats()
        stats[mode] = st
        # every tree edge passed the exact check
        states, parents = pl.graph()
        sel = np.nonzero(parents >= 0)[0][:2000]
        sp = orc.make_space(3, 7, sc["weights"])
        ok, _ = orc.valid_edges(sc, sp, states[parents[sel]], states[sel], sc["edge_step"], 0)
        assert ok.all()
        pl.close()
    print("link states checked: plain %d, surrogate %d; nodes: plain %d, surrogate %d" % (
        stats["plain"]["link_states_checked"], stats["surrogate"]["link_states_checked"],
        stats["plain"]["tree_size"], stats["surrogate"]["tree_size"]))
    assert stats["surrogate"]["link_states_checked"] < stats["plain"]["link_states_checked"]
    # biased sampling keeps the lowest-risk of 4 candidates: more of the exact
    # checks pass, so the tree grows faster per wavefront
    assert stats["biased"]["tree_size"] > stats["plain"]["tree_size"]


def test_biased_sampling_is_deterministic(ctx, trained):
    """The same seed gives the same tree with surrogate-biased sampling."""
    from mpt_gb300 import planner as P
    sc, sg, _ = trained
    out = []
    for _ in range(2):
        pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(512)), seed=23, ctx=ctx, max_nodes=1 << 20)
        pl.add_start(sc["start"])
        pl.set_surrogate(sg, threshold=2.0, points=2, candidates=4)
        pl.run(8)
        out.append(pl.graph())
        pl.close()
    (s0, p0), (s1, p1) = out
    assert len(s0) > 100 and np.array_equal(s0, s1) and np.array_equal(p0, p1)
