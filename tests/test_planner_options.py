"""CPU: the Planner mirror's option packs and dispatch (src/mpt/prrt.hpp:56-82,
src/mpt/prrt_star.hpp:56-95, src/mpt/pprm.hpp:56-84, src/mpt/planner_tags.hpp):
options in any order, thread-count tags accepted, unknown options rejected, and
Planner(scenario, PPRM(...)) building the roadmap planner."""
import pytest

from mpt_gb300 import planner as P


def test_option_order_and_tags():
    a = P.PRRT(P.gpu_wavefront(1024), P.report_stats(True), P.max_threads(8))
    b = P.PRRT(P.max_threads(1), P.report_stats(True), P.gpu_wavefront(1024))
    assert a == b and a.wavefront == 1024 and a.report_stats
    assert P.PRRT().wavefront == 4096 and not P.PRRT().report_stats
    assert P.PRRTStar.rewire and not P.PRRT.rewire
    assert isinstance(P.PPRM(P.gpu_wavefront(512)), P.PRRT) and P.PPRM(P.gpu_wavefront(512)).wavefront == 512
    with pytest.raises(TypeError):
        P.PRRT("unknown option")


def test_planner_dispatches_pprm():
    obj = P.Planner.__new__(P.Planner, None, P.PPRM())
    assert type(obj) is P.PPRMPlanner
    assert type(P.Planner.__new__(P.Planner, None, P.PRRTStar())) is P.Planner
    assert type(P.Planner.__new__(P.Planner, None, None)) is P.Planner


def test_gpu_device_tag():
    """gpu_device(i) picks the device of the context a Planner creates when it
    is given none (the C++ header's gpu_device<i>)."""
    assert P.PRRT().device == 0
    a = P.PRRT(P.gpu_device(1), P.gpu_wavefront(64))
    assert a.device == 1 and a == P.PRRT(P.gpu_wavefront(64), P.gpu_device(1))
    assert a != P.PRRT(P.gpu_wavefront(64))
    assert P.PPRM(P.gpu_device(2)).device == 2


def test_autotune_cache_hit_needs_no_gpu(tmp_path):
    """A cached autotuner result (keyed by scene kind, metric, dimension,
    capacity bucket and candidates) is returned without running the tuner;
    other keys in the file are kept when a result is stored."""
    from mpt_gb300 import scenes
    sc = P.Scenario(scenes.grid_scene())
    cache = str(tmp_path / "tune.json")
    key = P.autotune_cache_key(sc, (256, 512), 1 << 20)
    assert key == "grid/m0/d2/n2^20/256,512"
    assert P.autotune_cache_key(sc, (256, 512), (1 << 20) + 1) != key
    P._cache_store(cache, "other", 64, {64: 0.5})
    P._cache_store(cache, key, 512, {256: 0.02, 512: 0.01})
    best, med = P.autotune_wavefront(None, sc, sc.desc["start"], candidates=(256, 512), max_nodes=1 << 20,
                                     cache=cache)
    assert best == 512 and med == {256: 0.02, 512: 0.01}
    assert set(P._cache_load(cache)) == {"other", key}
