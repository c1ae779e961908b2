"""CPU, two gloo ranks: the host side of `bench.py --gpus N` (replicas only) --
rank/world parsing, the max-over-ranks timing rule, the whole-job rate, and
the reference arm's rule that only rank 0 runs and prints; and on one process
the bench's section time budget and its child-process time limit."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(ws),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        w, r, local = bench._dist_env()
        assert (w, r, local) == (ws, rank, rank)
        # rank r takes 100 + 50 r ms: the job's time is the slowest rank's
        t = bench._max_over_ranks(100.0 + 50.0 * rank, w, device="cpu")
        rate = bench._whole_job_rate(w, 65536, 10, t / 1000.0)

        class Args:
            gpus, steps, warmup = ws, 1, 1
        printed = None
        if rank != 0:
            import io
            import contextlib
            buf = io.StringIO()
            with contextlib.redirect_stdout(buf):
                bench.run_reference(Args())  # ranks other than 0 exit without work
            printed = buf.getvalue()
        out[rank] = (t, rate, printed)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_rate():
    ws = 2
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    t0, rate0, _ = out[0]
    t1, rate1, printed1 = out[1]
    assert t0 == t1 == 150.0
    assert rate0 == rate1 == 2 * 65536 * 10 / 0.15
    assert printed1 == ""


def test_reference_arm_line(monkeypatch, capsys):
    """`bench.py --impl reference` on rank 0: one JSON line with the contract's keys,
    the reference marker, and an e2e without device copies (a smaller tree here)."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "N_TREE", 20000)
    monkeypatch.setattr(bench, "BATCH", 4096)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)

    class Args:
        gpus, steps, warmup = 1, 2, 1
    bench.run_reference(Args())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"] == bench.NN_CONFIG  # the same config as the GPU arm's line
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_section_budget_and_child_timeout():
    """The bench's secondary sections stop starting once its time budget is
    spent (each skipped one is listed), and a reference child run that outlives
    its limit is reported (returncode None, what it printed kept) instead of
    ending the bench."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    b = bench.SectionBudget(60.0, t0=time.perf_counter())
    assert b.due("nn_1m") and b.skipped == {}
    b = bench.SectionBudget(1.0, t0=time.perf_counter() - 5.0)
    assert not b.due("pprm") and not b.due("prrt_star")
    assert set(b.skipped) == {"pprm", "prrt_star"} and all(v >= 5.0 for v in b.skipped.values())
    so, se, rc = bench._run_child(["--ref-serve-child", "2", "0.5", "1"], 0.3)
    assert rc is None and "timed out after 0.3 s" in se


def test_nn_roofline_bytes_formula():
    """The headline roofline's algorithmic bytes per k_nearest launch: FP32
    coordinates of each point evaluated (4D), an internal node's record and
    cell bounds (16 + 8D), a leaf record (16), a re-ranked candidate's FP64
    state and id (8D + 4), and each query in and answer out (8D + 12)."""
    sys.path.insert(0, ROOT)
    import bench
    D = 10
    per = {"points_evaluated": 1000, "internal_visited": 100, "leaves_visited": 40, "reranked": 3}
    want = 1000 * 40 + 100 * 96 + 40 * 16 + 3 * 84 + 2 * 92
    assert bench._nn_alg_bytes(per, 2, D) == want
    assert bench._nn_alg_bytes({k: 0 for k in per}, 0, D) == 0
