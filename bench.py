"""Benchmark of the planner hot path: exact nearest-neighbour queries against
a 1M-node tree (planar 10-link arm workload, SO(2)^10 metric), one JSON line.

A step = one batch of 65,536 seeded query states answered by the device
kd-tree (warp-per-query FP32 sweep + FP64 re-rank, bit-exact ids).  The tree
holds 1,048,576 seeded configurations inserted in batches of 65,536 (the
planner's wavefront size).  Secondary figures in the same line: edge checks/s
for the arm's DiscreteMotionValidator edges (max joint step 0.01 rad).

  value  -- queries/s with queries resident in HBM, CUDA events around each
            step, L2 flushed (256 MiB write) between steps
  e2e    -- the same metric through the C ABI with pinned host buffers
            (H2D of the queries and D2H of ids + distances inside the timing)
  --impl reference -- the CPU kd-tree of the oracle (the reference's nigh is
            not vendored) on all host cores, same tree and queries.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TREE = 1 << 20
BATCH = 65536
N_EDGES = 65536
# DRAM bytes (read + write) per query of k_nearest on the 1M-node tree, from one
# ncu capture of a 32,768-query launch: 4.589 GB read + 6.6 MB written
NN_DRAM_BYTES_PER_QUERY = (4.589e9 + 6.6e6) / 32768


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        cmd = ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
               "-lms", "200"]
        try:
            p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        try:
            while not self._stop.is_set():
                line = p.stdout.readline()
                if not line:
                    break
                parts = [x.strip() for x in line.split(",")]
                if len(parts) == 6:
                    self.samples.append(parts)
        finally:
            p.terminate()
            try:
                p.wait(timeout=2)
            except Exception:
                p.kill()

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=3)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons}


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(x: float, ws: int, device: str = "cuda") -> float:
    """The largest x over the ranks: the slowest replica sets the job's time."""
    if ws <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def _whole_job_rate(ws: int, units_per_rank_step: int, steps: int, max_seconds: float) -> float:
    """Units of all ranks per second of the slowest rank (weak scaling: every
    rank processes the same per-step work on its own replica)."""
    return ws * units_per_rank_step * steps / max_seconds


# The headline workload; both arms print this same config (the per-step query
# counts differ and are stated beside it).
NN_CONFIG = {"workload": "nn_so2x10_1M", "tree_nodes": N_TREE,
             "tree": "seeded uniform SO(2)^10 states (planar 10-link arm), inserted in batches of 65,536",
             "queries": "seeded uniform SO(2)^10 states", "answer": "exact FP64 nearest, lowest id on ties"}


def _workload(seed_base=20261205):
    from mpt_gb300 import scenes
    sc = scenes.arm_scene()
    tree_pts = scenes.uniform_states(sc, N_TREE, seed_base + 1)
    return sc, tree_pts


def _queries(sc, nbatches, seed):
    from mpt_gb300 import scenes
    return [scenes.uniform_states(sc, BATCH, seed + i) for i in range(nbatches)]


def edge_rates(ctx, m, stream, torch):
    """Edge checks/s through the batched DMV for the three scenes (device buffers)."""
    from mpt_gb300 import scenes
    out = {}
    for name, mk, n in [("grid_1024", scenes.grid_scene, 65536), ("arm_10link", scenes.arm_scene, 65536),
                        ("se3_mesh", scenes.mesh_scene, 16384)]:
        sc = mk()
        scene = m.Scene(ctx, sc)
        ea, eb = scenes.steered_edges(sc, 4096, 555)
        reps = n // len(ea)
        da = torch.from_numpy(np.tile(ea, (reps, 1))).cuda()
        db = torch.from_numpy(np.tile(eb, (reps, 1))).cuda()
        eo = torch.empty(len(da), dtype=torch.uint8, device="cuda")
        for _ in range(2):
            scene.link(da, db, sc["edge_step"], sc["resolution"], out=eo, stream=stream)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            scene.link(da, db, sc["edge_step"], sc["resolution"], out=eo, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = {"edges_per_s": len(da) * 3 / (e0.elapsed_time(e1) / 1000.0), "edges_per_launch": len(da),
                     "valid_fraction": float(eo.float().mean().item())}
        scene.close()
    return out


def _nn_alg_bytes(per, nq, D):
    """Algorithmic bytes of one k_nearest launch from its device counters: the
    FP32 coordinates of every point evaluated (4D), an internal node's record
    and cell bounds (16 + 8D), a leaf's record (16), a re-ranked candidate's
    FP64 state and point id (8D + 4; the ids of the other points are not
    read), and each query in and its answer out (8D + 12)."""
    return (per["points_evaluated"] * 4 * D + per["internal_visited"] * (16 + 8 * D) + per["leaves_visited"] * 16
            + per["reranked"] * (8 * D + 4) + nq * (8 * D + 12))


def _nn_roofline(cnt, steps, nq, D, avg_s, peak, kernel):
    """Algorithmic bytes of one NN launch from the device counters, over the
    launch time, against the HBM peak (the same formula as the headline)."""
    per = {k: v / steps for k, v in cnt.items()}
    alg = _nn_alg_bytes(per, nq, D)
    ach = alg / avg_s / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "kernel": kernel,
            "alg_bytes_per_launch": alg, "counters_per_launch": per}


def _grow_tree(ctx, sc, n, seed, W=65536):
    """A planner-grown tree: the plain wavefront PRRT on the scene (goal bias 0,
    no stop at the goal) until it holds n nodes.  Returns (planner, seconds)."""
    from mpt_gb300 import planner as P
    pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(W)), seed=seed, ctx=ctx, max_nodes=n)
    pl.set_goal_bias(0.0)
    pl.add_start(sc["start"])
    t0 = time.perf_counter()
    for _ in range(4096):
        if pl.size() >= n:
            break
        pl.run(8)
    return pl, time.perf_counter() - t0


def nn_1m_section(ctx, m, torch, steps=5, peak=None, cpu_sample=2048):
    """NN queries/s against 1,048,576-node trees of the three scenes: seeded
    uniform states (2-D grid, L2; SE(3) w = 2/1) and trees grown by the
    planner itself to 1M nodes (10-link arm, SO(2)^10; SE(3); grid).  65,536
    seeded uniform queries per step, L2 flushed between steps, CUDA events on
    the launching stream; ids and distances checked against the oracle's exact
    CPU kd-tree on a sample, which is also timed on all host cores."""
    import oracle
    from mpt_gb300 import scenes
    peak = peak or _peaks()[0]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    cores = os.cpu_count()
    out = {}
    cases = [("grid_l2_uniform", scenes.grid_scene, "uniform"), ("se3_uniform", scenes.mesh_scene, "uniform"),
             ("arm_so2x10_planner_grown", scenes.arm_scene, "grown"), ("se3_planner_grown", scenes.mesh_scene, "grown"),
             ("grid_l2_planner_grown", scenes.grid_scene, "grown")]
    for name, mk, how in cases:
        _progress("NN@1M: " + name)
        sc = mk()
        D = sc["dim"]
        pl = None
        t0 = time.perf_counter()
        if how == "uniform":
            tree = m.Tree(ctx, sc["metric"], D, N_TREE, sc["weights"])
            pts = scenes.uniform_states(sc, N_TREE, 4100 + D)
            dp = torch.from_numpy(pts).cuda()
            for lo in range(0, N_TREE, BATCH):
                tree.insert(dp[lo:lo + BATCH])
            del dp
            torch.cuda.synchronize()
        else:
            pl, _ = _grow_tree(ctx, sc, N_TREE, 4200 + D)
            tree = pl.tree()
            pts = tree.states()
        build_s = time.perf_counter() - t0
        q = scenes.uniform_states(sc, BATCH, 4300 + D)
        dq = torch.from_numpy(q).cuda()
        di = torch.empty(BATCH, dtype=torch.int32, device="cuda")
        dd = torch.empty(BATCH, dtype=torch.float64, device="cuda")
        for _ in range(3):
            tree.nearest(dq, di, dd, stream=stream)
        torch.cuda.synchronize()
        tree.counters(reset=True)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for s_, (a, b) in enumerate(ev):
            flush.fill_(s_ & 0xff)
            a.record(stream)
            tree.nearest(dq, di, dd, stream=stream)
            b.record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        cnt = tree.counters(reset=True)
        gi, gd = di[:cpu_sample].cpu().numpy(), dd[:cpu_sample].cpu().numpy()
        # the oracle's exact CPU kd-tree over the same states, all host cores
        osp = oracle.make_space(sc["metric"], D, sc["weights"])
        ot = oracle.KDTree(osp, pts, 8)
        ot.nearest(q[:64], cores)
        t1 = time.perf_counter()
        ci, cd = ot.nearest(q[:cpu_sample], cores)
        cpu_s = time.perf_counter() - t1
        avg = ms / 1000.0 / steps
        out[name] = {"tree_nodes": len(pts), "tree": how, "queries_per_step": BATCH, "steps": steps,
                     "queries_per_s": BATCH * steps / (ms / 1000.0), "ms_per_step": ms / steps,
                     "tree_build_s": build_s,
                     "roofline": _nn_roofline(cnt, steps, BATCH, D, avg, peak, "k_nearest<metric %d>" % sc["metric"]),
                     "cpu_kdtree": {"queries_per_s": cpu_sample / cpu_s, "cores": cores, "sample": cpu_sample,
                                    "kind": "port (oracle exact kd-tree, leaf 8)"},
                     "ids_equal_oracle": bool(np.array_equal(gi, ci)),
                     "max_abs_dist_err_vs_fp64_oracle": float(np.max(np.abs(gd - cd)))}
        del ot
        if pl is not None:
            tree.close()
            pl.close()
        else:
            tree.close()
    return out


def _solve_stats(ctx, sc, W, seeds, cap_s, surrogate=None, points=1, want_path=False, candidates=1):
    """p50/p99 wall time to the first solution over seeds 1000.., with the phase timers."""
    from mpt_gb300 import planner as P
    import oracle
    osp = oracle.make_space(sc["metric"], sc["dim"], sc["weights"])
    times, solved, nodes, checked, timers, seed_times = [], 0, [], [], [], []
    validated, costs, first_path = 0, [], None
    for s in range(seeds):
        pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(W)), seed=1000 + s, ctx=ctx, max_nodes=1 << 21)
        if surrogate is not None:
            pl.set_surrogate(surrogate, threshold=2.0, points=points, candidates=candidates)
        pl.add_start(sc["start"])
        pl.prepare()  # allocations outside the timing, as the reference's constructor
        t0 = time.perf_counter()
        pl.solve_for(cap_s, lambda: pl.solved())
        dt = time.perf_counter() - t0
        if pl.solved():
            solved += 1
            times.append(dt)
            # every path re-validated by the CPU checker (outside the timed region)
            path = np.array(pl.solution())
            ok, _ = oracle.valid_edges(sc, osp, path[:-1], path[1:], sc["edge_step"], sc["resolution"])
            validated += int(ok.all())
            costs.append(pl.last_cost)
            if s == 0:
                first_path = (path, pl.last_cost)
        seed_times.append(dt if pl.solved() else None)
        nodes.append(pl.size())
        checked.append(pl.stats()["link_states_checked"])
        timers.append(pl.timers())
        pl.close()
    med_t = {k: statistics.median(t[k] for t in timers) for k in timers[0]}
    res = {"wavefront": W, "seed_times_s": seed_times, "paths_validated_by_checker": validated, "median_path_cost": statistics.median(costs) if costs else None,
            "p50_s": statistics.median(times) if times else None,
            "p99_s": max(times) if times else None, "solved": solved, "seeds": seeds, "cap_s": cap_s,
            "median_nodes": statistics.median(nodes), "median_link_states_checked": statistics.median(checked),
            "median_phase_s": med_t}
    return (res, first_path) if want_path else res


SOLVE_SCENES = [("grid_1024", "grid_scene", 2048), ("arm_10link", "arm_scene", 4096), ("se3_mesh", "mesh_scene", 4096)]


def block_planner_sweep(ctx, widths=(32, 48, 64, 128), seeds=10, cap_s=20.0):
    """The persistent block planner (k_bplan_grid) on the grid: time to the first
    solution per wavefront size, with its wavefronts, its kernel time per
    wavefront and the split of that time over the phases (the block's own
    SM-cycle counters, at the bench's measured clock)."""
    from mpt_gb300 import planner as P
    from mpt_gb300 import scenes
    sc = scenes.grid_scene()
    out = {}
    for W in widths:
        times, waves, prof = [], [], []
        for s in range(seeds):
            pl = P.Planner(P.Scenario(sc), P.PRRT(P.gpu_wavefront(W)), seed=1000 + s, ctx=ctx, max_nodes=1 << 21)
            pl.add_start(sc["start"])
            pl.prepare()
            t0 = time.perf_counter()
            pl.solve_for(cap_s, lambda: pl.solved())
            dt = time.perf_counter() - t0
            if pl.solved():
                times.append(dt)
            waves.append(pl.stats()["wavefronts"])
            prof.append(pl.block_profile())
            pl.close()
        tot = {k: sum(p[k] for p in prof) for k in prof[0]}
        cyc = sum(v for k, v in tot.items() if k.startswith("cyc_"))
        out[str(W)] = {"p50_s": statistics.median(times) if times else None, "solved": len(times), "seeds": seeds,
                       "median_wavefronts": statistics.median(waves),
                       "kernel_cycles_per_wavefront": cyc / max(1.0, sum(waves)),
                       "phase_share": {k[4:]: round(v / cyc, 3) for k, v in tot.items() if k.startswith("cyc_") and cyc},
                       "fp64_fallbacks": {k: int(v) for k, v in tot.items() if not k.startswith("cyc_")}}
    return out


def solve_times(ctx, seeds=None, cap_s=20.0, tune=True):
    """Wall time to the first solution of the plain wavefront planner per scene
    (p50 over seeds 1000..), at the default wavefront and at the one the native
    autotuner picks (tuned on seeds 500.. of the same query).  seeds: per-scene
    counts (default grid 50, arm 20, SE(3) 50: the arm's solves take up to
    seconds each)."""
    from mpt_gb300 import planner as P
    from mpt_gb300 import scenes
    seeds = seeds or {"grid_1024": 50, "arm_10link": 20, "se3_mesh": 50}
    res = {}
    for name, mk, W in SOLVE_SCENES:
        sc = getattr(scenes, mk)()
        n = seeds[name] if isinstance(seeds, dict) else int(seeds)
        r = {"default": _solve_stats(ctx, sc, W, n, cap_s)}
        if tune:
            t0 = time.perf_counter()
            best, med = P.autotune_wavefront(ctx, P.Scenario(sc), sc["start"], trials=7, time_limit=1.0, seed=500)
            r["autotune"] = {"best": best, "median_s": {str(k): v for k, v in med.items()},
                             "tuning_s": time.perf_counter() - t0}
            r["tuned"] = _solve_stats(ctx, sc, best, n, cap_s)
        res[name] = r
    return res


# The reference's planners timed on this host: (scene, planner, threads) ->
# (seeds, cap s).  threads 0 = every host core (the reference's OpenMP worker
# pool); 1 = its single_threaded variant.  Bounded so the section stays within
# about two minutes: the arm and SE(3) runs are validity-bound on the CPU and
# take seconds each.
REF_PLAN_RUNS = {
    "grid_1024": {"prrt": [(1, 20, 5.0), (0, 20, 5.0)], "prrt_star": [(1, 20, 5.0), (0, 20, 5.0)],
                  "pprm": [(1, 20, 5.0), (0, 20, 5.0)]},
    "arm_10link": {"prrt": [(1, 2, 5.0), (0, 5, 5.0)], "prrt_star": [(0, 2, 5.0)],
                   "pprm": [(1, 10, 5.0), (0, 10, 5.0)]},
    "se3_mesh": {"prrt": [(0, 5, 5.0)], "prrt_star": [(0, 2, 5.0)], "pprm": [(0, 2, 5.0)]},
}


def _run_child(argv, timeout):
    """Runs this file as a child process with argv; returns (stdout, stderr,
    returncode).  A child that outlives timeout is killed and reported with
    returncode None and the lines it printed before, so one stuck run of the
    reference's code cannot end the bench."""
    try:
        p = subprocess.run([sys.executable, os.path.abspath(__file__)] + argv, capture_output=True, text=True,
                           timeout=timeout)
        return p.stdout, p.stderr, p.returncode
    except subprocess.TimeoutExpired as e:
        def _s(x):
            return x.decode(errors="replace") if isinstance(x, bytes) else (x or "")
        return _s(e.stdout), _s(e.stderr) + "\ntimed out after %g s" % timeout, None


def reference_planners(runs=None):
    """Time to the first solution of the reference's own PRRT, PRRT* and PPRM
    (src/mpt/prrt.hpp, prrt_star.hpp, pprm.hpp, compiled by oracle/ref from the
    reference headers) on the same three scenes, on this host's cores: the
    oracle's valid(), the reference's DiscreteMotionValidator (joint-step check
    on the arm), and the project-written exact NN container standing in for
    nigh (absent from the reference).  An unsolved seed counts as the cap.
    Returns None where the reference headers are not present."""
    from oracle import ref
    from mpt_gb300 import scenes
    if not ref.available():
        return None
    ref.lib()
    runs = runs or REF_PLAN_RUNS
    out = {"kind": "reference (the reference's planners compiled from its headers; NN and collision stand-ins)",
           "host_cores": os.cpu_count()}
    for name, mk, _ in SOLVE_SCENES:
        per = {}
        for algo, cfgs in runs.get(name, {}).items():
            for threads, nseeds, cap in cfgs:
                key = "%s_%s" % (algo, "1_core" if threads == 1 else "all_cores")
                _progress("reference %s %s" % (name, key))
                # each configuration in a child process: a crash inside the
                # reference's code is recorded, not fatal to the bench
                so, se, rc = _run_child(["--ref-plan-child", mk, algo, str(threads), str(nseeds), str(cap)],
                                        nseeds * (cap + 30) + 120)
                rows = [json.loads(l_) for l_ in so.splitlines() if l_.startswith("{")]
                t = sorted(r_["solve_s"] if r_["solved"] else cap for r_ in rows)
                solved = [r_ for r_ in rows if r_["solved"]]
                per[key] = {"threads": threads or os.cpu_count(), "seeds": nseeds, "cap_s": cap, "solved": len(solved),
                            "p50_s": statistics.median(t) if t else None, "max_s": t[-1] if t else None,
                            "median_cost": statistics.median([r_["cost"] for r_ in solved]) if solved else None,
                            "median_nodes": statistics.median([r_["nodes"] for r_ in solved]) if solved else None}
                if rc != 0 or len(rows) < nseeds:
                    per[key]["incomplete"] = {"seeds_finished": len(rows), "returncode": rc,
                                              "stderr_tail": se[-200:]}
        out[name] = per
    return out


def reference_serving(sample=48, cap_s=2.0, seed=20261208):
    """The serving batch's CPU baseline: the reference's own PRRT (all host
    cores, its OpenMP worker pool) answering the first `sample` queries of the
    512-query batch one after another, as one Planner per query, with the
    same starts, goals and scenes, each until its first solution or cap_s (the
    reference has no node budget).  A bounded sample of the batch; returns its
    queries/s and time-to-solution figures.  None where the reference headers
    are not present."""
    from oracle import ref
    if not ref.available():
        return None
    ref.lib()
    so, se, rc = _run_child(["--ref-serve-child", str(sample), str(cap_s), str(seed)], sample * (cap_s + 30) + 300)
    rows = [json.loads(l_) for l_ in so.splitlines() if l_.startswith("{")]
    wall = sum(r_["wall_s"] for r_ in rows)
    sol = sorted(r_["solve_s"] for r_ in rows if r_["solved"])
    per = {}
    for k in ("grid", "arm", "mesh"):
        rk = [r_ for r_ in rows if r_["kind"] == k]
        sk = sorted(r_["solve_s"] for r_ in rk if r_["solved"])
        per[k] = {"queries": len(rk), "solved": len(sk), "p50_s": sk[len(sk) // 2] if sk else None}
    out = {"kind": "reference PRRT (compiled from its headers; NN and collision stand-ins), all host cores",
           "host_cores": os.cpu_count(), "queries": len(rows), "sample_of": 512, "cap_s": cap_s,
           "wall_s": wall, "queries_per_s": len(rows) / wall if wall > 0 else None, "solved": len(sol),
           "p50_solve_s": sol[len(sol) // 2] if sol else None, "per_scene": per}
    if rc != 0 or len(rows) < sample:
        out["incomplete"] = {"queries_finished": len(rows), "returncode": rc, "stderr_tail": se[-200:]}
    return out


def _ref_serve_child(sample, cap, seed):
    """Child process of reference_serving: one JSON line per query."""
    import oracle
    from oracle import ref

    def orc_valid(d, c):
        return oracle.valid_states(d, oracle.make_space(d["metric"], d["dim"], d["weights"]), c)

    for i, (d, a, b, budget) in enumerate(_serving_pairs(512, seed, orc_valid)[:sample]):
        q = dict(d)
        q["start"], q["goal"] = a, b
        t0 = time.perf_counter()
        r_ = ref.plan_solve(q, seed + i, algo="prrt", threads=0, time_limit_s=cap)
        print(json.dumps({"i": i, "kind": d["kind"], "solved": r_["solved"], "solve_s": r_["solve_s"],
                          "wall_s": time.perf_counter() - t0}), flush=True)


def _ref_plan_child(mk, algo, threads, nseeds, cap):
    """Child process of reference_planners: one JSON line per seed."""
    from oracle import ref
    from mpt_gb300 import scenes
    sc = getattr(scenes, mk)()
    for s_ in range(nseeds):
        r_ = ref.plan_solve(sc, 1000 + s_, algo=algo, threads=threads, time_limit_s=cap)
        print(json.dumps({"seed": 1000 + s_, "solved": r_["solved"], "solve_s": r_["solve_s"], "cost": r_["cost"],
                          "nodes": r_["nodes"]}), flush=True)


def _labelled_mesh_states(m, ctx, sc, n, seed):
    """SE(3) states, half uniform and half near contact, labelled 1 = in collision by the exact checker."""
    from mpt_gb300 import scenes
    q = np.concatenate([scenes.uniform_states(sc, n // 2, seed), scenes.near_contact_states(sc, n - n // 2, seed + 7)])
    scene = m.Scene(ctx, sc)
    y = (1 - scene.valid(q)).astype(np.uint8)
    scene.close()
    return q, y


def surrogate_rates(ctx, m, torch, n_train=1 << 22, epochs=10):
    """Train the SE(3) collision surrogate on n_train labelled states and time
    training and scoring: (results, trained surrogate, scene)."""
    from mpt_gb300 import scenes
    from mpt_gb300.surrogate import Surrogate, se3_normalisation
    sc = scenes.mesh_scene()
    t0 = time.perf_counter()
    q, y = _labelled_mesh_states(m, ctx, sc, n_train, 21)
    label_s = time.perf_counter() - t0
    qt, yt = _labelled_mesh_states(m, ctx, sc, 65536, 99)
    scale, shift = se3_normalisation(sc["lo"], sc["hi"], 20.0)
    sg = Surrogate(ctx, 7, scale, shift, seed=5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = sg.fit(q, y, epochs=epochs, batch=8192, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    z = sg.score(qt)
    pred = (z > 0).astype(np.uint8)
    fp = float(((pred == 1) & (yt == 0)).sum() / max(1, (yt == 0).sum()))
    fn = float(((pred == 0) & (yt == 1)).sum() / max(1, (yt == 1).sum()))
    # scoring throughput: 65,536 device-resident states per launch
    dq = torch.from_numpy(np.ascontiguousarray(qt)).cuda()
    dz = torch.empty(len(qt), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(3):
        sg.lib.mptg_surrogate_score(sg.h, dq.data_ptr(), len(qt), dz.data_ptr(), stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nvtx = getattr(torch.cuda, "nvtx", None)
    if nvtx is not None:  # lets a profiler pick these launches (ncu --nvtx --nvtx-include sg_score/)
        nvtx.range_push("sg_score")
    e0.record(stream)
    for _ in range(10):
        sg.lib.mptg_surrogate_score(sg.h, dq.data_ptr(), len(qt), dz.data_ptr(), stream.cuda_stream)
    e1.record(stream)
    if nvtx is not None:
        nvtx.range_pop()
    torch.cuda.synchronize()
    score_s = e0.elapsed_time(e1) / 1000.0 / 10
    flops_fwd = 2.0 * (7 * 256 + 3 * 256 * 256 + 256)
    res = {"train_states": int(n_train), "label_s": label_s, "epochs": epochs, "train_s": train_s,
           "train_samples_per_s": n_train * epochs / train_s, "final_loss": hist[-1],
           "heldout_accuracy": float((pred == yt).mean()), "fp_rate": fp, "fn_rate": fn,
           "score_states_per_s": len(qt) / score_s,
           "score_tflops": flops_fwd * len(qt) / score_s / 1e12,
           "train_tflops": 3 * flops_fwd * n_train * epochs / train_s / 1e12}
    return res, sg, sc


LEARNED_MODES = (("plain", 0, 1), ("learned_new_state", 1, 1), ("learned_edge_4pts", 4, 1),
                 ("learned_biased_x4", 1, 4))


def learned_vs_plain(ctx, m, torch, seeds=50, cap_s=20.0, n_train=1 << 22, epochs=10, wavefront_tuned=None):
    """Learned collision surrogate on the SE(3) scene: training throughput, held-out
    FP/FN rates, scoring throughput against the bf16 tensor peak, and time to
    solve versus the plain planner on the same seeds: culling by the new state's
    logit, by 4 points per edge, and surrogate-biased sampling (each slot keeps
    the lowest-risk of 4 candidate edges, then the same culling).  Every solved
    path is re-validated by the CPU checker."""
    res, sg, sc = surrogate_rates(ctx, m, torch, n_train, epochs)
    # at the configured wavefront (4096) and at the autotuned one for this scene
    Ws = sorted({4096, int(wavefront_tuned or 4096)})
    for W in Ws:
        for mode, points, cand in LEARNED_MODES:
            res["%s_w%d" % (mode, W)] = _solve_stats(ctx, sc, W, seeds, cap_s, sg if points else None, points,
                                                     candidates=cand)
        plain = res["plain_w%d" % W]["p50_s"]
        res["p50_speedup_vs_plain_w%d" % W] = {mode: (plain / res["%s_w%d" % (mode, W)]["p50_s"]
                                                      if plain and res["%s_w%d" % (mode, W)]["p50_s"] else None)
                                               for mode, _, _ in LEARNED_MODES[1:]}
    return res, sg


def prrt_star_section(ctx, wave_for=None, refine_s=1.0, seeds=3):
    """PRRT* (k-nearest rewiring) against PRRT on the same seeds: time to the
    first solution, and the best path cost after refining for refine_s more."""
    from mpt_gb300 import planner as P
    from mpt_gb300 import scenes
    out = {}
    for name, mk, kind in [("grid_1024", scenes.grid_scene, "grid"), ("arm_10link", scenes.arm_scene, "arm"),
                           ("se3_mesh", scenes.mesh_scene, "mesh")]:
        sc = mk()
        W = (wave_for or {}).get(kind, 1024)
        res = {"wavefront": W}
        for label, algo in (("prrt", P.PRRT), ("prrt_star", P.PRRTStar)):
            first_t, first_c, final_c, rewires = [], [], [], []
            for s in range(seeds):
                pl = P.Planner(P.Scenario(sc), algo(P.gpu_wavefront(W)), seed=2000 + s, ctx=ctx, max_nodes=1 << 21)
                pl.add_start(sc["start"])
                pl.prepare()
                t0 = time.perf_counter()
                pl.solve_for(20.0, lambda: pl.solved())
                if not pl.solved():
                    pl.close()
                    continue
                first_t.append(time.perf_counter() - t0)
                first_c.append(pl.solution_cost())
                pl.solve_for(refine_s)
                final_c.append(pl.solution_cost())
                if algo is P.PRRTStar:
                    rewires.append(pl.rewire_stats()["rewires"])
                pl.close()
            res[label] = {"solved": len(first_t), "seeds": seeds,
                          "p50_first_solution_s": statistics.median(first_t) if first_t else None,
                          "median_first_cost": statistics.median(first_c) if first_c else None,
                          "median_cost_after_refine": statistics.median(final_c) if final_c else None,
                          "refine_s": refine_s}
            if rewires:
                res[label]["median_rewires"] = statistics.median(rewires)
        out[name] = res
    return out


def prm_section(ctx, seeds=3, cap_s=20.0):
    """PPRM (k-nearest roadmap) per scene: p50 time to the first solution and
    the path cost, and the roadmap build rate against the oracle's
    one-sample-at-a-time replay (one core) on the same sample stream, with the
    two roadmaps compared edge for edge."""
    import oracle
    from mpt_gb300 import planner as P
    from mpt_gb300 import scenes
    out = {}
    for name, mk, W, cmp_waves in [("grid_1024", scenes.grid_scene, 1024, 8), ("arm_10link", scenes.arm_scene, 4096, 2),
                                   ("se3_mesh", scenes.mesh_scene, 1024, 2)]:
        sc = mk()
        times, costs, nodes, edges, links = [], [], [], [], []
        for s in range(seeds):
            pl = P.Planner(P.Scenario(sc), P.PPRM(P.gpu_wavefront(W)), seed=3000 + s, ctx=ctx, max_nodes=1 << 21)
            t0 = time.perf_counter()
            pl.add_start(sc["start"])
            pl.add_goal(sc["goal"])
            pl.solve_for(cap_s, lambda: pl.solved())
            dt = time.perf_counter() - t0
            if pl.solved():
                times.append(dt)
                pl.solution()
                costs.append(pl.last_cost)
            st = pl.stats()
            nodes.append(pl.size())
            edges.append(st["edges"])
            links.append(st["links_checked"] / dt)
            pl.close()
        # build rate on the same sample prefix: GPU planner vs oracle replay
        pl = P.Planner(P.Scenario(sc), P.PPRM(P.gpu_wavefront(W)), seed=76, ctx=ctx, max_nodes=1 << 21)
        pl.add_start(sc["start"])
        pl.add_goal(sc["goal"])
        pl.run(1)  # warm-up
        pl.close()
        pl = P.Planner(P.Scenario(sc), P.PPRM(P.gpu_wavefront(W)), seed=77, ctx=ctx, max_nodes=1 << 21)
        t0 = time.perf_counter()
        pl.add_start(sc["start"])
        pl.add_goal(sc["goal"])
        pl.run(cmp_waves)
        gpu_s = time.perf_counter() - t0
        _, (gf, gt, gd) = pl.graph()
        n_gpu = pl.size()
        pl.close()
        sp = oracle.make_space(sc["metric"], sc["dim"], sc["weights"])
        params = {"goal_radius": sc["goal_radius"], "edge_step": sc["edge_step"], "resolution": sc["resolution"],
                  "wavefront": W, "seed": 77, "max_nodes": 1 << 21}
        oracle.prm(sc, sp, params, sc["lo"], sc["hi"], sc["goal"], sc["start"], sc["goal"], 1)
        t0 = time.perf_counter()
        ref = oracle.prm(sc, sp, params, sc["lo"], sc["hi"], sc["goal"], sc["start"], sc["goal"], cmp_waves)
        cpu_s = time.perf_counter() - t0
        rf, rt, rd = ref["edges"]
        out[name] = {"wavefront": W, "solved": len(times), "seeds": seeds,
                     "p50_first_solution_s": statistics.median(times) if times else None,
                     "median_path_cost": statistics.median(costs) if costs else None,
                     "median_nodes": statistics.median(nodes), "median_edges": statistics.median(edges),
                     "median_links_checked_per_s": statistics.median(links),
                     "build": {"samples": cmp_waves * W, "gpu_samples_per_s": cmp_waves * W / gpu_s,
                               "cpu_oracle_samples_per_s": cmp_waves * W / cpu_s, "cpu_cores": 1,
                               "roadmap_equal": bool(n_gpu == len(ref["states"]) and np.array_equal(gf, rf)
                                                     and np.array_equal(gt, rt) and np.array_equal(gd, rd))}}
    return out


def _serving_pairs(n, seed, valid):
    """The serving benchmark's queries without a GPU: per query its scene kind,
    start, goal and node budget, the starts and goals rejection-sampled valid
    by valid(desc, states) -> 1/0 per state (the GPU's validity or the
    oracle's, which agree bit for bit)."""
    from mpt_gb300 import scenes
    rng = np.random.default_rng(seed)
    descs = [scenes.grid_scene(), scenes.arm_scene(), scenes.mesh_scene()]
    kinds = rng.integers(0, 3, n)
    pools = []
    for k, d in enumerate(descs):
        need = 2 * int((kinds == k).sum())
        got = []
        s = 0
        while sum(len(g) for g in got) < need:
            c = scenes.uniform_states(d, 8 * need + 64, seed + 17 * k + s)
            got.append(c[valid(d, c) == 1])
            s += 1
        pools.append(np.concatenate(got)[:need])
    used = [0, 0, 0]
    out = []
    for i in range(n):
        k = int(kinds[i])
        a, b = pools[k][used[k]], pools[k][used[k] + 1]
        used[k] += 2
        budget = int(round(math.exp(rng.uniform(math.log(1000), math.log(200000)))))
        out.append((descs[k], a, b, budget))
    return out


def batch_queries(m, ctx, n, seed=20261208, time_limit=10.0, wave_for=None, surrogate=None):
    """Config of the serving benchmark: n queries uniform over the three scenes,
    start and goal rejection-sampled valid, node budgets log-uniform in
    [1k, 200k]; wavefront = the scene's autotuned size (wave_for[kind]) when
    given, else budget/16 clipped to [256, 4096]; at most budget/4.  Off the
    grid a wavefront is several kernels and host round trips (0.3-1 ms), so
    there the size grows with the budget to at least budget/128: a query that
    cannot be solved within its budget then ends after about 128 wavefronts
    instead of a thousand (the grid's persistent block planner runs a
    wavefront in microseconds and keeps the tuned size)."""
    from mpt_gb300 import planner as P
    from mpt_gb300.batch import Query

    def gpu_valid(d, c):
        scene = m.Scene(ctx, d)
        try:
            return scene.valid(c)
        finally:
            scene.close()

    qs = []
    for i, (d, a, b, budget) in enumerate(_serving_pairs(n, seed, gpu_valid)):
        W = wave_for[d["kind"]] if wave_for else min(4096, max(256, budget // 16))
        if d["kind"] != "grid":
            W = min(4096, max(W, budget // 128))
        W = int(max(1, min(W, budget // 4)))
        sc = P.Scenario(d, P.GoalState(d["goal_radius"], b))
        q = Query(sc, a, seed=seed + i, max_nodes=budget, wavefront=W, time_limit=time_limit)
        if surrogate is not None and d["kind"] == "mesh":  # the surrogate is trained on the SE(3) scene
            q.surrogate, q.threshold, q.surrogate_candidates = surrogate, 2.0, 4
        qs.append(q)
    return qs


def batch_serving(m, ctx, n=512, concurrency=8, seq_sample=64, wave_for=None, surrogate=None):
    """Batched multi-query serving: queries/s and time to solution over n queries
    with `concurrency` concurrent planners, against the same planner running the
    queries one after another (on the first seq_sample queries).  The grid
    queries run together as one persistent launch, a thread block each; with a
    surrogate, the SE(3) queries use surrogate-biased sampling and culling."""
    from mpt_gb300.batch import plan_batch
    qs = batch_queries(m, ctx, n, wave_for=wave_for, surrogate=surrogate)
    plan_batch(ctx, qs[:8], concurrency=concurrency)  # warm-up: planners, kernels
    t0 = time.perf_counter()
    r = plan_batch(ctx, qs, concurrency=concurrency)
    wall = time.perf_counter() - t0
    sol = sorted(x["solve_s"] for x in r if x["solved"])
    kinds = [q.scenario.desc["kind"] for q in qs]
    per = {}
    for k in ("grid", "arm", "mesh"):
        idx = [i for i in range(n) if kinds[i] == k]
        sk = sorted(r[i]["solve_s"] for i in idx if r[i]["solved"])
        per[k] = {"queries": len(idx), "solved": len(sk), "p50_s": sk[len(sk) // 2] if sk else None}
    t0 = time.perf_counter()
    rs = plan_batch(ctx, qs[:seq_sample], concurrency=1)
    seq_wall = time.perf_counter() - t0
    t0 = time.perf_counter()
    plan_batch(ctx, qs[:seq_sample], concurrency=concurrency)
    conc_wall = time.perf_counter() - t0
    same = all(a["solved"] == b["solved"] and a["nodes"] == b["nodes"] for a, b in zip(r[:seq_sample], rs))
    return {"queries": n, "concurrency": concurrency, "wall_s": wall, "queries_per_s": n / wall,
            "solved": len(sol), "p50_solve_s": sol[len(sol) // 2] if sol else None,
            "p99_solve_s": sol[min(len(sol) - 1, int(0.99 * len(sol)))] if sol else None,
            "per_scene": per, "time_limit_s": qs[0].time_limit,
            "sequential_sample": {"queries": seq_sample, "sequential_queries_per_s": seq_sample / seq_wall,
                                  "concurrent_queries_per_s": seq_sample / conc_wall,
                                  "results_identical": bool(same)}}


def run_reference(args):
    """CPU kd-tree (oracle port) on all host cores, bounded sample per step."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    import oracle
    sc, pts = _workload()
    sp = oracle.make_space(sc["metric"], sc["dim"])
    t0 = time.perf_counter()
    tree = oracle.KDTree(sp, pts, 8)
    build_s = time.perf_counter() - t0
    cores = os.cpu_count()
    sample = 4096
    qs = _queries(sc, 1, 777)[0][:sample]
    for _ in range(max(1, args.warmup)):
        tree.nearest(qs[:512], cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tree.nearest(qs, cores)
        times.append(time.perf_counter() - t0)
    qps = sample * len(times) / sum(times)
    line = {"metric": "NN queries/s @1M nodes (SO(2)^10, 10-link arm)", "value": qps, "unit": "queries/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform SO(2)^10 states)",
            "config": dict(NN_CONFIG), "queries_per_step": sample,
            "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": cores, "kind": "port",
                             "sample": "%d queries per step against the full 1,048,576-node tree" % sample},
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "tree_build_s": build_s}
    print(json.dumps(line))


def _progress(msg):
    """One line per bench section on stderr (the JSON line goes to stdout)."""
    sys.stderr.write("[bench %.1fs] %s\n" % (time.perf_counter() - _T0, msg))
    sys.stderr.flush()


_T0 = time.perf_counter()


class SectionBudget:
    """The secondary sections run while the bench is within budget_s seconds
    of its start (t0); one due later is skipped and listed in `skipped`
    (section -> seconds elapsed), so the one JSON line is printed however slow
    the host or the box is."""

    def __init__(self, budget_s, t0=None):
        self.budget_s = budget_s
        self.t0 = _T0 if t0 is None else t0
        self.skipped = {}

    def due(self, what):
        el = time.perf_counter() - self.t0
        if el <= self.budget_s:
            return True
        self.skipped[what] = round(el, 1)
        _progress("skipped %s (%.0f s elapsed, budget %.0f s)" % (what, el, self.budget_s))
        return False


def run_gpu(args):
    import torch
    import mpt_gb300 as m
    ws, rank, local = _dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    ctx = m.Context(local)
    if (args.edges_only or args.solve_only or args.star_only or args.prm_only or args.sg_only or args.nn1m_only
            or args.bplan_only):
        # profiling modes: one secondary section alone
        if args.nn1m_only:
            out = {"nn_1m": nn_1m_section(ctx, m, torch)}
        elif args.edges_only:
            out = {"edge_checks": edge_rates(ctx, m, torch.cuda.current_stream(), torch)}
        elif args.star_only:
            out = {"prrt_star": prrt_star_section(ctx)}
        elif args.prm_only:
            out = {"pprm": prm_section(ctx)}
        elif args.sg_only:
            out = {"surrogate": surrogate_rates(ctx, m, torch, n_train=1 << 18, epochs=1)[0]}
        elif args.bplan_only:
            out = {"block_planner": block_planner_sweep(ctx, seeds=args.solve_seeds or 10)}
        else:
            out = {"time_to_solve": solve_times(ctx, seeds=args.solve_seeds)}
            if not args.no_ref_planners:
                out["reference_planners"] = reference_planners()
        out["gpu_launches"] = ctx.kernel_launches()
        if rank == 0:
            print(json.dumps(out))
        return
    budget = SectionBudget(args.budget_s)
    due, skipped = budget.due, budget.skipped

    _progress("headline tree")
    sc, pts = _workload()
    tree = m.Tree(ctx, sc["metric"], sc["dim"], N_TREE)
    t0 = time.perf_counter()
    dpts = torch.from_numpy(pts).cuda()
    for lo in range(0, N_TREE, BATCH):
        tree.insert(dpts[lo:lo + BATCH])
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    del dpts

    nbuf = 4
    nqb = min(args.queries, BATCH)
    hq = [x[:nqb] for x in _queries(sc, nbuf, 1000 + 97 * rank)]
    dq = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in hq]
    di = torch.empty(nqb, dtype=torch.int32, device="cuda")
    dd = torch.empty(nqb, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    for i in range(max(3, args.warmup)):
        tree.nearest(dq[i % nbuf], di, dd, stream=stream)
    torch.cuda.synchronize()
    tree.counters(reset=True)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = ctx.kernel_launches()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for s in range(args.steps):
            flush.fill_(s & 0xff)  # L2 flush between steps (outside the events)
            starts[s].record(stream)
            tree.nearest(dq[s % nbuf], di, dd, stream=stream)
            ends[s].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    launches = ctx.kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = sum(step_ms)
    total_ms = _max_over_ranks(total_ms, ws)
    cnt = tree.counters(reset=True)
    value = _whole_job_rate(ws, nqb, args.steps, total_ms / 1000.0)

    # roofline of k_nearest: algorithmic bytes per launch from the device counters
    D = sc["dim"]
    per_launch = {k: v / args.steps for k, v in cnt.items()}
    alg_bytes = _nn_alg_bytes(per_launch, nqb, D)
    avg_s = total_ms / 1000.0 / args.steps
    peak, peak_kind = _peaks()
    achieved = alg_bytes / avg_s / 1e9
    if args.nn_only:
        if rank == 0:
            print(json.dumps({"metric": "NN queries/s (profiling case)", "value": value, "unit": "queries/s",
                              "queries_per_step": nqb, "steps": args.steps, "ms_per_step": total_ms / args.steps,
                              "alg_bytes_per_launch": alg_bytes, "achieved_gbs": achieved,
                              "counters_per_launch": per_launch, "gpu_launches": launches}))
        return

    _progress("headline e2e")
    # end to end through the C ABI with pinned host buffers
    hq_pinned = [torch.from_numpy(x).pin_memory() for x in hq]
    hi = torch.empty(nqb, dtype=torch.int32).pin_memory()
    hd = torch.empty(nqb, dtype=torch.float64).pin_memory()
    qn = [x.numpy() for x in hq_pinned]
    for i in range(3):
        ctx.lib.mptg_nearest(tree.h, qn[i % nbuf].ctypes.data, nqb, hi.data_ptr(), hd.data_ptr(), None)
    torch.cuda.synchronize()
    e2e_t = []
    for s in range(args.steps):
        flush.fill_(s & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = ctx.lib.mptg_nearest(tree.h, qn[s % nbuf].ctypes.data, nqb, hi.data_ptr(), hd.data_ptr(), None)
        e2e_t.append(time.perf_counter() - t0)
        assert st == 0
    e2e_total = _max_over_ranks(sum(e2e_t), ws)
    e2e_val = _whole_job_rate(ws, nqb, args.steps, e2e_total)
    # results of the host path equal the device path
    assert np.array_equal(hi.numpy(), tree.nearest(hq[(args.steps - 1) % nbuf])[0])

    # secondary figures: NN@1M on the other scenes and on planner-grown trees,
    # edge checks/s (three scenes) and time to solve
    _progress("NN@1M of the other scenes")
    nn1m = nn_1m_section(ctx, m, torch, peak=_peaks()[0]) if not args.no_nn1m and due("nn_1m") else None
    _progress("edge checks")
    edges = edge_rates(ctx, m, stream, torch)
    _progress("time to solve")
    solves = solve_times(ctx) if not args.no_solve and due("time_to_solve") else None
    _progress("block planner sweep")
    bplan = block_planner_sweep(ctx) if not args.no_solve and due("block_planner_grid") else None
    w_se3 = solves["se3_mesh"]["autotune"]["best"] if solves and "autotune" in solves["se3_mesh"] else None
    _progress("learned surrogate")
    learned, sg = (learned_vs_plain(ctx, m, torch, wavefront_tuned=w_se3)
                   if not (args.no_solve or args.no_learned) and due("learned_surrogate_se3") else (None, None))
    wave_for = None
    if solves and all("autotune" in solves[k] for k in solves):
        wave_for = {"grid": solves["grid_1024"]["autotune"]["best"], "arm": solves["arm_10link"]["autotune"]["best"],
                    "mesh": solves["se3_mesh"]["autotune"]["best"]}
    _progress("batched serving")
    serving = None
    if not (args.no_solve or args.no_batch) and due("batch_serving"):
        serving = {"plain": batch_serving(m, ctx, wave_for=wave_for)}
        if sg is not None and due("batch_serving.surrogate"):
            _progress("batched serving with the surrogate")
            serving["surrogate"] = batch_serving(m, ctx, wave_for=wave_for, surrogate=sg)
    _progress("PRRT*")
    star = prrt_star_section(ctx, wave_for) if not (args.no_solve or args.no_star) and due("prrt_star") else None
    _progress("PPRM")
    prm = prm_section(ctx) if not (args.no_solve or args.no_prm) and due("pprm") else None

    _progress("CPU baselines")
    # CPU baselines: oracle kd-tree and DMV on the host cores, bounded samples;
    # the reference's own DMV and planners where its headers are present
    cpu = None
    ref_plans = None
    if rank == 0:
        import oracle
        from oracle import ref as oref
        from mpt_gb300 import scenes
        for name, mk in [("grid_1024", scenes.grid_scene), ("arm_10link", scenes.arm_scene),
                         ("se3_mesh", scenes.mesh_scene)]:
            scx = mk()
            ea, eb = scenes.steered_edges(scx, 4096, 555)
            osp = oracle.make_space(scx["metric"], scx["dim"], scx["weights"])
            oracle.valid_edges(scx, osp, ea[:64], eb[:64], scx["edge_step"], scx["resolution"])
            t0 = time.perf_counter()
            want, _ = oracle.valid_edges(scx, osp, ea, eb, scx["edge_step"], scx["resolution"])
            edges[name]["cpu_edges_per_s"] = len(ea) / (time.perf_counter() - t0)
            edges[name]["cpu_cores"] = os.cpu_count()
            if scx["resolution"] == 0 and oref.available():
                # the reference's DiscreteMotionValidator itself (the arm's joint-step
                # check has no reference counterpart: its demo bisects in L-infinity)
                oref.dmv_edges(scx, ea[:64], eb[:64], scx["edge_step"])
                t0 = time.perf_counter()
                got, _ = oref.dmv_edges(scx, ea, eb, scx["edge_step"])
                edges[name]["reference_dmv_edges_per_s"] = len(ea) / (time.perf_counter() - t0)
                edges[name]["reference_dmv_equals_oracle"] = bool(np.array_equal(got, want))
        if not args.no_solve and not args.no_ref_planners and due("reference_planners"):
            _progress("reference planners")
            ref_plans = reference_planners()
            if serving is not None and due("batch_serving.reference_sample"):
                _progress("reference serving sample")
                serving["reference_sample"] = reference_serving()
        osp = oracle.make_space(sc["metric"], sc["dim"])
        ot = oracle.KDTree(osp, pts, 8)
        sample = 2048
        cores = os.cpu_count()
        ot.nearest(hq[0][:256], cores)
        t0 = time.perf_counter()
        ci, cd = ot.nearest(hq[0][:sample], cores)
        cpu_s = time.perf_counter() - t0
        gi, gd = tree.nearest(hq[0][:sample])
        cpu = {"value": sample / cpu_s, "unit": "queries/s", "cores": cores, "kind": "port",
               "sample": "%d queries against the full 1,048,576-node tree" % sample,
               "ids_equal_gpu": bool(np.array_equal(ci, gi)),
               "max_abs_dist_err_vs_fp64_oracle": float(np.max(np.abs(gd - cd)))}

    if rank == 0:
        line = {"metric": "NN queries/s @1M nodes (SO(2)^10, 10-link arm)", "value": value, "unit": "queries/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded uniform SO(2)^10 states)",
                "config": dict(NN_CONFIG), "queries_per_step": nqb,
                "l2": "flushed (256 MiB write) between steps", "parallelism": "replicas",
                "e2e": {"value": e2e_val, "unit": "queries/s", "h2d_bytes_per_step": nqb * D * 8,
                        "d2h_bytes_per_step": nqb * 12},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": NN_DRAM_BYTES_PER_QUERY * nqb,
                             "traffic_source": "ncu dram__bytes_read+write of a 32,768-query launch, scaled by "
                                               "queries (profiles/k_nearest_so2x10_1M.md)",
                             "peak_source": peak_kind,
                             "kernel": "k_nearest<SO2,10>", "alg_bytes_per_launch": alg_bytes,
                             "counters_per_launch": per_launch},
                "cpu_baseline": cpu,
                "nn_1m": nn1m,
                "edge_checks": {"unit": "edges/s", "per_scene": edges,
                                "cpu_kind": "port (oracle DMV + exact validity, all host cores)",
                                "reference_kind": "the reference's DiscreteMotionValidator over the oracle's valid(), "
                                                  "all host cores"},
                "time_to_solve": {"unit": "s", "planner": "plain wavefront PRRT (GPU)", "per_scene": solves,
                                  "reference_planners": ref_plans, "block_planner_grid": bplan},
                "learned_surrogate_se3": learned,
                "batch_serving": serving,
                "prrt_star": star,
                "pprm": prm,
                "clocks": clk.summary(), "gpu_launches": launches, "tree_build_s": build_s,
                "wall_s_timed": wall}
        if skipped:
            line["skipped_sections"] = {"budget_s": args.budget_s, "elapsed_s_at_skip": skipped}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    import faulthandler
    faulthandler.enable()  # a native crash prints the Python stack on stderr
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--queries", type=int, default=BATCH, help="queries per step (profiling: a smaller case)")
    ap.add_argument("--nn-only", action="store_true", help="time the NN kernel only (profiling)")
    ap.add_argument("--no-solve", action="store_true", help="skip the time-to-solve, surrogate and serving runs")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-surrogate comparison")
    ap.add_argument("--no-nn1m", action="store_true", help="skip the NN@1M runs of the other scenes")
    ap.add_argument("--no-ref-planners", action="store_true", help="skip timing the reference's own planners")
    ap.add_argument("--nn1m-only", action="store_true", help="the NN@1M runs of the other scenes only (profiling)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched serving run")
    ap.add_argument("--no-star", action="store_true", help="skip the PRRT* comparison")
    ap.add_argument("--star-only", action="store_true", help="the PRRT* comparison only (profiling)")
    ap.add_argument("--no-prm", action="store_true", help="skip the PPRM roadmap run")
    ap.add_argument("--prm-only", action="store_true", help="the PPRM roadmap run only (profiling)")
    ap.add_argument("--sg-only", action="store_true",
                    help="surrogate training (262,144 states, 1 epoch) and scoring rates only (profiling)")
    ap.add_argument("--edges-only", action="store_true", help="edge checks/s of the three scenes only (profiling)")
    ap.add_argument("--bplan-only", action="store_true", help="the block planner's wavefront sweep only (profiling)")
    ap.add_argument("--solve-only", action="store_true", help="time to solve of the three scenes only (profiling)")
    ap.add_argument("--budget-s", type=float, default=900.0,
                    help="seconds from the start after which the secondary sections are skipped")
    ap.add_argument("--solve-seeds", type=int, default=None, help="seeds per scene (default grid 50, arm 20, SE(3) 50)")
    ap.add_argument("--ref-plan-child", nargs=5, default=None, help=argparse.SUPPRESS)
    ap.add_argument("--ref-serve-child", nargs=3, default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.ref_plan_child:
        mk, algo, threads, nseeds, cap = args.ref_plan_child
        _ref_plan_child(mk, algo, int(threads), int(nseeds), float(cap))
        return
    if args.ref_serve_child:
        sample, cap, seed = args.ref_serve_child
        _ref_serve_child(int(sample), float(cap), int(seed))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
