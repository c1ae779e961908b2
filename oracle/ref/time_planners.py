"""Time to first solution of the reference's own planners (PRRT, PRRT*, PPRM),
compiled in place by oracle/ref, on the synthetic grid, planar-arm and SE(3)
scenes -- TEST INFRASTRUCTURE ONLY, and only where the reference sources exist.

    python -m oracle.ref.time_planners [--scenes grid,arm,se3] [--algos prrt]
        [--threads 1,0] [--seeds 20] [--cap 20]

One JSON line per (scene, planner, threads): solved count, p50 / p99 / max
seconds (an unsolved seed counts as the cap), median path cost and median node
count of the solved seeds.  Seeds are 1000, 1001, ...; threads 0 = every
OpenMP thread.  The nearest-neighbour structure is the exact brute-force
stand-in for nigh and the SE(3) collision check is the oracle's AABB-tree
triangle test standing in for FCL, so these are the reference's planners over
the oracle's checkers, not over its original libraries.
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", default="grid,arm,se3")
    ap.add_argument("--algos", default="prrt")
    ap.add_argument("--threads", default="1,0")
    ap.add_argument("--seeds", type=int, default=20)
    ap.add_argument("--cap", type=float, default=20.0)
    a = ap.parse_args(argv)

    from mpt_gb300 import scenes

    from . import available, plan_solve

    if not available():
        raise SystemExit("reference sources not present")
    makers = {"grid": scenes.grid_scene, "arm": scenes.arm_scene, "se3": scenes.mesh_scene}
    for name in a.scenes.split(","):
        sc = makers[name]()
        for algo in a.algos.split(","):
            for th in (int(t) for t in a.threads.split(",")):
                rows = [plan_solve(sc, 1000 + s, algo=algo, threads=th, time_limit_s=a.cap) for s in range(a.seeds)]
                t = np.array([r["solve_s"] if r["solved"] else a.cap for r in rows])
                solved = [r for r in rows if r["solved"]]
                print(json.dumps({
                    "scene": name, "planner": algo, "threads": th or os.cpu_count(), "cap_s": a.cap,
                    "solved": len(solved), "of": len(rows),
                    "p50_s": float(np.median(t)), "p99_s": float(np.percentile(t, 99)), "max_s": float(t.max()),
                    "median_cost": float(np.median([r["cost"] for r in solved])) if solved else None,
                    "median_nodes": float(np.median([r["nodes"] for r in solved])) if solved else None,
                }), flush=True)


if __name__ == "__main__":
    main()
