"""Planner<Scenario, PRRT<options...>> mirror over the wavefront planner.

Mirrors the reference's planner interface (src/mpt/planner.hpp:46-47,
src/mpt/prrt.hpp:56-82, src/mpt/impl/prrt/prrt.hpp:149-316,
src/mpt/impl/planner_base.hpp:58-80): ``add_start`` / ``addStart``,
``solve(done_fn)``, ``solve_for`` / ``solveFor``, ``solve_until`` /
``solveUntil``, ``solved``, ``size``, ``set_range`` / ``get_range``,
``set_goal_bias`` / ``get_goal_bias``, ``solution()`` / ``solution(fn)``,
``print_stats`` / ``printStats`` and ``visit_graph`` / ``visitGraph``.

Scenarios follow the reference contract (space, bounds, valid, link, goal)
through a GPU description of their collision world: ``Scenario(scene_dict)``
for the grid, planar-arm and rigid-mesh scene kinds of mpt_gb300.scenes.

Option tags: ``gpu_wavefront(W)`` (samples per wavefront), ``report_stats(b)``;
the thread-count tags of planner_tags.hpp (``max_threads``,
``single_threaded``, ``hardware_concurrency``) are accepted and have no effect
because wavefronts replace the worker pool.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import time

import numpy as np

from . import Context, MptgError, Scene, Tree, _check, load


# ------------------------------------------------------------------ option tags
class gpu_wavefront:  # noqa: N801 (reference tag naming)
    def __init__(self, n: int):
        self.n = int(n)


class report_stats:  # noqa: N801
    def __init__(self, enabled: bool = True):
        self.enabled = bool(enabled)


class max_threads:  # noqa: N801
    def __init__(self, n: int):
        self.n = int(n)


class gpu_device:  # noqa: N801
    """The CUDA device a planner creates its context on when none is given."""

    def __init__(self, index: int):
        self.index = int(index)


single_threaded = max_threads(1)
hardware_concurrency = max_threads(0)


class PRRT:
    """Option pack (src/mpt/prrt.hpp:56-71); order of options does not matter."""

    rewire = False

    def __init__(self, *options):
        self.wavefront = 4096
        self.report_stats = False
        self.device = 0
        for o in options:
            if isinstance(o, gpu_wavefront):
                self.wavefront = o.n
            elif isinstance(o, report_stats):
                self.report_stats = o.enabled
            elif isinstance(o, gpu_device):
                self.device = o.index
            elif isinstance(o, max_threads):
                pass
            else:
                raise TypeError("unknown PRRT option %r" % (o,))

    def __eq__(self, other):
        return isinstance(other, PRRT) and (self.wavefront, self.report_stats, self.device) == (
            other.wavefront, other.report_stats, other.device)


class PRRTStar(PRRT):
    """Option pack of PRRTStar (src/mpt/prrt_star.hpp:56-95): the wavefront
    planner with k-nearest rewiring (rewire_k_nearest, the reference default)."""

    rewire = True


class PPRM(PRRT):
    """Option pack of PPRM (src/mpt/pprm.hpp:56-84): the parallel k-nearest
    probabilistic roadmap (Planner(scenario, PPRM(...)) builds a PPRMPlanner)."""


class GoalState:
    """GoalState(radius, state) (src/mpt/goal_state.hpp:43-90)."""

    def __init__(self, radius: float, state):
        self.radius = float(radius)
        self.state = np.asarray(state, dtype=np.float64)


class Scenario:
    """A scenario described for the GPU: scene dict + goal + bounds + link resolution."""

    def __init__(self, desc: dict, goal: GoalState | None = None):
        self.desc = desc
        self.goal = goal if goal is not None else GoalState(desc.get("goal_radius", 1e-6), desc["goal"])
        self.lo = np.asarray(desc["lo"], dtype=np.float64)
        self.hi = np.asarray(desc["hi"], dtype=np.float64)
        self.edge_step = float(desc["edge_step"])
        self.resolution = int(desc.get("resolution", 0))
        self.default_range = float(desc.get("range", math.inf))


class _Params(ctypes.Structure):
    _fields_ = [("range", ctypes.c_double), ("goal_bias", ctypes.c_double), ("goal_radius", ctypes.c_double),
                ("edge_step", ctypes.c_double), ("resolution", ctypes.c_int), ("wavefront", ctypes.c_int),
                ("seed", ctypes.c_uint64), ("max_nodes", ctypes.c_size_t)]


def _sig(L):
    if getattr(L, "_planner_sig", False):
        return
    P, S = ctypes.c_void_p, ctypes.c_size_t
    for name, res, args in [
        ("mptg_planner_create", ctypes.c_int, [P, P, P, P, P, ctypes.POINTER(P)]),
        ("mptg_planner_destroy", ctypes.c_int, [P]),
        ("mptg_planner_add_start", ctypes.c_int, [P, P]),
        ("mptg_planner_set_goal", ctypes.c_int, [P, P, ctypes.c_double]),
        ("mptg_planner_run", ctypes.c_int, [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
        ("mptg_planner_size", ctypes.c_int, [P, ctypes.POINTER(S)]),
        ("mptg_planner_goals", ctypes.c_int, [P, ctypes.POINTER(S)]),
        ("mptg_planner_solution", ctypes.c_int, [P, P, S, ctypes.POINTER(S), ctypes.POINTER(ctypes.c_double)]),
        ("mptg_planner_graph", ctypes.c_int, [P, P, P, S, ctypes.POINTER(S)]),
        ("mptg_planner_tree", ctypes.c_int, [P, ctypes.POINTER(P)]),
        ("mptg_planner_set_persistent", ctypes.c_int, [P, ctypes.c_int]),
        ("mptg_planner_set_block_search", ctypes.c_int, [P, ctypes.c_longlong]),
        ("mptg_planner_graph_runs", ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint64)]),
        ("mptg_planner_stats", ctypes.c_int, [P, P]),
        ("mptg_planner_timers", ctypes.c_int, [P, P]),
        ("mptg_planner_block_profile", ctypes.c_int, [P, P]),
        ("mptg_planner_set_rewire", ctypes.c_int, [P, ctypes.c_int, ctypes.c_double]),
        ("mptg_planner_rewire_stats", ctypes.c_int, [P, P]),
        ("mptg_planner_costs", ctypes.c_int, [P, P, S, ctypes.POINTER(S)]),
        ("mptg_autotune_wavefront", ctypes.c_int, [P, P, P, P, P, P, P, ctypes.c_double, P, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int), P]),
        ("mptg_prm_create", ctypes.c_int, [P, P, P, P, P, P, ctypes.POINTER(P)]),
        ("mptg_prm_destroy", ctypes.c_int, [P]),
        ("mptg_prm_add_start", ctypes.c_int, [P, P, ctypes.POINTER(ctypes.c_int32)]),
        ("mptg_prm_add_goal", ctypes.c_int, [P, P, ctypes.POINTER(ctypes.c_int32)]),
        ("mptg_prm_run", ctypes.c_int, [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
        ("mptg_prm_size", ctypes.c_int, [P, ctypes.POINTER(S), ctypes.POINTER(S)]),
        ("mptg_prm_graph", ctypes.c_int, [P, P, S, P, P, P, S, ctypes.POINTER(S), ctypes.POINTER(S)]),
        ("mptg_prm_solution", ctypes.c_int, [P, P, S, ctypes.POINTER(S), ctypes.POINTER(ctypes.c_double)]),
        ("mptg_prm_stats", ctypes.c_int, [P, P]),
    ]:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L._planner_sig = True


class Planner:
    """Planner<Scenario, PRRT<...>>(scenario, seed) on one GPU; with a PPRM
    option pack the planner is a PPRMPlanner."""

    def __new__(cls, scenario=None, algorithm=None, *args, **kwargs):
        if cls is Planner and isinstance(algorithm, PPRM):
            return super().__new__(PPRMPlanner)
        return super().__new__(cls)

    def __init__(self, scenario: Scenario, algorithm: PRRT | None = None, seed: int | None = None,
                 ctx: Context | None = None, max_nodes: int = 1 << 20):
        self.lib = load()
        _sig(self.lib)
        self.algorithm = algorithm or PRRT()
        self.ctx = ctx or Context(self.algorithm.device)
        self.scenario = scenario
        if seed is None:  # RandomDeviceSeed: fresh entropy (src/mpt/random_device_seed.hpp:62-88)
            seed = int.from_bytes(np.random.default_rng().bytes(8), "little")
        self.seed = int(seed) & ((1 << 64) - 1)
        self.max_nodes = int(max_nodes)
        self._range = scenario.default_range
        self._goal_bias = 0.01
        self._rewire_factor = 1.1
        self._starts = []
        self._surrogate = None
        self._persistent = 1
        self._brute_pairs = None
        self.scene = Scene(self.ctx, scenario.desc)
        self.h = None

    def set_persistent(self, on: bool):
        """Run wavefronts inside the persistent block planner where it applies
        (grid scenes, wavefront <= 1024; the default) or always as separate
        kernels (False).  The two build the same tree."""
        self._persistent = 1 if on else 0
        if self.h is not None:
            _check(self.ctx.h, self.lib.mptg_planner_set_persistent(self.h, self._persistent))

    def set_block_search(self, brute_pairs: int):
        """The block planner's nearest search: wavefronts with W x nodes up to
        brute_pairs sweep every node, larger ones search a bucket grid; the
        answers are the same (mptg_planner_set_block_search)."""
        self._brute_pairs = int(brute_pairs)
        if self.h is not None:
            _check(self.ctx.h, self.lib.mptg_planner_set_block_search(self.h, self._brute_pairs))

    def set_surrogate(self, surrogate, threshold: float = 0.0, points: int = 1, candidates: int = 1):
        """Cull edges the surrogate scores above `threshold` (collision logit)
        before the exact check: the new state and points-1 interior states of
        each candidate edge are scored.  candidates > 1: each wavefront slot
        keeps the lowest-risk of that many candidate edges (surrogate-biased
        sampling).  None removes it."""
        self._surrogate = ((surrogate, float(threshold), int(points), int(candidates)) if surrogate is not None
                           else None)
        if self.h is not None:
            self._apply_surrogate()

    def _apply_surrogate(self):
        from . import surrogate as S
        S._sig(self.lib)
        sg, thr, pts, cand = self._surrogate if self._surrogate else (None, 0.0, 1, 1)
        _check(self.ctx.h, self.lib.mptg_planner_set_surrogate_points(self.h, pts))
        _check(self.ctx.h, self.lib.mptg_planner_set_surrogate_bias(self.h, cand))
        _check(self.ctx.h, self.lib.mptg_planner_set_surrogate(self.h, sg.h if sg else None, thr))

    # -- configuration (prrt.hpp:159-175)
    def set_range(self, r: float):
        assert r > 0
        self._range = float(r)
        self._require_fresh("set_range")

    def get_range(self) -> float:
        return self._range

    def set_goal_bias(self, b: float):
        assert 0 <= b <= 1
        self._goal_bias = float(b)
        self._require_fresh("set_goal_bias")

    def set_rewire_factor(self, f: float):
        """PRRTStar::setRewireFactor (src/mpt/impl/prrt_star/prrt_star.hpp:234-240)."""
        assert f > 0
        self._rewire_factor = float(f)
        self._require_fresh("set_rewire_factor")

    def get_rewire_factor(self) -> float:
        return self._rewire_factor

    def get_goal_bias(self) -> float:
        return self._goal_bias

    def _require_fresh(self, what):
        if self.h is not None:
            raise RuntimeError("%s must be called before the first solve" % what)

    # -- tree
    def add_start(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        if self.h is None:
            self._starts.append(q)
        else:
            _check(self.ctx.h, self.lib.mptg_planner_add_start(self.h, q.ctypes.data))

    def prepare(self):
        """Create the device planner now -- its tree, buffers and the starts
        added so far -- as the reference's constructor and addStart do, so
        that the first solve does not pay for the allocations."""
        self._create()

    def _create(self):
        if self.h is not None:
            return
        sc = self.scenario
        prm = _Params()
        prm.range = self._range if math.isfinite(self._range) else 0.0
        prm.goal_bias = self._goal_bias
        prm.goal_radius = sc.goal.radius
        prm.edge_step = sc.edge_step
        prm.resolution = sc.resolution
        prm.wavefront = self.algorithm.wavefront
        prm.seed = self.seed
        prm.max_nodes = self.max_nodes
        h = ctypes.c_void_p()
        _check(self.ctx.h, self.lib.mptg_planner_create(self.ctx.h, self.scene.h, ctypes.byref(prm),
                                                        sc.lo.ctypes.data, sc.hi.ctypes.data, ctypes.byref(h)))
        self.h = h
        _check(self.ctx.h, self.lib.mptg_planner_set_persistent(h, self._persistent))
        if self._brute_pairs is not None:
            _check(self.ctx.h, self.lib.mptg_planner_set_block_search(h, self._brute_pairs))
        g = np.ascontiguousarray(sc.goal.state, dtype=np.float64)
        _check(self.ctx.h, self.lib.mptg_planner_set_goal(h, g.ctypes.data, sc.goal.radius))
        if self.algorithm.rewire:
            _check(self.ctx.h, self.lib.mptg_planner_set_rewire(h, 1, self._rewire_factor))
        for q in self._starts:
            _check(self.ctx.h, self.lib.mptg_planner_add_start(h, q.ctypes.data))
        self._starts = []
        if self._surrogate:
            self._apply_surrogate()

    # -- solving (planner_base.hpp:58-80, prrt.hpp:194-201)
    def run(self, max_wavefronts: int = 1, time_limit: float = 0.0, stop_when_solved: bool = False) -> bool:
        self._create()
        solved = ctypes.c_int(0)
        _check(self.ctx.h, self.lib.mptg_planner_run(self.h, int(max_wavefronts), float(time_limit),
                                                     int(stop_when_solved), ctypes.byref(solved)))
        return bool(solved.value)

    # seconds of wavefronts per call between polls of done_fn: each call also
    # stops at the first solution, so a solve until solved() ends on the
    # wavefront that finds it; a call runs at least one wavefront
    POLL_SECONDS = 0.005

    def solve(self, done_fn, deadline: float | None = None):
        """Runs wavefronts until done_fn() is true: polled between calls of up
        to POLL_SECONDS of wavefronts, each of which ends early at the first
        solution or at the deadline (time.monotonic()), or when the node
        budget is reached."""
        if self.size() == 0:
            raise RuntimeError("there are no valid initial states")
        self._create()
        while not done_fn():
            limit = self.POLL_SECONDS
            if deadline is not None:
                left = deadline - time.monotonic()
                if left <= 0:
                    break
                limit = min(limit, left)
            self.run(0, time_limit=limit, stop_when_solved=not self.solved())
            if self.size() >= self.max_nodes:  # node budget reached
                break

    def solve_for(self, seconds: float, done_fn=None):
        deadline = time.monotonic() + seconds
        self.solve_until(deadline, done_fn)

    def solve_until(self, deadline: float, done_fn=None):
        if done_fn is None:
            self.solve(lambda: time.monotonic() >= deadline, deadline)
        else:
            self.solve(lambda: time.monotonic() >= deadline or done_fn(), deadline)

    def solved(self) -> bool:
        if self.h is None:
            return False
        n = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_planner_goals(self.h, ctypes.byref(n)))
        return n.value > 0

    def size(self) -> int:
        if self.h is None:
            return len(self._starts)
        n = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_planner_size(self.h, ctypes.byref(n)))
        return n.value

    # -- results (prrt.hpp:208-316)
    def solution(self, fn=None):
        if self.h is None:
            return []
        n = ctypes.c_size_t()
        cost = ctypes.c_double()
        _check(self.ctx.h, self.lib.mptg_planner_solution(self.h, None, 0, ctypes.byref(n), ctypes.byref(cost)))
        D = self.scene.dim
        path = np.empty((n.value, D), dtype=np.float64)
        if n.value:
            _check(self.ctx.h, self.lib.mptg_planner_solution(self.h, path.ctypes.data, n.value, ctypes.byref(n),
                                                              ctypes.byref(cost)))
        self.last_cost = cost.value
        if fn is None:
            return [p for p in path]
        for p in path:
            fn(p)
        return None

    def solution_cost(self) -> float:
        self.solution()
        return self.last_cost

    def graph(self):
        n = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_planner_graph(self.h, None, None, 0, ctypes.byref(n)))
        states = np.empty((n.value, self.scene.dim), dtype=np.float64)
        parents = np.empty(n.value, dtype=np.int32)
        _check(self.ctx.h, self.lib.mptg_planner_graph(self.h, states.ctypes.data, parents.ctypes.data, n.value,
                                                       ctypes.byref(n)))
        return states, parents

    def tree(self):
        """The planner's nearest-neighbour tree (PRRT's nn_, prrt.hpp:121-122) as a
        borrowed ``Tree``: nearest / nearest_k / counters on the planner-grown
        tree.  Owned by the planner; valid while the planner is open."""
        self._create()
        h = ctypes.c_void_p()
        _check(self.ctx.h, self.lib.mptg_planner_tree(self.h, ctypes.byref(h)))
        return Tree.borrow(self.ctx, h, self.scene.metric, self.scene.dim, self.scene.weights, owner=self)

    def visit_graph(self, visitor):
        states, parents = self.graph()
        for i in range(len(states)):
            visitor.vertex(states[i])
            if parents[i] >= 0:
                visitor.edge(states[parents[i]])

    def stats(self) -> dict:
        out = (ctypes.c_double * 8)()
        _check(self.ctx.h, self.lib.mptg_planner_stats(self.h, out))
        keys = ["wavefronts", "samples", "nodes_added", "tree_size", "goals", "link_states_checked", "seconds",
                "wavefront_counter"]
        return dict(zip(keys, [float(v) for v in out]))

    def graph_runs(self) -> int:
        """Block-planner runs replayed through the planner's captured CUDA graph."""
        n = ctypes.c_uint64(0)
        if self.h is not None:
            _check(self.ctx.h, self.lib.mptg_planner_graph_runs(self.h, ctypes.byref(n)))
        return int(n.value)

    def block_profile(self) -> dict:
        """The persistent block planner's SM cycles per phase and FP64 fallback
        counts, summed over its runs (mptg_planner_block_profile)."""
        out = (ctypes.c_double * 9)()
        _check(self.ctx.h, self.lib.mptg_planner_block_profile(self.h, out))
        # cyc_nearest covers each sample's steer and link set-up as well;
        # cyc_steer and cyc_link_setup stay zero
        keys = ["cyc_sample", "cyc_nearest", "cyc_steer", "cyc_link_setup", "cyc_link_samples", "cyc_insert",
                "near_ties_fp64", "samples_fp64", "step_counts_fp64"]
        return dict(zip(keys, [float(v) for v in out]))

    def costs(self) -> np.ndarray:
        """Each node's cost (PRRTStar only)."""
        n = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_planner_costs(self.h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.float64)
        _check(self.ctx.h, self.lib.mptg_planner_costs(self.h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def rewire_stats(self) -> dict:
        out = (ctypes.c_double * 6)()
        _check(self.ctx.h, self.lib.mptg_planner_rewire_stats(self.h, out))
        return {"rewires": int(out[0]), "rewire_tests": int(out[1]), "knn_s": out[2], "choose_s": out[3],
                "rewire_s": out[4], "costs_s": out[5]}

    def timers(self) -> dict:
        """Seconds per phase on the GPU timeline (WorkerStats' nearest / validMotion
        timers, src/mpt/impl/prrt/prrt.hpp:72-101)."""
        out = (ctypes.c_double * 4)()
        _check(self.ctx.h, self.lib.mptg_planner_timers(self.h, out))
        return dict(zip(["nearest", "surrogate", "valid_motion", "insert"], [float(v) for v in out]))

    def print_stats(self):
        s = self.stats() if self.h is not None else {}
        print("nodes in graph: %d" % self.size())
        if self.solved():
            self.solution()
            print("solutions: %d, best cost=%g" % (s.get("goals", 0), self.last_cost))
        if self.algorithm.report_stats:
            for k, v in s.items():
                print("%s: %g" % (k, v))
            if self.h is not None:
                for k, v in self.timers().items():
                    print("%s: %.6f s" % (k, v))

    def close(self):
        if self.h is not None:
            self.lib.mptg_planner_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference spellings
    addStart = add_start
    solveFor = solve_for
    solveUntil = solve_until
    setRange = set_range
    getRange = get_range
    setGoalBias = set_goal_bias
    getGoalBias = get_goal_bias
    setRewireFactor = set_rewire_factor
    getRewireFactor = get_rewire_factor
    printStats = print_stats
    visitGraph = visit_graph


class PPRMPlanner(Planner):
    """Planner<Scenario, PPRM<...>>(scenario, seed) (src/mpt/impl/pprm/pprm.hpp:141-250):
    add_start / addStart, add_goal / addGoal, solve(done_fn), solve_for,
    solve_until, solved, size, solution() (Dijkstra's shortest roadmap path,
    pprm.hpp:230-240), print_stats and visit_graph (every node, then the far
    end of each of its edges, pprm.hpp:381-388)."""

    def __init__(self, scenario: Scenario, algorithm: PPRM | None = None, seed: int | None = None,
                 ctx: Context | None = None, max_nodes: int = 1 << 20):
        self.lib = load()
        _sig(self.lib)
        self.algorithm = algorithm or PPRM()
        self.ctx = ctx or Context(self.algorithm.device)
        self.scenario = scenario
        if seed is None:
            seed = int.from_bytes(np.random.default_rng().bytes(8), "little")
        self.seed = int(seed) & ((1 << 64) - 1)
        self.max_nodes = int(max_nodes)
        self.scene = Scene(self.ctx, scenario.desc)
        prm = _Params()
        prm.range = 0.0
        prm.goal_bias = 0.0
        prm.goal_radius = scenario.goal.radius
        prm.edge_step = scenario.edge_step
        prm.resolution = scenario.resolution
        prm.wavefront = self.algorithm.wavefront
        prm.seed = self.seed
        prm.max_nodes = self.max_nodes
        g = np.ascontiguousarray(scenario.goal.state, dtype=np.float64)
        h = ctypes.c_void_p()
        _check(self.ctx.h, self.lib.mptg_prm_create(self.ctx.h, self.scene.h, ctypes.byref(prm),
                                                    scenario.lo.ctypes.data, scenario.hi.ctypes.data, g.ctypes.data,
                                                    ctypes.byref(h)))
        self.h = h
        self.last_cost = math.inf

    def add_start(self, q) -> int:
        """addSample with the start flag: the node id, or -1 (invalid or duplicate)."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        i = ctypes.c_int32(-1)
        _check(self.ctx.h, self.lib.mptg_prm_add_start(self.h, q.ctypes.data, ctypes.byref(i)))
        return i.value

    def add_goal(self, q) -> int:
        q = np.ascontiguousarray(q, dtype=np.float64)
        i = ctypes.c_int32(-1)
        _check(self.ctx.h, self.lib.mptg_prm_add_goal(self.h, q.ctypes.data, ctypes.byref(i)))
        return i.value

    def run(self, max_wavefronts: int = 1, time_limit: float = 0.0, stop_when_solved: bool = False) -> bool:
        solved = ctypes.c_int(0)
        _check(self.ctx.h, self.lib.mptg_prm_run(self.h, int(max_wavefronts), float(time_limit),
                                                 int(stop_when_solved), ctypes.byref(solved)))
        return bool(solved.value)

    def solve(self, done_fn, deadline: float | None = None):
        """Runs wavefronts until done_fn() is true: polled between calls of up
        to POLL_SECONDS of wavefronts (at least one), each of which ends early
        at the first solution or at the deadline (time.monotonic())."""
        while not done_fn():
            before = self.stats()["wavefronts"]
            limit = self.POLL_SECONDS
            if deadline is not None:
                left = deadline - time.monotonic()
                if left <= 0:
                    break
                limit = min(limit, left)
            self.run(0, time_limit=limit, stop_when_solved=not self.solved())
            if self.stats()["wavefronts"] == before:  # node budget exhausted
                break

    def solved(self) -> bool:
        return bool(self.stats()["solved"])

    def size(self) -> int:
        n = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_prm_size(self.h, ctypes.byref(n), None))
        return n.value

    def edges(self) -> int:
        e = ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_prm_size(self.h, None, ctypes.byref(e)))
        return e.value

    def solution(self, fn=None):
        n = ctypes.c_size_t()
        cost = ctypes.c_double()
        _check(self.ctx.h, self.lib.mptg_prm_solution(self.h, None, 0, ctypes.byref(n), ctypes.byref(cost)))
        path = np.empty((n.value, self.scene.dim), dtype=np.float64)
        if n.value:
            _check(self.ctx.h, self.lib.mptg_prm_solution(self.h, path.ctypes.data, n.value, ctypes.byref(n),
                                                          ctypes.byref(cost)))
        self.last_cost = cost.value
        if fn is None:
            return [p for p in path]
        for p in path:
            fn(p)
        return None

    def graph(self):
        """(states [n][dim], (from, to, distance)) with from > to, sorted by (from, to)."""
        n, ne = ctypes.c_size_t(), ctypes.c_size_t()
        _check(self.ctx.h, self.lib.mptg_prm_size(self.h, ctypes.byref(n), ctypes.byref(ne)))
        states = np.empty((n.value, self.scene.dim), dtype=np.float64)
        ef = np.empty(ne.value, dtype=np.int32)
        et = np.empty(ne.value, dtype=np.int32)
        ed = np.empty(ne.value, dtype=np.float64)
        _check(self.ctx.h, self.lib.mptg_prm_graph(self.h, states.ctypes.data, n.value, ef.ctypes.data,
                                                   et.ctypes.data, ed.ctypes.data, ne.value, ctypes.byref(n),
                                                   ctypes.byref(ne)))
        return states, (ef, et, ed)

    def visit_graph(self, visitor):
        states, (ef, et, _) = self.graph()
        adj = [[] for _ in range(len(states))]
        for a, b in zip(ef.tolist(), et.tolist()):
            adj[a].append(b)
            adj[b].append(a)
        for i in range(len(states)):
            visitor.vertex(states[i])
            for j in adj[i]:
                visitor.edge(states[j])

    def stats(self) -> dict:
        out = (ctypes.c_uint64 * 8)()
        _check(self.ctx.h, self.lib.mptg_prm_stats(self.h, out))
        keys = ["wavefronts", "samples", "valid_samples", "duplicates", "links_checked", "edges", "goal_nodes",
                "solved"]
        return dict(zip(keys, [int(v) for v in out]))

    def print_stats(self):
        print("nodes in graph: %d" % self.size())
        if self.algorithm.report_stats:
            for k, v in self.stats().items():
                print("%s: %d" % (k, v))

    def close(self):
        if self.h is not None:
            self.lib.mptg_prm_destroy(self.h)
            self.h = None

    addStart = add_start
    addGoal = add_goal
    printStats = print_stats
    visitGraph = visit_graph


def autotune_cache_key(scenario: Scenario, candidates, max_nodes: int) -> str:
    """Key of an autotuner result: scene kind, metric, dimension, the tree
    capacity's power-of-two bucket and the candidate sizes."""
    d = scenario.desc
    bucket = max(0, int(max_nodes) - 1).bit_length()
    return "%s/m%d/d%d/n2^%d/%s" % (d["kind"], int(d["metric"]), int(d["dim"]), bucket,
                                     ",".join(str(int(c)) for c in candidates))


def _cache_load(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _cache_store(path: str, key: str, best: int, med: dict):
    data = _cache_load(path)
    data[key] = {"best": int(best), "median_s": {str(k): float(v) for k, v in med.items()}}
    tmp = "%s.tmp%d" % (path, os.getpid())
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune_wavefront(ctx: Context, scenario: Scenario, start, candidates=(32, 48, 64, 128, 256, 512, 1024, 2048, 4096, 8192),
                       trials: int = 3, time_limit: float = 2.0, seed: int = 1, max_nodes: int = 1 << 21,
                       goal_bias: float = 0.01, range_: float | None = None, cache: str | None = None):
    """Native wavefront-size autotuner (mptg_autotune_wavefront): `trials`
    seeds per size, then 2 * trials more for the three sizes with the lowest
    median time to the first solution; the lowest median of those three over
    all their seeds wins.  Returns (best size, {size: median seconds over the
    seeds it ran}).

    cache: a JSON file of earlier results keyed by autotune_cache_key (scene
    kind, metric, dimension, capacity bucket, candidates).  A hit returns the
    stored result without running the GPU; a miss runs the tuner and stores
    its result."""
    key = autotune_cache_key(scenario, candidates, max_nodes) if cache else None
    if cache:
        hit = _cache_load(cache).get(key)
        if hit:
            return int(hit["best"]), {int(k): float(v) for k, v in hit["median_s"].items()}
    lib = load()
    _sig(lib)
    scene = Scene(ctx, scenario.desc)
    prm = _Params()
    rng = scenario.default_range if range_ is None else float(range_)
    prm.range = rng if math.isfinite(rng) else 0.0
    prm.goal_bias = goal_bias
    prm.goal_radius = scenario.goal.radius
    prm.edge_step = scenario.edge_step
    prm.resolution = scenario.resolution
    prm.wavefront = max(candidates)
    prm.seed = int(seed) & ((1 << 64) - 1)
    prm.max_nodes = int(max_nodes)
    cand = (ctypes.c_int * len(candidates))(*candidates)
    med = (ctypes.c_double * len(candidates))()
    best = ctypes.c_int()
    q0 = np.ascontiguousarray(start, dtype=np.float64)
    g = np.ascontiguousarray(scenario.goal.state, dtype=np.float64)
    _check(ctx.h, lib.mptg_autotune_wavefront(ctx.h, scene.h, ctypes.byref(prm), scenario.lo.ctypes.data,
                                              scenario.hi.ctypes.data, q0.ctypes.data, g.ctypes.data,
                                              scenario.goal.radius, cand, len(candidates), int(trials),
                                              float(time_limit), ctypes.byref(best), med))
    scene.close()
    result = {c: med[i] for i, c in enumerate(candidates)}
    if cache:
        _cache_store(cache, key, best.value, result)
    return best.value, result


__all__ = ["Planner", "PRRTStar", "PPRM", "autotune_wavefront", "autotune_cache_key", "PRRT", "Scenario", "GoalState", "gpu_wavefront",
           "gpu_device", "report_stats", "max_threads", "single_threaded", "hardware_concurrency", "MptgError"]
