"""GPU: scenes loaded from files (mpt_gb300.ingest) run through the C ABI --
validity and DMV links equal the oracle's on the loaded geometry, and the
planners solve the loaded problems."""
import numpy as np
import pytest

from mpt_gb300 import ingest, scenes

pytestmark = pytest.mark.gpu


def _write_se3_problem(tmp_path):
    sc = scenes.mesh_scene()
    ingest.write_obj(str(tmp_path / "env.obj"), sc["env_tris"])
    ingest.write_obj(str(tmp_path / "robot.obj"), sc["robot_tris"])
    lines = ["[problem]", "world = env.obj", "robot = robot.obj"]
    for name, st in (("start", sc["start"]), ("goal", sc["goal"])):
        lines += ["%s.%s = %r" % (name, c, float(v)) for c, v in zip("xyz", st[4:])]
        lines += ["%s.theta = 0.3" % name, "%s.axis.x = 0" % name, "%s.axis.y = 1" % name, "%s.axis.z = 0" % name]
    lines += ["volume.min.x = 0", "volume.min.y = 0", "volume.min.z = 0",
              "volume.max.x = 20", "volume.max.y = 20", "volume.max.z = 20", "[planner]", "rrt.range = 40"]
    (tmp_path / "prob.cfg").write_text("\n".join(lines) + "\n")
    return ingest.se3_problem(str(tmp_path / "prob.cfg"))


def test_loaded_se3_problem_validity_matches_oracle(ctx, orc, tmp_path):
    import mpt_gb300 as m
    pr = _write_se3_problem(tmp_path)
    scene = m.Scene(ctx, pr)
    sp = orc.make_space(pr["metric"], pr["dim"], pr["weights"])
    q = np.concatenate([scenes.uniform_states(pr, 3000, 41), scenes.near_contact_states(scenes.mesh_scene(), 1000, 42)])
    q[:, 4:] = np.clip(q[:, 4:], 0.0, 20.0)
    got = scene.valid(q)
    want = orc.valid_states(pr, sp, q)
    assert np.array_equal(got, want) and 0 < got.mean() < 1
    a, b = q[:400], q[400:800]
    gl = scene.link(a, b, pr["edge_step"], 0)
    wl, _ = orc.valid_edges(pr, sp, a, b, pr["edge_step"], 0)
    assert np.array_equal(gl, wl)
    scene.close()


def test_loaded_png_grid_solves(ctx, orc, tmp_path):
    from mpt_gb300 import planner as P
    base = scenes.grid_scene()
    # the obstacles in the demo's brown, free space green (white is an obstacle colour of the demo), as P6
    rgb = np.where(base["grid"][:, :, None] == 1, np.array([126, 106, 61], np.uint8),
                   np.array([30, 160, 30], np.uint8)).astype(np.uint8)
    h, w = base["grid"].shape
    (tmp_path / "map.ppm").write_bytes(b"P6\n%d %d\n255\n" % (w, h) + rgb.tobytes())
    sc = ingest.png_grid_scene(str(tmp_path / "map.ppm"), base["start"], base["goal"])
    assert np.array_equal(sc["grid"], base["grid"])
    sc["goal_radius"] = 8.0
    pl = P.Planner(P.Scenario(sc), P.PPRM(P.gpu_wavefront(1024)), seed=3, ctx=ctx, max_nodes=1 << 18)
    pl.add_start(sc["start"])
    pl.add_goal(sc["goal"])
    pl.solve_for(20.0, lambda: pl.solved())
    assert pl.solved()
    path = np.array(pl.solution())
    sp = orc.make_space(sc["metric"], sc["dim"], sc["weights"])
    ok, _ = orc.valid_edges(sc, sp, path[:-1], path[1:], sc["edge_step"], sc["resolution"])
    assert ok.all()
    pl.close()


def test_export_real_runs(ctx, tmp_path):
    """The writers on real planners: the PPRM roadmap of the grid (each
    undirected edge visited from both ends) and a PRRT arm solution."""
    import xml.etree.ElementTree as ET
    import json
    from mpt_gb300 import export
    from mpt_gb300 import planner as P
    sc = scenes.grid_scene()
    pl = P.Planner(P.Scenario(sc), P.PPRM(P.gpu_wavefront(1024)), seed=9, ctx=ctx, max_nodes=1 << 18)
    pl.add_start(sc["start"])
    pl.add_goal(sc["goal"])
    pl.solve_for(20.0, lambda: pl.solved())
    n = export.svg_2d(str(tmp_path / "prm.svg"), pl, sc)
    assert n == 2 * pl.edges() and n > 0
    root = ET.parse(str(tmp_path / "prm.svg")).getroot()
    assert len(root.findall("{http://www.w3.org/2000/svg}line")) == n + len(pl.solution()) - 1
    pl.close()
    arm = scenes.arm_scene()
    pa = P.Planner(P.Scenario(arm), P.PRRT(P.gpu_wavefront(4096)), seed=1000, ctx=ctx, max_nodes=1 << 21)
    pa.add_start(arm["start"])
    pa.solve_for(20.0, lambda: pa.solved())
    assert pa.solved()
    k = export.arm_solution_js(str(tmp_path / "solution.js"), pa, arm)
    d = json.loads(open(str(tmp_path / "solution.js")).read()[len("data = "):])
    assert k == len(d["solution"]) >= 2 and d["solution"][0] == [float(v) for v in arm["start"]]
    pa.close()
