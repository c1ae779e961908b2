"""CPU: solution export (mpt_gb300.export) -- the 2-D SVG of
demo/png_2d_planning.cpp:110-166 and the arm demo's solution data file
(demo/link_manipulator_planning.cpp:90-166), from a planner-shaped object."""
import json
import xml.etree.ElementTree as ET

import numpy as np

from mpt_gb300 import export, ingest, scenes


class _Planner:
    """visit_graph / solution with a fixed graph (the planner interface the writers use)."""

    def __init__(self, states, edges, path):
        self.states, self.edges, self.path = states, edges, path

    def solution(self):
        return [self.states[i] for i in self.path]

    def visit_graph(self, visitor):
        for i, s in enumerate(self.states):
            visitor.vertex(s)
            for a, b in self.edges:
                if a == i:
                    visitor.edge(self.states[b])


def test_svg_2d(tmp_path):
    sc = scenes.grid_scene()
    st = np.array([[10.0, 10.0], [100.5, 40.0], [300.0, 500.25], [1014.0, 1014.0]])
    pl = _Planner(st, [(1, 0), (2, 1), (3, 2), (2, 0)], [0, 1, 2, 3])
    p = str(tmp_path / "run.svg")
    assert export.svg_2d(p, pl, sc) == 4
    root = ET.parse(p).getroot()
    ns = "{http://www.w3.org/2000/svg}"
    lines = root.findall(ns + "line")
    assert len(lines) == 4 + 3
    red = [l for l in lines if l.get("stroke") == "rgb(250, 50, 50)"]
    assert [(float(l.get("x1")), float(l.get("y1"))) for l in red] == [(10.0, 10.0), (100.5, 40.0), (300.0, 500.25)]
    assert [t.text.strip() for t in root.findall(ns + "text")] == ["S", "G"]
    bg = ingest.read_image(str(tmp_path / "run_grid.png"))
    assert np.array_equal(bg[:, :, 0] == 0, sc["grid"] == 1)
    # no solution: no file
    assert export.svg_2d(str(tmp_path / "none.svg"), _Planner(st, [], []), sc) == 0
    assert not (tmp_path / "none.svg").exists()


def test_arm_solution_js(tmp_path):
    sc = scenes.arm_scene()
    st = np.stack([sc["start"], sc["goal"]])
    p = str(tmp_path / "solution.js")
    assert export.arm_solution_js(p, _Planner(st, [(1, 0)], [0, 1]), sc) == 2
    text = open(p).read()
    assert text.startswith("data = \n{")
    d = json.loads(text[len("data = "):])
    assert d["dimension"] == 10 and len(d["armLengths"]) == 10
    assert d["lengthSum"] == sum(float(v) for v in sc["link_len"])  # accumulated in link order
    assert len(d["circles"]) == len(sc["discs"]) and d["circles"][0]["r"] == float(sc["discs"][0][2])
    assert np.array_equal(np.array(d["solution"]), st)
