"""Solution export as plain files (no graphics API): the SVG of a 2-D planning
run and the arm demo's solution data file.

* ``svg_2d``: demo/png_2d_planning.cpp:110-166 with the SVG primitives of
  demo/shape_hierarchy.hpp:85-166 -- a background image, every graph edge
  from ``visit_graph`` (grey, rgb(125, 125, 125)), the solution path (red,
  rgb(250, 50, 50)) and labelled start / goal circles; nothing is written
  when there is no solution.
* ``arm_solution_js``: demo/link_manipulator_planning.cpp:90-166 -- the
  ``data = {...}`` file the arm demo's HTML viewer reads (robot radius,
  dimension, link lengths and their sum, obstacle discs, solution states).
* ``write_png``: an RGB image as PNG (zlib, filter 0), used for the grid
  scene's background when no image file exists.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


def write_png(path: str, rgb: np.ndarray):
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def _num(v) -> str:
    return repr(float(v)) if not float(v).is_integer() else str(int(v))


def _attr(name, value, unit=""):
    return ' %s="%s%s"' % (name, value, unit)


def _line(x1, y1, x2, y2, width, rgb) -> str:
    return ("\t<line" + _attr("x1", _num(x1)) + _attr("y1", _num(y1)) + _attr("x2", _num(x2)) +
            _attr("y2", _num(y2)) + _attr("stroke", "rgb(%d, %d, %d)" % rgb) + _attr("stroke-width", _num(width)) +
            _attr("stroke-linecap", "round") + "/>\n")


def _state(x, y, r, label) -> str:
    return ("\t<circle" + _attr("cx", _num(x)) + _attr("cy", _num(y)) + _attr("r", _num(r)) +
            _attr("fill", "rgb(230, 230, 230)") + _attr("stroke", "red") + _attr("stroke-width", _num(r / 5)) +
            "/>\n\t<text" + _attr("x", _num(x)) + _attr("y", _num(y + r / 3.0)) + _attr("fill", "black") +
            _attr("text-anchor", "middle") + _attr("font-size", _num(r)) + "> %s </text>\n" % label)


def svg_2d(path: str, planner, scene: dict, start=None, goal=None, background: str | None = None,
           edge_width: float = 0.3, path_width: float = 10.0, state_radius: float = 40.0) -> int:
    """Writes the run as SVG and returns the number of graph edges drawn
    (0 and no file when the planner has no solution).  For a grid scene
    without a background image, the grid is written beside the SVG as
    ``<name>_grid.png`` (obstacles black, free space white) and referenced."""
    sol = planner.solution()
    if len(sol) == 0:
        return 0
    if scene.get("dim") != 2:
        raise ValueError("svg_2d draws 2-D states only")
    w, h = scene["hi"][0] - scene["lo"][0], scene["hi"][1] - scene["lo"][1]
    if background is None and scene.get("kind") == "grid":
        background = os.path.splitext(path)[0] + "_grid.png"
        g = np.asarray(scene["grid"])
        write_png(background, np.repeat(np.where(g[:, :, None] != 0, 0, 255).astype(np.uint8), 3, axis=2))
    out = ['<?xml version="1.0" standalone="no" ?>\n',
           '<!DOCTYPE svg PUBLIC "-//W3C//DTD SVG 1.1//EN" "http://www.w3.org/Graphics/SVG/1.1/DTD/svg11.dtd">\n',
           "<svg" + _attr("width", _num(w), "px") + _attr("height", _num(h), "px") +
           _attr("xmlns", "http://www.w3.org/2000/svg") + _attr("xmlns:xlink", "http://www.w3.org/1999/xlink") +
           _attr("version", "1.1") + ">\n"]
    if background:
        out.append("\t<image" + _attr("xlink:href", os.path.basename(background)) + _attr("width", _num(w)) +
                   _attr("height", _num(h)) + "/>\n")

    class Visitor:
        def __init__(self):
            self.frm = None
            self.n = 0

        def vertex(self, q):
            self.frm = q

        def edge(self, to):
            out.append(_line(self.frm[0], self.frm[1], to[0], to[1], edge_width, (125, 125, 125)))
            self.n += 1

    vis = Visitor()
    planner.visit_graph(vis)
    for a, b in zip(sol[:-1], sol[1:]):
        out.append(_line(a[0], a[1], b[0], b[1], path_width, (250, 50, 50)))
    s = scene["start"] if start is None else start
    g = scene["goal"] if goal is None else goal
    out.append(_state(s[0], s[1], state_radius, "S"))
    out.append(_state(g[0], g[1], state_radius, "G"))
    out.append("</svg>\n")
    with open(path, "w") as f:
        f.writelines(out)
    return vis.n


def arm_solution_js(path: str, planner, scene: dict) -> int:
    """Writes the arm demo's ``data = {...}`` file; returns the number of
    solution states (0 and no file when there is no solution)."""
    sol = planner.solution()
    if len(sol) == 0:
        return 0
    L = [float(v) for v in scene["link_len"]]
    lines = ["data = ", "{",
             '\t"radius": %r,' % float(scene.get("robot_radius", 0.0)), "",
             '\t"dimension": %d,' % len(L), "",
             '\t"armLengths": [%s],' % ", ".join(repr(v) for v in L), "",
             '\t"lengthSum": %r,' % float(sum(L)), "",
             '\t"circles": [']
    discs = np.asarray(scene["discs"], dtype=np.float64).reshape(-1, 3)
    for i, (cx, cy, r) in enumerate(discs):
        lines += ["\t\t{", '\t\t\t"cx": %r,' % float(cx), '\t\t\t"cy": %r,' % float(cy), '\t\t\t"r": %r' % float(r),
                  "", "\t\t}" + ("," if i + 1 < len(discs) else "")]
    lines += ["\t],", "", '\t"solution": [']
    for i, s in enumerate(sol):
        lines.append("\t\t[%s]" % ", ".join(repr(float(v)) for v in s) + ("," if i + 1 < len(sol) else ""))
    lines += ["\t]", "}"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return len(sol)
