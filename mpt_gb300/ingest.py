"""Scene ingestion without assimp or libpng: Wavefront OBJ meshes, PNG and
Netpbm occupancy images, and the OMPL.app-style problem files of the
reference's demos, turned into the scene dictionaries of mpt_gb300.scenes.

* ``read_cfg`` / ``cfg_*``: demo/scenario_config.hpp:73-160 -- ``[section]``
  headers, ``key = value`` properties (surrounding whitespace trimmed), blank
  lines skipped, other lines and properties before any section skipped with a
  warning; numbers must parse completely; a 3-vector is ``name.x/.y/.z``, a
  rotation ``name.theta`` + ``name.axis.x/.y/.z`` (Eigen AngleAxis ->
  Quaternion), an SE(3) state the rotation then the vector under one name.
* ``load_obj``: the triangles that demo/se3_rigid_body_scenario.hpp:155-208
  hands to FCL -- polygons fanned around their first vertex (faces with fewer
  than three indices skipped, the visitTriangles rule of :97-134), optionally
  shifted so the mean of the mesh's vertices is the origin (the robot; the
  environment is not shifted).
* ``read_image`` + ``obstacle_grid``: demo/png_2d_scenario.hpp:198-282 --
  palette expanded to RGB, 16-bit samples reduced to 8, sub-byte depths
  unpacked, alpha dropped; a pixel is an obstacle when some FilterColor
  (r, g, b, tol) holds every channel within tol (:50-69).  PNG is decoded
  with zlib (plain and Adam7-interlaced images); Netpbm P1-P6 is read directly.
* ``se3_problem`` / ``png_grid_scene``: the scenarios of
  demo/se3_rigid_body_planning.cpp:237-281 and demo/png_2d_planning.cpp:60-90
  as scene dictionaries (see each docstring for the parameters they fix).
"""
from __future__ import annotations

import ctypes
import math
import os
import re
import struct
import warnings
import zlib

import numpy as np

from . import load
from .scenes import L2, SE3

# ------------------------------------------------------------------ config files
_SECTION = re.compile(r"\s*\[\s*([^\]]+?)\s*\]\s*")
_KEYVAL = re.compile(r"\s*([^=]*?)\s*=\s*(.*?)\s*")
_NUMBER = re.compile(r"\s*[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)", re.IGNORECASE)


def read_cfg(path: str) -> dict:
    """{section: {key: value}} of an INI-style problem file."""
    props: dict = {}
    section = ""
    with open(path, "r") as f:
        for no, line in enumerate(f, 1):
            line = line.rstrip("\n")
            if not line.strip():
                continue
            m = _SECTION.fullmatch(line)
            if m:
                section = m.group(1)
                if section in props:
                    warnings.warn("%s:%d: duplicate section" % (path, no))
                props.setdefault(section, {})
                continue
            m = _KEYVAL.fullmatch(line)
            if m:
                if not section:
                    warnings.warn("%s:%d: property without section header" % (path, no))
                else:
                    props[section][m.group(1)] = m.group(2)
                continue
            warnings.warn("%s:%d: invalid line" % (path, no))
    return props


def cfg_has(cfg: dict, section: str, name: str) -> bool:
    return section in cfg and name in cfg[section]


def cfg_get(cfg: dict, section: str, name: str) -> str:
    if section not in cfg:
        raise ValueError("missing section [%s]" % section)
    if name not in cfg[section]:
        raise ValueError("missing property [%s] %s" % (section, name))
    return cfg[section][name]


def cfg_float(cfg: dict, section: str, name: str) -> float:
    s = cfg_get(cfg, section, name)
    m = _NUMBER.match(s)
    if not m or m.end() != len(s):  # std::stod must consume the whole value
        raise ValueError("invalid numeric value: " + s)
    return float(s)


def cfg_vec3(cfg: dict, section: str, name: str) -> np.ndarray:
    return np.array([cfg_float(cfg, section, name + "." + c) for c in "xyz"])


def cfg_quat(cfg: dict, section: str, name: str) -> np.ndarray:
    """(qx, qy, qz, qw) of the rotation name.theta about name.axis
    (w = cos(theta/2), xyz = sin(theta/2) axis).  Eigen's AngleAxis takes a
    unit axis; a non-unit one is normalised first, so the result is the
    rotation by theta about the axis direction (the planner's spaces need
    unit quaternions)."""
    theta = cfg_float(cfg, section, name + ".theta")
    axis = cfg_vec3(cfg, section, name + ".axis")
    n = math.sqrt(float(np.dot(axis, axis)))
    if not n > 0:
        raise ValueError("rotation %s has a zero axis" % name)
    axis = axis / n
    h = 0.5 * theta
    return np.array([axis[0] * math.sin(h), axis[1] * math.sin(h), axis[2] * math.sin(h), math.cos(h)])


def cfg_se3(cfg: dict, section: str, name: str) -> np.ndarray:
    """SE(3) state (qx, qy, qz, qw, x, y, z): the rotation, then the vector."""
    return np.concatenate([cfg_quat(cfg, section, name), cfg_vec3(cfg, section, name)])


# ------------------------------------------------------------------ meshes
def load_obj(path: str, shift_to_center: bool = False):
    """(triangles [n][9], center [3], vertex count) of a Wavefront OBJ file.

    ``f`` entries may be ``i``, ``i/t``, ``i//n`` or ``i/t/n`` with 1-based or
    negative (relative) indices; every object and group of the file is one
    mesh.  The center is the mean of the distinct vertex positions the faces
    use (assimp's JoinIdenticalVertices keeps each position once)."""
    with open(path, "r") as f:
        lines = f.read().splitlines()
    vlines = [ln[2:] for ln in lines if ln.startswith("v ")]
    flines = [ln[2:] for ln in lines if ln.startswith("f ")]
    if not flines:
        raise ValueError("mesh file '%s' does not contain meshes" % path)
    # fast paths for the common layout (three coordinates per vertex, triangles
    # of positive plain indices); anything else goes line by line
    if all(len(ln.split()) == 3 for ln in vlines):
        V = np.array(" ".join(vlines).split(), dtype=np.float64).reshape(-1, 3)
    else:
        V = np.array([[float(x) for x in ln.split()[:3]] for ln in vlines], dtype=np.float64).reshape(-1, 3)
    T = None
    if all(len(ln.split()) == 3 for ln in flines):
        ft = " ".join(flines).split()
        if all(c.isdigit() for c in ft):
            T = np.array(ft, dtype=np.int64).reshape(-1, 3) - 1
    if T is None:
        tri = []
        nv = 0
        for ln in lines:  # relative indices count the vertices read so far
            if ln.startswith("v "):
                nv += 1
            elif ln.startswith("f "):
                idx = []
                for tok in ln.split()[1:]:
                    i = int(tok.split("/")[0])
                    idx.append(i - 1 if i > 0 else nv + i)
                for k in range(1, len(idx) - 1):  # fan around the first vertex; < 3 indices: skipped
                    tri.append((idx[0], idx[k], idx[k + 1]))
        T = np.asarray(tri, dtype=np.int64).reshape(-1, 3)
    if T.size and (T.min() < 0 or T.max() >= len(V)):
        raise ValueError("mesh file '%s' has a face index out of range" % path)
    used = np.unique(V[np.unique(T)], axis=0) if T.size else V[:0]
    center = used.mean(axis=0) if len(used) else np.zeros(3)
    P = V - center if shift_to_center else V
    return P[T].reshape(-1, 9), center, len(used)


def write_obj(path: str, tris: np.ndarray):
    """Triangles [n][9] as an OBJ file (three vertices per face, full precision)."""
    t = np.asarray(tris, dtype=np.float64).reshape(-1, 3, 3)
    with open(path, "w") as f:
        for tr in t:
            for v in tr:
                f.write("v %r %r %r\n" % (float(v[0]), float(v[1]), float(v[2])))
        for i in range(len(t)):
            f.write("f %d %d %d\n" % (3 * i + 1, 3 * i + 2, 3 * i + 3))


# ------------------------------------------------------------------ images
def _png_samples(raw: np.ndarray, w: int, h: int, depth: int, ctype: int):
    """8-bit samples [h][w * channels] of one (sub-)image of filtered scanlines
    at the start of raw, and the number of bytes it took."""
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = depth * chans
    stride = (w * bits + 7) // 8
    bpp = max(1, bits // 8)
    need = h * (stride + 1)
    if len(raw) < need:
        raise ValueError("truncated PNG image data")
    out = np.empty((h, stride), dtype=np.uint8)
    lib = load()
    lib.mptg_png_unfilter.restype = ctypes.c_int
    lib.mptg_png_unfilter.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    rows = np.ascontiguousarray(raw[:need])
    if lib.mptg_png_unfilter(rows.ctypes.data, h, stride, bpp, out.ctypes.data) != 0:
        raise ValueError("PNG row with an unknown filter type")
    if depth == 16:
        px = out.reshape(h, w * chans, 2)[:, :, 0]  # strip to the high byte
    elif depth < 8:
        px = np.unpackbits(out, axis=1).reshape(h, -1, depth)[:, :w * chans]
        px = (px * (1 << np.arange(depth - 1, -1, -1))).sum(axis=2).astype(np.uint8)
        if ctype == 0:
            px = (px * (255 // ((1 << depth) - 1))).astype(np.uint8)
    else:
        px = out[:, :w * chans]
    return px, need


def _png_rgb(data: bytes) -> np.ndarray:
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, plte, hdr = 8, [], None, None
    while pos < len(data):
        if pos + 12 > len(data):
            raise ValueError("truncated PNG chunk")
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if len(body) < n:
            raise ValueError("truncated PNG chunk")
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    # the colour type / bit depth pairs of the PNG specification
    if depth not in {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}.get(ctype, ()):
        raise ValueError("unsupported PNG colour type %d with bit depth %d" % (ctype, depth))
    if w < 1 or h < 1:
        raise ValueError("PNG with an empty image")
    if ctype == 3 and plte is None:
        raise ValueError("palette PNG without PLTE")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    try:
        raw = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    except zlib.error as e:
        raise ValueError("corrupt PNG image data: %s" % e) from None
    if not interlace:
        px, _ = _png_samples(raw, w, h, depth, ctype)
    else:
        # Adam7: seven passes of sub-images, each filtered on its own
        px = np.zeros((h, w, chans), dtype=np.uint8)
        off = 0
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            pw, ph = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
            if pw <= 0 or ph <= 0:
                continue
            sub, used = _png_samples(raw[off:], pw, ph, depth, ctype)
            px[y0::dy, x0::dx] = sub.reshape(ph, pw, chans)
            off += used
    px = px.reshape(h, w, chans)
    if ctype == 3:
        if px.size and int(px.max()) >= len(plte):
            raise ValueError("PNG palette index beyond its PLTE")
        return plte[px[:, :, 0]]
    if ctype in (0, 4):
        return np.repeat(px[:, :, :1], 3, axis=2)
    return px[:, :, :3].copy()


def _pnm_rgb(data: bytes) -> np.ndarray:
    magic = data[:2]
    toks, pos, end = [], 2, len(data)
    need = 2 if magic in (b"P1", b"P4") else 3
    while len(toks) < need:
        while pos < end and data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            while data[pos:pos + 1] not in (b"\n", b""):
                pos += 1
            continue
        start = pos
        while pos < end and not data[pos:pos + 1].isspace():
            pos += 1
        if start == pos:
            raise ValueError("truncated Netpbm header")
        if not data[start:pos].isdigit():
            raise ValueError("invalid Netpbm header value %r" % data[start:pos])
        toks.append(int(data[start:pos]))
    w, h = toks[0], toks[1]
    maxv = toks[2] if need == 3 else 1
    if w < 1 or h < 1 or not 1 <= maxv <= 65535:
        raise ValueError("invalid Netpbm size or maximum value")
    if magic in (b"P1", b"P2", b"P3"):
        body = re.sub(rb"#[^\n]*", b"", data[pos:])
        if magic == b"P1":
            vals = np.array([c - 48 for c in body if c in b"01"], dtype=np.int64)[:w * h]
            if len(vals) < w * h:
                raise ValueError("truncated Netpbm image data")
            g = np.where(vals.reshape(h, w) == 1, 0, 255).astype(np.uint8)
            return np.repeat(g[:, :, None], 3, axis=2)
        ch = 1 if magic == b"P2" else 3
        try:
            vals = np.array(body.split(), dtype=np.int64)
        except ValueError:
            raise ValueError("invalid Netpbm sample value") from None
        if len(vals) < w * h * ch:
            raise ValueError("truncated Netpbm image data")
        px = (vals[:w * h * ch] * 255 // maxv).astype(np.uint8).reshape(h, w, ch)
        return np.repeat(px, 3, axis=2) if ch == 1 else px
    pos += 1  # the single whitespace after the header
    if magic == b"P4":
        stride = (w + 7) // 8
        if end - pos < stride * h:
            raise ValueError("truncated Netpbm image data")
        bitsarr = np.unpackbits(np.frombuffer(data[pos:pos + stride * h], dtype=np.uint8).reshape(h, stride), axis=1)
        g = np.where(bitsarr[:, :w] == 1, 0, 255).astype(np.uint8)
        return np.repeat(g[:, :, None], 3, axis=2)
    ch = 1 if magic == b"P5" else 3
    dt = np.dtype(">u2") if maxv > 255 else np.dtype(np.uint8)
    if end - pos < w * h * ch * dt.itemsize:
        raise ValueError("truncated Netpbm image data")
    px = np.frombuffer(data[pos:pos + w * h * ch * dt.itemsize], dtype=dt).reshape(h, w, ch).astype(np.int64)
    px = (px * 255 // maxv).astype(np.uint8)
    return np.repeat(px, 3, axis=2) if ch == 1 else px


def read_image(path: str) -> np.ndarray:
    """RGB pixels [height][width][3] (uint8) of a PNG or Netpbm (P1-P6) file.
    A malformed, truncated or unsupported file raises ValueError."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] == b"\x89PNG\r\n\x1a\n":
        return _png_rgb(data)
    if data[:1] == b"P" and data[1:2] in b"123456":
        return _pnm_rgb(data)
    raise ValueError("unsupported image format: '%s'" % path)


# FilterColor table of demo/png_2d_planning.cpp:69-72 (r, g, b, tolerance)
PNG_DEMO_FILTERS = ((126, 106, 61, 15), (61, 53, 6, 15), (255, 255, 255, 5))


def obstacle_grid(rgb: np.ndarray, filters) -> np.ndarray:
    """uint8 [height][width]: 1 where some filter (r, g, b, tol) holds every
    channel within tol (inclusive), else 0."""
    px = rgb.astype(np.int64)
    obst = np.zeros(rgb.shape[:2], dtype=bool)
    for r, g, b, tol in filters:
        c = np.array([r, g, b])
        obst |= np.all((px >= c - tol) & (px <= c + tol), axis=2)
    return obst.astype(np.uint8)


# ------------------------------------------------------------------ scenarios
def png_grid_scene(path: str, start, goal, filters=PNG_DEMO_FILTERS, edge_step: float = 1.0,
                   goal_radius: float = 1e-6) -> dict:
    """A grid scene from an image (PNG2dScenario, demo/png_2d_scenario.hpp:71-166):
    L2 space bounded by [0, width] x [0, height], GoalState radius 1e-6,
    cells (int)(x + 0.5).  Links go through the DMV at edge_step, as for the
    synthetic grid scene."""
    rgb = read_image(path)
    grid = obstacle_grid(rgb, filters)
    h, w = grid.shape
    return {"kind": "grid", "grid": grid, "metric": L2, "dim": 2, "weights": (1.0, 1.0),
            "lo": np.array([0.0, 0.0]), "hi": np.array([float(w), float(h)]),
            "start": np.asarray(start, dtype=np.float64), "goal": np.asarray(goal, dtype=np.float64),
            "goal_radius": goal_radius, "range": math.inf, "edge_step": edge_step, "resolution": 0}


SO3_WEIGHT = 50.0  # SE3Space<Scalar, 50> of demo/se3_rigid_body_scenario.hpp:54,250


def se3_problem(cfg_path: str, check_resolution: float = 0.01) -> dict:
    """A rigid-body scene from an OMPL.app-style problem file
    (demo/se3_rigid_body_planning.cpp:237-281): [problem] world / robot (OBJ
    paths relative to the file), start / goal (SE(3) states), volume.min /
    volume.max; [planner] rrt.range when present.  The robot mesh is shifted
    to its center, the environment is not; SO(3) weight 50; the DMV step is
    (|volume.max - volume.min| + 50 pi/2) * check_resolution
    (se3_rigid_body_scenario.hpp:333); GoalState radius 1e-6 (:279)."""
    cfg = read_cfg(cfg_path)
    base = os.path.dirname(os.path.abspath(cfg_path))
    env, _, _ = load_obj(os.path.join(base, cfg_get(cfg, "problem", "world")), shift_to_center=False)
    robot, _, _ = load_obj(os.path.join(base, cfg_get(cfg, "problem", "robot")), shift_to_center=True)
    vmin = cfg_vec3(cfg, "problem", "volume.min")
    vmax = cfg_vec3(cfg, "problem", "volume.max")
    rng = cfg_float(cfg, "planner", "rrt.range") if cfg_has(cfg, "planner", "rrt.range") else math.inf
    step = (float(np.linalg.norm(vmax - vmin)) + SO3_WEIGHT * math.pi / 2) * check_resolution
    rv = robot.reshape(-1, 3)
    return {"kind": "mesh", "robot_tris": robot, "env_tris": env,
            "robot_bound": float(np.sqrt((rv * rv).sum(axis=1)).max()),
            "metric": SE3, "dim": 7, "weights": (SO3_WEIGHT, 1.0),
            "lo": np.concatenate([-np.ones(4), vmin]), "hi": np.concatenate([np.ones(4), vmax]),
            "start": cfg_se3(cfg, "problem", "start"), "goal": cfg_se3(cfg, "problem", "goal"),
            "goal_radius": 1e-6, "range": rng, "edge_step": step, "resolution": 0, "boxes": []}
