"""CPU: scene ingestion (mpt_gb300.ingest) -- OBJ meshes, PNG / Netpbm
occupancy images and OMPL.app-style problem files, against the reference
demos' loading rules (demo/se3_rigid_body_scenario.hpp:97-208,
demo/scenario_config.hpp:73-160, demo/png_2d_scenario.hpp:50-69,198-282)."""
import math
import os
import struct
import zlib

import numpy as np
import pytest

from mpt_gb300 import ingest, scenes


# ------------------------------------------------------------------ PNG writer (test side)
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filtered(rows: np.ndarray, bpp: int) -> bytes:
    """PNG scanlines of rows [h][stride], filter type y % 5 on row y."""
    h, stride = rows.shape
    raw = bytearray()
    prev = np.zeros(stride, dtype=np.int64)
    for y in range(h):
        ft = y % 5
        cur = rows[y].astype(np.int64)
        out = np.zeros(stride, dtype=np.int64)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            p = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            out[x] = (cur[x] - p) & 0xFF
        raw.append(ft)
        raw += bytes(out.astype(np.uint8))
        prev = cur
    return bytes(raw)


def _write_png(path, w, h, ctype, depth, raw: bytes, palette=None, interlace=0):
    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    if palette is not None:
        data += chunk(b"PLTE", bytes(np.asarray(palette, dtype=np.uint8).ravel()))
    data += chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)


def _png(path, rows: np.ndarray, ctype: int, depth: int, palette=None, width=None):
    """rows: [h][stride] packed sample bytes; filter type y % 5 on row y."""
    h, stride = rows.shape
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = max(1, chans * depth // 8)
    w = width if width is not None else stride * 8 // (depth * chans)
    _write_png(path, w, h, ctype, depth, _filtered(rows, bpp), palette)


ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _png_adam7(path, px: np.ndarray, ctype: int, depth: int, palette=None):
    """px: [h][w][channels] samples of the given bit depth; Adam7 order, each
    pass's scanlines packed and filtered on their own (empty passes omitted)."""
    h, w, chans = px.shape
    bpp = max(1, chans * depth // 8)
    raw = b""
    for x0, y0, dx, dy in ADAM7:
        sub = px[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        vals = sub.reshape(sub.shape[0], -1).astype(np.int64)
        if depth < 8:  # MSB-first bit packing, rows padded to whole bytes
            bits = (vals[:, :, None] >> np.arange(depth - 1, -1, -1)) & 1
            rows = np.packbits(bits.reshape(vals.shape[0], -1).astype(np.uint8), axis=1)
        elif depth == 16:
            rows = vals.astype(">u2").view(np.uint8).reshape(vals.shape[0], -1)
        else:
            rows = vals.astype(np.uint8)
        raw += _filtered(rows, bpp)
    _write_png(path, w, h, ctype, depth, raw, palette=palette, interlace=1)


def test_png_color_types_and_filters(tmp_path):
    rng = np.random.default_rng(1)
    rgb = rng.integers(0, 256, (11, 13, 3), dtype=np.uint8)
    p = str(tmp_path / "rgb.png")
    _png(p, rgb.reshape(11, -1), 2, 8)
    assert np.array_equal(ingest.read_image(p), rgb)
    # RGBA: alpha dropped
    rgba = np.concatenate([rgb, rng.integers(0, 256, (11, 13, 1), dtype=np.uint8)], axis=2)
    _png(p, rgba.reshape(11, -1), 6, 8)
    assert np.array_equal(ingest.read_image(p), rgb)
    # 16-bit RGB: the high byte
    rgb16 = rng.integers(0, 65536, (7, 5, 3)).astype(">u2")
    _png(p, rgb16.view(np.uint8).reshape(7, -1), 2, 16)
    assert np.array_equal(ingest.read_image(p), (rgb16 >> 8).astype(np.uint8))
    # grey and palette
    g = rng.integers(0, 256, (9, 6), dtype=np.uint8)
    _png(p, g, 0, 8)
    assert np.array_equal(ingest.read_image(p), np.repeat(g[:, :, None], 3, axis=2))
    pal = rng.integers(0, 256, (16, 3), dtype=np.uint8)
    idx = rng.integers(0, 16, (9, 6), dtype=np.uint8)
    _png(p, idx, 3, 8, palette=pal)
    assert np.array_equal(ingest.read_image(p), pal[idx])
    # 1-bit grey, width not a multiple of 8
    bits = rng.integers(0, 2, (5, 11), dtype=np.uint8)
    _png(p, np.packbits(bits, axis=1), 0, 1, width=11)
    assert np.array_equal(ingest.read_image(p)[:, :, 0], bits * 255)


@pytest.mark.parametrize("h,w", [(1, 1), (3, 2), (5, 9), (17, 13), (8, 8)])
def test_png_adam7_interlaced(tmp_path, h, w):
    rng = np.random.default_rng(h * 100 + w)
    p = str(tmp_path / "i.png")
    rgb = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    _png_adam7(p, rgb, 2, 8)
    assert np.array_equal(ingest.read_image(p), rgb)
    for depth in (1, 2, 4):  # sub-byte grey, scaled to 8 bits
        g = rng.integers(0, 1 << depth, (h, w, 1), dtype=np.uint8)
        _png_adam7(p, g, 0, depth)
        assert np.array_equal(ingest.read_image(p)[:, :, 0], g[:, :, 0] * (255 // ((1 << depth) - 1)))
    pal = rng.integers(0, 256, (16, 3), dtype=np.uint8)  # 4-bit palette
    idx = rng.integers(0, 16, (h, w, 1), dtype=np.uint8)
    _png_adam7(p, idx, 3, 4, palette=pal)
    assert np.array_equal(ingest.read_image(p), pal[idx[:, :, 0]])
    rgba16 = rng.integers(0, 65536, (h, w, 4))  # 16-bit RGBA: high bytes, alpha dropped
    _png_adam7(p, rgba16, 6, 16)
    assert np.array_equal(ingest.read_image(p), (rgba16[:, :, :3] >> 8).astype(np.uint8))


def test_pnm_formats(tmp_path):
    rgb = np.array([[[255, 0, 0], [0, 255, 0]], [[0, 0, 255], [10, 20, 30]]], dtype=np.uint8)
    p6 = tmp_path / "a.ppm"
    p6.write_bytes(b"P6\n# comment\n2 2\n255\n" + rgb.tobytes())
    assert np.array_equal(ingest.read_image(str(p6)), rgb)
    p3 = tmp_path / "b.ppm"
    p3.write_text("P3 2 2 255\n" + " ".join(str(v) for v in rgb.ravel()) + "\n")
    assert np.array_equal(ingest.read_image(str(p3)), rgb)
    p5 = tmp_path / "c.pgm"
    p5.write_bytes(b"P5 2 2 255\n" + bytes([0, 64, 128, 255]))
    assert np.array_equal(ingest.read_image(str(p5))[:, :, 1], [[0, 64], [128, 255]])
    p1 = tmp_path / "d.pbm"
    p1.write_text("P1\n3 2\n1 0 1\n0 1 0\n")
    assert np.array_equal(ingest.read_image(str(p1))[:, :, 0], [[0, 255, 0], [255, 0, 255]])
    p4 = tmp_path / "e.pbm"
    p4.write_bytes(b"P4\n3 2\n" + bytes([0b10100000, 0b01000000]))
    assert np.array_equal(ingest.read_image(str(p4))[:, :, 0], [[0, 255, 0], [255, 0, 255]])
    with pytest.raises(ValueError):
        bad = tmp_path / "f.bin"
        bad.write_bytes(b"GIF89a")
        ingest.read_image(str(bad))


def test_obstacle_filter_tolerance():
    # FilterColor::isObstacle: every channel within [c - tol, c + tol]
    rgb = np.array([[[126, 106, 61], [141, 121, 76], [142, 106, 61], [111, 91, 46], [110, 106, 61],
                     [250, 250, 250], [249, 255, 255], [0, 0, 0]]], dtype=np.uint8)
    g = ingest.obstacle_grid(rgb, ingest.PNG_DEMO_FILTERS)
    assert g.tolist() == [[1, 1, 0, 1, 0, 1, 0, 0]]


def test_reference_demo_png_decodes():
    from oracle.ref import stage
    src = os.environ.get("MPT_REFERENCE_SRC") or stage.DEFAULT_SOURCE
    path = os.path.join(os.path.dirname(src), "demo", "png_planning_input.png")
    if not os.path.exists(path):
        pytest.skip("reference demo image not present")
    sc = ingest.png_grid_scene(path, (430.0, 1300.0), (3150.0, 950.0))
    h, w = sc["grid"].shape
    assert w > 3150 and h > 1300
    assert 0.01 < sc["grid"].mean() < 0.9
    # the demo's start and goal cells are free (png_2d_planning.cpp:85-87)
    assert sc["grid"][1300, 430] == 0 and sc["grid"][950, 3150] == 0


# ------------------------------------------------------------------ OBJ
def test_obj_fan_triangulation_and_indices(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("""# cube-ish
o part
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 0.5 1
vt 0 0
vn 0 0 1
g side
f 1/1/1 2/1/1 3/1/1 4/1/1
f -5//1 -4//1 -1//1
f 2 3
f 1 2 3 4 5
""")
    tris, center, nv = ingest.load_obj(str(p))
    V = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0.5, 0.5, 1]], float)
    want = [(0, 1, 2), (0, 2, 3), (0, 1, 4), (0, 1, 2), (0, 2, 3), (0, 3, 4)]
    assert np.array_equal(tris, V[np.array(want)].reshape(-1, 9))
    assert nv == 5 and np.allclose(center, V.mean(axis=0))
    shifted, c2, _ = ingest.load_obj(str(p), shift_to_center=True)
    assert np.allclose(shifted.reshape(-1, 3) + c2, tris.reshape(-1, 3))
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError):
        ingest.load_obj(str(bad))


def test_obj_round_trip_bit_exact(tmp_path):
    sc = scenes.mesh_scene()
    p = str(tmp_path / "robot.obj")
    ingest.write_obj(p, sc["robot_tris"])
    tris, _, _ = ingest.load_obj(p)
    assert np.array_equal(tris.view(np.int64), sc["robot_tris"].view(np.int64))


# ------------------------------------------------------------------ cfg
def test_cfg_parsing_rules(tmp_path):
    p = tmp_path / "p.cfg"
    p.write_text("stray = 1\n[problem]\n  start.x =  1.5  \nstart.y=-2e-1\nstart.z = 3\n"
                 "start.theta = 1.0\nstart.axis.x = 0\nstart.axis.y = 0\nstart.axis.z = 2\n"
                 "name = a b c\nnot a property line\n\n[problem]\nbad = 1.0x\n")
    with pytest.warns(UserWarning):
        cfg = ingest.read_cfg(str(p))
    assert ingest.cfg_get(cfg, "problem", "name") == "a b c"
    assert list(ingest.cfg_vec3(cfg, "problem", "start")) == [1.5, -0.2, 3.0]
    q = ingest.cfg_quat(cfg, "problem", "start")
    assert np.allclose(q, [0, 0, math.sin(0.5), math.cos(0.5)])
    s = ingest.cfg_se3(cfg, "problem", "start")
    assert np.allclose(s, [0, 0, math.sin(0.5), math.cos(0.5), 1.5, -0.2, 3.0])
    with pytest.raises(ValueError, match="invalid numeric value"):
        ingest.cfg_float(cfg, "problem", "bad")
    with pytest.raises(ValueError, match="missing property"):
        ingest.cfg_get(cfg, "problem", "goal.x")
    with pytest.raises(ValueError, match="missing section"):
        ingest.cfg_get(cfg, "planner", "rrt.range")
    assert "stray" not in str(cfg)


def test_se3_problem_from_files(tmp_path):
    sc = scenes.mesh_scene()
    ingest.write_obj(str(tmp_path / "env.obj"), sc["env_tris"])
    ingest.write_obj(str(tmp_path / "robot.obj"), sc["robot_tris"])
    s, g = sc["start"][4:], sc["goal"][4:]
    lines = ["[problem]", "world = env.obj", "robot = robot.obj"]
    for name, p in (("start", s), ("goal", g)):
        lines += ["%s.%s = %r" % (name, c, float(v)) for c, v in zip("xyz", p)]
        lines += ["%s.theta = 0" % name, "%s.axis.x = 0" % name, "%s.axis.y = 0" % name, "%s.axis.z = 1" % name]
    lines += ["volume.min.x = 0", "volume.min.y = 0", "volume.min.z = 0",
              "volume.max.x = 20", "volume.max.y = 20", "volume.max.z = 20", "[planner]", "rrt.range = 2.5"]
    (tmp_path / "prob.cfg").write_text("\n".join(lines) + "\n")
    pr = ingest.se3_problem(str(tmp_path / "prob.cfg"))
    assert np.array_equal(pr["env_tris"], sc["env_tris"])
    rv = sc["robot_tris"].reshape(-1, 3)
    c = np.unique(rv, axis=0).mean(axis=0)
    assert np.allclose(pr["robot_tris"].reshape(-1, 3), rv - c)
    assert np.array_equal(pr["start"], np.concatenate([[0, 0, 0, 1.0], s]))
    assert pr["range"] == 2.5 and pr["weights"] == (50.0, 1.0)
    assert pr["edge_step"] == (math.sqrt(3 * 400.0) + 50 * math.pi / 2) * 0.01
    assert list(pr["lo"][4:]) == [0, 0, 0] and list(pr["hi"][4:]) == [20, 20, 20]


@pytest.mark.timeout(10)
@pytest.mark.parametrize("data", [
    b"P5\n64",                          # header ends inside the width
    b"P5",                              # no header at all
    b"P6 2 # a comment to the end",     # comment, then nothing
    b"P5 2 2 255\n\x00\x01\x02",        # one sample short
    b"P4\n9 2\n\xff\xff\xff",           # one packed byte short
    b"P2 2 2 255\n1 2 x 4\n",           # a sample that is not a number
    b"P3 2 1 255\n1 2 3 4 5\n",         # one sample short
    b"P1\n3 2\n1 0 1\n0\n",             # one bit short
    b"P6 0 2 255\n",                    # empty image
    b"P5 2 2 70000\n",                  # maximum value beyond 16 bits
    b"P5 2 -2 255\n",                   # a signed size
])
def test_pnm_malformed_inputs_raise(tmp_path, data):
    """A malformed or truncated Netpbm file is a ValueError, never a hang or
    a numpy error (a header cut short used to loop for ever)."""
    p = tmp_path / "bad.pnm"
    p.write_bytes(data)
    with pytest.raises(ValueError):
        ingest.read_image(str(p))


def test_png_malformed_inputs_raise(tmp_path):
    """Unsupported colour type / depth pairs, a palette image without PLTE or
    with an index beyond it, corrupt and truncated data: each a ValueError."""
    rows = np.zeros((2, 2), dtype=np.uint8)
    raw = _filtered(rows, 1)
    cases = [dict(ctype=5, depth=8), dict(ctype=3, depth=16), dict(ctype=2, depth=4), dict(ctype=3, depth=8)]
    for i, c in enumerate(cases):  # the last: a palette image without its PLTE
        p = tmp_path / ("c%d.png" % i)
        _write_png(p, 2, 2, c["ctype"], c["depth"], raw)
        with pytest.raises(ValueError):
            ingest.read_image(str(p))
    p = tmp_path / "idx.png"  # index 7 into a 2-entry palette
    _write_png(p, 2, 2, 3, 8, _filtered(np.array([[0, 1], [7, 0]], dtype=np.uint8), 1),
               palette=[[0, 0, 0], [255, 255, 255]])
    with pytest.raises(ValueError):
        ingest.read_image(str(p))
    good = tmp_path / "good.png"
    _write_png(good, 2, 2, 0, 8, raw)
    assert ingest.read_image(str(good)).shape == (2, 2, 3)
    data = good.read_bytes()
    for cut in (len(data) - 20, 40, 20):  # inside IDAT, inside a chunk header, inside IHDR
        q = tmp_path / ("cut%d.png" % cut)
        q.write_bytes(data[:cut])
        with pytest.raises(ValueError):
            ingest.read_image(str(q))
    bad = bytearray(data)
    i = data.index(b"IDAT") + 4
    bad[i:i + 4] = b"\xff\xff\xff\xff"  # corrupt the compressed stream
    q = tmp_path / "corrupt.png"
    q.write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        ingest.read_image(str(q))
