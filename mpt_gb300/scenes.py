"""Seeded synthetic scenes and workloads for the planner hot path.

The reference's demos read a PNG occupancy grid, a hand-written arm scene and
OMPL.app meshes through assimp/libpng; none of those inputs or libraries are
available, so each workload is synthesised from a seed with the shapes, sizes
and value ranges of the benchmark configurations:

* ``grid_scene``  -- 1024x1024 uint8 occupancy grid, 40 axis-aligned rectangles
  with sides U[20, 200] px; start (10, 10) and goal (1014, 1014) forced free.
  Model: demo/png_2d_scenario.hpp:104-110 (cell = (int)(x + 0.5)).
* ``arm_scene``   -- planar 10-link arm, links 0.1 long, base at the origin,
  64 discs with radius U(0.02, 0.08) centred in [-1, 1]^2 and none closer than
  0.1 to the base.  Model: demo/link_manipulator_scenario.hpp:99-116.
* ``mesh_scene``  -- SE(3) rigid body: star-shaped closed robot mesh of 2,048
  triangles (radii U[0.5, 1.0]) against ~250k environment triangles made of
  400 tessellated boxes plus a wall with one square aperture, in a 20^3 cube.
  Model: demo/se3_rigid_body_scenario.hpp:282-312.

State layouts: grid (x, y); arm (theta_0..theta_9); SE(3)
(qx, qy, qz, qw, px, py, pz) -- the quaternion coefficient order of Eigen's
coeffs() that src/mpt/so3_space.hpp:52-55 sums.
"""
from __future__ import annotations

import math

import numpy as np

L2, SO2, SO3, SE3, L1 = 0, 1, 2, 3, 4


# --------------------------------------------------------------------------- grid
def grid_scene(seed: int = 20261204, width: int = 1024, height: int = 1024, nrect: int = 40,
               side_min: int = 20, side_max: int = 200, free_radius: int = 12):
    rng = np.random.default_rng(seed)
    grid = np.zeros((height, width), dtype=np.uint8)
    for _ in range(nrect):
        sx, sy = rng.integers(side_min, side_max + 1, size=2)
        x0 = int(rng.integers(0, width - sx + 1))
        y0 = int(rng.integers(0, height - sy + 1))
        grid[y0:y0 + sy, x0:x0 + sx] = 1
    start = np.array([10.0, 10.0])
    goal = np.array([width - 10.0, height - 10.0])
    for c in (start, goal):
        cx, cy = int(c[0]), int(c[1])
        grid[max(0, cy - free_radius):cy + free_radius + 1, max(0, cx - free_radius):cx + free_radius + 1] = 0
    return {
        "kind": "grid", "grid": grid, "metric": L2, "dim": 2, "weights": (1.0, 1.0),
        "lo": np.array([0.0, 0.0]), "hi": np.array([float(width), float(height)]),
        "start": start, "goal": goal, "goal_radius": 8.0, "range": 32.0,
        "edge_step": 1.0, "resolution": 0,
    }


# --------------------------------------------------------------------------- arm
def _arm_clearance(q: np.ndarray, link_len: np.ndarray, discs: np.ndarray) -> np.ndarray:
    """Smallest (link-to-disc distance - radius) over links and discs, vectorised.
    Used only to pick start/goal states with a clear margin."""
    q = np.atleast_2d(q)
    ang = np.cumsum(q, axis=1)
    px = np.concatenate([np.zeros((q.shape[0], 1)), np.cumsum(link_len * np.cos(ang), axis=1)], axis=1)
    py = np.concatenate([np.zeros((q.shape[0], 1)), np.cumsum(link_len * np.sin(ang), axis=1)], axis=1)
    def pt_seg(qx, qy, ax, ay, bx, by):
        vx, vy = bx - ax, by - ay
        c2 = vx * vx + vy * vy
        t = np.clip(((qx - ax) * vx + (qy - ay) * vy) / np.maximum(c2, 1e-300), 0.0, 1.0)
        dx, dy = ax + t * vx - qx, ay + t * vy - qy
        return np.sqrt(dx * dx + dy * dy)

    best = np.full(q.shape[0], np.inf)
    for i in range(q.shape[1]):
        ax, ay, bx, by = px[:, i:i + 1], py[:, i:i + 1], px[:, i + 1:i + 2], py[:, i + 1:i + 2]
        d = pt_seg(discs[None, :, 0], discs[None, :, 1], ax, ay, bx, by) - discs[None, :, 2]
        best = np.minimum(best, d.min(axis=1))
    # non-adjacent links: distance between the segments (the minimum of the four
    # endpoint-to-segment distances, valid when they do not cross; crossing
    # segments have an endpoint distance that the orientation test catches below)
    for i in range(q.shape[1]):
        for j in range(i + 2, q.shape[1]):
            a = (px[:, i], py[:, i], px[:, i + 1], py[:, i + 1])
            b = (px[:, j], py[:, j], px[:, j + 1], py[:, j + 1])
            d = np.minimum.reduce([pt_seg(a[0], a[1], *b), pt_seg(a[2], a[3], *b), pt_seg(b[0], b[1], *a),
                                   pt_seg(b[2], b[3], *a)])

            def orient(p, r, s):
                return (r[0] - p[0]) * (s[1] - p[1]) - (r[1] - p[1]) * (s[0] - p[0])
            o1 = orient((a[0], a[1]), (a[2], a[3]), (b[0], b[1]))
            o2 = orient((a[0], a[1]), (a[2], a[3]), (b[2], b[3]))
            o3 = orient((b[0], b[1]), (b[2], b[3]), (a[0], a[1]))
            o4 = orient((b[0], b[1]), (b[2], b[3]), (a[2], a[3]))
            cross = (o1 * o2 <= 0) & (o3 * o4 <= 0)
            best = np.minimum(best, np.where(cross, -1.0, d))
    return best


def arm_scene(seed: int = 20261205, nlinks: int = 10, link: float = 0.1, ndiscs: int = 64,
              r_min: float = 0.02, r_max: float = 0.08, base_clear: float = 0.1):
    rng = np.random.default_rng(seed)
    discs = []
    while len(discs) < ndiscs:
        r = rng.uniform(r_min, r_max)
        c = rng.uniform(-1.0, 1.0, size=2)
        if math.hypot(c[0], c[1]) - r < base_clear:
            continue
        discs.append((c[0], c[1], r))
    discs = np.array(discs, dtype=np.float64)
    link_len = np.full(nlinks, link, dtype=np.float64)
    pts = []
    while len(pts) < 2:
        cand = rng.uniform(-math.pi, math.pi, size=(256, nlinks))
        cl = _arm_clearance(cand, link_len, discs)
        for i in np.nonzero(cl > 0.02)[0]:
            pts.append(cand[i])
            if len(pts) == 2:
                break
    return {
        "kind": "arm", "link_len": link_len, "discs": discs, "robot_radius": 0.0, "self_collision": 1,
        "metric": SO2, "dim": nlinks, "weights": (1.0, 1.0),
        "lo": np.full(nlinks, -math.pi), "hi": np.full(nlinks, math.pi),
        "start": pts[0], "goal": pts[1], "goal_radius": 1e-6, "range": 1.0,
        "edge_step": 0.01, "resolution": 1,
    }


# --------------------------------------------------------------------------- mesh
def _sphere_mesh(rng, n_lon: int = 32, n_bands: int = 33, r_min: float = 0.5, r_max: float = 1.0):
    """Closed star-shaped mesh: a latitude/longitude sphere with per-vertex radii.
    2 * n_lon * (n_bands - 1) triangles (2,048 for the defaults)."""
    verts = [np.array([0.0, 0.0, 1.0]) * rng.uniform(r_min, r_max)]
    for b in range(1, n_bands):
        th = math.pi * b / n_bands
        for k in range(n_lon):
            ph = 2 * math.pi * k / n_lon
            d = np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])
            verts.append(d * rng.uniform(r_min, r_max))
    verts.append(np.array([0.0, 0.0, -1.0]) * rng.uniform(r_min, r_max))
    V = np.array(verts)
    top, bot = 0, len(verts) - 1

    def ring(b, k):
        return 1 + (b - 1) * n_lon + (k % n_lon)

    tris = []
    for k in range(n_lon):
        tris.append((top, ring(1, k), ring(1, k + 1)))
    for b in range(1, n_bands - 1):
        for k in range(n_lon):
            a, bb, c, d = ring(b, k), ring(b, k + 1), ring(b + 1, k), ring(b + 1, k + 1)
            tris.append((a, c, bb))
            tris.append((bb, c, d))
    for k in range(n_lon):
        tris.append((bot, ring(n_bands - 1, k + 1), ring(n_bands - 1, k)))
    T = V[np.array(tris)]  # (ntri, 3, 3)
    return T.reshape(-1, 9), float(np.linalg.norm(V, axis=1).max())


def _box_tris(lo, hi, k: int) -> np.ndarray:
    """Axis-aligned box surface, each face tessellated into a k x k grid of quads
    (2 triangles each): 12 k^2 triangles."""
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    out = []
    u = np.linspace(0.0, 1.0, k + 1)
    for axis in range(3):
        a1, a2 = [d for d in range(3) if d != axis]
        for side in (lo[axis], hi[axis]):
            P = np.zeros((k + 1, k + 1, 3))
            P[..., axis] = side
            P[..., a1] = lo[a1] + (hi[a1] - lo[a1]) * u[:, None]
            P[..., a2] = lo[a2] + (hi[a2] - lo[a2]) * u[None, :]
            p00, p10, p01, p11 = P[:-1, :-1], P[1:, :-1], P[:-1, 1:], P[1:, 1:]
            t1 = np.stack([p00, p10, p11], axis=2).reshape(-1, 9)
            t2 = np.stack([p00, p11, p01], axis=2).reshape(-1, 9)
            out += [t1, t2]
    return np.concatenate(out)


def mesh_scene(seed: int = 20261206, nboxes: int = 400, cube: float = 20.0, box_k: int = 7,
               wall_k: int = 15, aperture_factor: float = 1.3, wall_thickness: float = 0.5):
    rng = np.random.default_rng(seed)
    robot, rbound = _sphere_mesh(rng)
    boxes = []
    wall_x = cube / 2
    half_ap = aperture_factor * rbound  # aperture side = 2 * 1.3 * bounding radius
    ay, az = cube / 2, cube / 2
    # the wall: four boxes framing the square aperture
    w0, w1 = wall_x - wall_thickness / 2, wall_x + wall_thickness / 2
    wall = [((w0, 0, 0), (w1, ay - half_ap, cube)), ((w0, ay + half_ap, 0), (w1, cube, cube)),
            ((w0, ay - half_ap, 0), (w1, ay + half_ap, az - half_ap)),
            ((w0, ay - half_ap, az + half_ap), (w1, ay + half_ap, cube))]
    while len(boxes) < nboxes:
        size = rng.uniform(0.4, 1.6, size=3)
        lo = rng.uniform(0.0, cube - size)
        hi = lo + size
        # keep the aperture's corridor open
        if lo[0] < wall_x + 3 and hi[0] > wall_x - 3 and lo[1] < ay + half_ap + 1 and hi[1] > ay - half_ap - 1 \
                and lo[2] < az + half_ap + 1 and hi[2] > az - half_ap - 1:
            continue
        boxes.append((lo, hi))
    env = [_box_tris(lo, hi, box_k) for lo, hi in boxes] + [_box_tris(lo, hi, wall_k) for lo, hi in wall]
    env = np.concatenate(env)
    all_boxes = [(np.asarray(lo, float), np.asarray(hi, float)) for lo, hi in boxes + wall]

    def clear(p, margin):
        for lo, hi in all_boxes:
            d = np.maximum(np.maximum(lo - p, p - hi), 0.0)
            if np.linalg.norm(d) < rbound + margin:
                return False
        return bool(np.all(p > rbound + margin) and np.all(p < cube - rbound - margin))

    def pick(xlo, xhi):
        while True:
            p = np.array([rng.uniform(xlo, xhi), rng.uniform(0, cube), rng.uniform(0, cube)])
            if clear(p, 0.05):
                return p

    ident = np.array([0.0, 0.0, 0.0, 1.0])
    start = np.concatenate([ident, pick(1.0, wall_x - 2.0)])
    goal = np.concatenate([ident, pick(wall_x + 2.0, cube - 1.0)])
    return {
        "kind": "mesh", "robot_tris": robot, "env_tris": env, "robot_bound": rbound,
        "metric": SE3, "dim": 7, "weights": (2.0, 1.0),
        "lo": np.array([-1, -1, -1, -1, 0, 0, 0], float), "hi": np.array([1, 1, 1, 1, cube, cube, cube], float),
        "start": start, "goal": goal, "goal_radius": 1e-6, "range": 2.0,
        "edge_step": 0.05, "resolution": 0, "boxes": all_boxes,
    }


def near_contact_states(scene: dict, n: int, seed: int) -> np.ndarray:
    """SE(3) states whose robot sits within about one bounding radius of a box
    face (random orientation): the near-contact half of the surrogate's
    training set."""
    rng = np.random.default_rng(seed)
    boxes = scene["boxes"]
    out = uniform_states(scene, n, seed + 1)
    for i in range(n):
        lo, hi = boxes[rng.integers(len(boxes))]
        p = rng.uniform(lo, hi)
        ax = rng.integers(3)
        side = rng.integers(2)
        p[ax] = (hi if side else lo)[ax] + (1 if side else -1) * rng.uniform(0.3, 1.2) * scene["robot_bound"]
        out[i, 4:] = p
    return out


# --------------------------------------------------------------------------- samplers
def uniform_states(scene: dict, n: int, seed: int) -> np.ndarray:
    """Uniform states in the scene's sampling space (box for Lp/SO(2)^n, Shoemake
    uniform rotation for SO(3) as in src/mpt/impl/uniform_sampler_so3.hpp:55-68)."""
    rng = np.random.default_rng(seed)
    m, d = scene["metric"], scene["dim"]
    if m in (L2, L1, SO2):
        lo, hi = scene["lo"], scene["hi"]
        return rng.uniform(lo, hi, size=(n, d))
    if m in (SO3, SE3):
        a = rng.uniform(0, 1, n)
        b = rng.uniform(0, 2 * math.pi, n)
        c = rng.uniform(0, 2 * math.pi, n)
        q = np.stack([np.sqrt(1 - a) * np.sin(b), np.sqrt(1 - a) * np.cos(b), np.sqrt(a) * np.sin(c),
                      np.sqrt(a) * np.cos(c)], axis=1)
        if m == SO3:
            return q
        lo, hi = scene["lo"][4:], scene["hi"][4:]
        return np.concatenate([q, rng.uniform(lo, hi, size=(n, 3))], axis=1)
    raise ValueError(m)


def steered_edges(scene: dict, n: int, seed: int, near_frac: float = 0.5):
    """Edge lists for the validity checks: pairs (a, b) at most the steer range
    apart in the scene's metric (b = interpolate(a, c, range/d) of a random c)."""
    from_ = uniform_states(scene, n, seed)
    to = uniform_states(scene, n, seed + 1)
    rng = np.random.default_rng(seed + 2)
    r = scene["range"]
    m = scene["metric"]
    out = np.empty_like(to)
    for i in range(n):
        a, c = from_[i], to[i]
        frac = rng.uniform(0.2, 1.0)
        if m == L2:
            d = np.linalg.norm(c - a)
            t = min(1.0, r * frac / d) if d > 0 else 1.0
            out[i] = (c - a) * t + a
        elif m == SO2:
            dd = np.mod(c - a + math.pi, 2 * math.pi) - math.pi
            tot = np.abs(dd).sum()
            t = min(1.0, r * frac / tot) if tot > 0 else 1.0
            out[i] = np.mod(a + dd * t + math.pi, 2 * math.pi) - math.pi
        else:
            dp = c[4:] - a[4:]
            dn = np.linalg.norm(dp)
            t = min(1.0, r * frac / max(dn, 1e-12))
            # small rotation change: slerp fraction of the way to c
            qa, qc = a[:4], c[:4]
            if np.dot(qa, qc) < 0:
                qc = -qc
            q = qa + (qc - qa) * min(1.0, 0.3 * frac)
            q /= np.linalg.norm(q)
            out[i] = np.concatenate([q, a[4:] + dp * t])
    return from_, out
