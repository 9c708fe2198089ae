"""Synthetic depth-frame generator for the fusion workloads.

The reference is driven by recorded RGB-D datasets (ICL-NUIM, TUM, SUN3D, PKU),
which are not available here.  This module renders seeded synthetic depth
frames with the same shapes, depth range and value distribution:

* an analytic scene: the interior of a box room plus spheres and solid
  axis-aligned boxes, intersected exactly in float64;
* camera trajectories (a circle looking at the room centre, or a smooth random
  6-DoF path with bounded speed);
* sensor noise: Gaussian sigma = 0.0012 * z^2, uniform outliers and missing
  (zero) pixels, all drawn from a seeded ``numpy.random.Generator``.

Depth is z-depth in metres in the reference's camera convention: x right,
y down, z forward, pixel (u, v) -> ((u - cx) / fx * z, (v - cy) / fy * z, z)
(``geometry/geometry_helper.h:163-170``).  Poses are camera-to-world ``wTc``
as row-major float32 4x4 matrices, like ``Sensor::wTc`` (``sensor/rgbd_sensor.h``).

Everything here is input generation only; nothing in it is on the fusion path.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np


@dataclasses.dataclass
class Scene:
    room_lo: np.ndarray                      # (3,) interior box lower corner
    room_hi: np.ndarray                      # (3,)
    spheres: np.ndarray                      # (S, 4): cx, cy, cz, r
    boxes: np.ndarray                        # (B, 6): lo xyz, hi xyz
    rooms: Optional[np.ndarray] = None       # unused by the single-room scenes

    def hit(self, o: np.ndarray, d: np.ndarray) -> np.ndarray:
        """Nearest positive hit distance along rays ``o + t d`` (d unnormalised).

        o: (3,), d: (N, 3).  Returns (N,) float64, +inf where nothing is hit.
        """
        n = d.shape[0]
        t = np.full(n, np.inf)
        # room interior: the ray leaves the box through the nearest face
        with np.errstate(divide="ignore", invalid="ignore"):
            for ax in range(3):
                da = d[:, ax]
                tp = np.where(da > 0, (self.room_hi[ax] - o[ax]) / da, np.inf)
                tn = np.where(da < 0, (self.room_lo[ax] - o[ax]) / da, np.inf)
                t = np.minimum(t, np.minimum(tp, tn))
            for cx, cy, cz, r in self.spheres:
                oc = o - np.array([cx, cy, cz])
                a = np.einsum("ij,ij->i", d, d)
                b = d @ oc
                c = oc @ oc - r * r
                disc = b * b - a * c
                ok = disc >= 0
                sq = np.sqrt(np.where(ok, disc, 0.0))
                t0 = (-b - sq) / a
                t1 = (-b + sq) / a
                th = np.where(t0 > 1e-9, t0, np.where(t1 > 1e-9, t1, np.inf))
                t = np.minimum(t, np.where(ok, th, np.inf))
            for bx in self.boxes:
                lo, hi = bx[:3], bx[3:]
                inv = 1.0 / d
                t1 = (lo - o) * inv
                t2 = (hi - o) * inv
                tmin = np.nanmax(np.minimum(t1, t2), axis=1)
                tmax = np.nanmin(np.maximum(t1, t2), axis=1)
                ok = (tmax >= tmin) & (tmax > 1e-9)
                th = np.where(tmin > 1e-9, tmin, tmax)
                t = np.minimum(t, np.where(ok, th, np.inf))
        return t


@dataclasses.dataclass
class Camera:
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float

    def rays(self) -> np.ndarray:
        """Camera-frame ray directions with z == 1, shape (H*W, 3), row-major."""
        u = np.arange(self.width, dtype=np.float64)
        v = np.arange(self.height, dtype=np.float64)
        uu, vv = np.meshgrid(u, v)
        x = (uu - self.cx) / self.fx
        y = (vv - self.cy) / self.fy
        return np.stack([x.ravel(), y.ravel(), np.ones(x.size)], axis=1)


def look_at(pos, target, roll: float = 0.0) -> np.ndarray:
    """Camera-to-world pose: +z towards ``target``, +y down (world up is +z)."""
    pos = np.asarray(pos, np.float64)
    f = np.asarray(target, np.float64) - pos
    f /= np.linalg.norm(f)
    up = np.array([0.0, 0.0, 1.0])
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    dn = np.cross(f, r)
    if roll:
        c, s = math.cos(roll), math.sin(roll)
        r, dn = c * r + s * dn, -s * r + c * dn
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, dn, f, pos
    return m


def render_depth(scene: Scene, cam: Camera, wTc: np.ndarray) -> np.ndarray:
    """Noise-free z-depth image (H, W) float64; 0 where nothing is hit."""
    dc = cam.rays()
    R = wTc[:3, :3]
    o = wTc[:3, 3]
    dw = dc @ R.T
    t = scene.hit(o, dw)          # with d_cam.z == 1 the hit parameter is z
    t = np.where(np.isfinite(t), t, 0.0)
    return t.reshape(cam.height, cam.width)


def add_noise(depth: np.ndarray, rng: np.random.Generator, sigma_coef: float = 0.0012,
              outlier_frac: float = 0.0, outlier_range=(0.3, 5.0),
              zero_frac: float = 0.0) -> np.ndarray:
    """Gaussian sigma = sigma_coef * z^2, then uniform outliers, then zeros."""
    z = depth.copy()
    valid = z > 0
    z = z + rng.standard_normal(z.shape) * sigma_coef * z * z
    z = np.where(valid, z, 0.0)
    if outlier_frac > 0:
        m = rng.random(z.shape) < outlier_frac
        z = np.where(m, rng.uniform(outlier_range[0], outlier_range[1], z.shape), z)
    if zero_frac > 0:
        m = rng.random(z.shape) < zero_frac
        z = np.where(m, 0.0, z)
    return z


# ---------------------------------------------------------------- scenes

ROOM_LO = np.array([-2.0, -2.0, 0.0])
ROOM_HI = np.array([2.0, 2.0, 3.0])
CORNERS = [(1.4, 1.4), (-1.4, 1.4), (-1.4, -1.4), (1.4, -1.4)]


def room_scene(seed: int, extra: int = 0) -> Scene:
    """4x4x3 m box room with 3 spheres (r 0.3-0.6 m) and 2 axis-aligned boxes.

    One sphere sits near the room centre, the other four primitives in the
    corners, so a camera on the 1.2 m circle (or the 0.95-1.35 m annulus of
    the spline path) never enters them.  ``extra`` adds small random
    primitives in the same free regions.
    """
    rng = np.random.default_rng(1000 + seed)
    corners = list(CORNERS)
    rng.shuffle(corners)
    sph = []
    r0 = rng.uniform(0.3, 0.5)
    off = rng.uniform(-0.15, 0.15, 2)
    sph.append([off[0], off[1], rng.uniform(0.6, 1.3), r0])
    for k in range(2):
        r = rng.uniform(0.3, 0.6)
        cx, cy = corners[k]
        sph.append([cx, cy, rng.uniform(r, 2.0), r])
    boxes = []
    for k in range(2, 4):
        cx, cy = corners[k]
        h = rng.uniform(0.2, 0.4, 2)
        top = rng.uniform(0.3, 1.2)
        boxes.append([cx - h[0], cy - h[1], 0.0, cx + h[0], cy + h[1], top])
    for _ in range(extra):
        size = rng.uniform(0.08, 0.25)
        while True:
            ang = rng.uniform(0, 2 * math.pi)
            # (the outer ring is empty for size > 0.225: its range collapses to a point)
            rad = rng.choice([rng.uniform(0.0, 0.7 - size), rng.uniform(1.55 + size, max(2.0 - size, 1.55 + size))])
            x, y = rad * math.cos(ang), rad * math.sin(ang)
            if abs(x) <= 2.0 - size and abs(y) <= 2.0 - size:
                break
        z = rng.uniform(size, 3.0 - size)
        if rng.random() < 0.5:
            sph.append([x, y, z, size])
        else:
            boxes.append([x - size, y - size, z - size, x + size, y + size, z + size])
    return Scene(ROOM_LO.copy(), ROOM_HI.copy(), np.array(sph, np.float64),
                 np.array(boxes, np.float64).reshape(-1, 6))


def circle_trajectory(n: int, radius: float = 1.2, height: float = 1.5,
                      centre=(0.0, 0.0, 1.5)) -> List[np.ndarray]:
    """n poses on a horizontal circle, each looking at ``centre``."""
    poses = []
    for i in range(n):
        a = 2 * math.pi * i / n
        p = (radius * math.cos(a), radius * math.sin(a), height)
        poses.append(look_at(p, centre))
    return poses


def spline_trajectory(n: int, seed: int, fps: float = 30.0, vmax: float = 0.5) -> List[np.ndarray]:
    """Smooth random 6-DoF path with speed <= vmax at ``fps`` frames/s.

    Position: angle, radius (0.95-1.35 m) and height (1.2-1.8 m) are sums of
    low-frequency sinusoids; orientation looks at a jittered point near the
    room centre with a small roll.  The time axis is rescaled so that the
    finite-difference speed never exceeds ``vmax``.
    """
    rng = np.random.default_rng(2000 + seed)

    def smooth(k, amp):
        fr = rng.uniform(0.05, 0.25, k)
        ph = rng.uniform(0, 2 * math.pi, k)
        am = amp * rng.uniform(0.5, 1.0, k) / k
        return lambda s: float(np.sum(am * np.sin(2 * math.pi * fr * s + ph)))

    th0 = rng.uniform(0, 2 * math.pi)
    w = rng.choice([-1, 1]) * rng.uniform(0.15, 0.3)
    rad, hgt = smooth(3, 0.18), smooth(3, 0.25)
    tx, ty, tz, roll = smooth(3, 0.3), smooth(3, 0.3), smooth(3, 0.2), smooth(2, 0.08)

    def pos(s):
        a = th0 + w * s
        r = 1.15 + rad(s)
        return np.array([r * math.cos(a), r * math.sin(a), 1.5 + hgt(s)])

    dt = 1.0 / fps
    ss = [0.0]
    for _ in range(n - 1):
        s = ss[-1]
        v = np.linalg.norm(pos(s + 1e-3) - pos(s)) / 1e-3
        step = dt if v * dt <= vmax * dt else dt * vmax / v
        ss.append(s + step * 0.98)
    poses = []
    for s in ss:
        tgt = np.array([tx(s), ty(s), 1.2 + tz(s)])
        poses.append(look_at(pos(s), tgt, roll(s)))
    return poses


# ---------------------------------------------------------------- floor plan

PLAN_LO = np.array([-6.0, -5.0, 0.0])
PLAN_HI = np.array([6.0, 5.0, 3.0])
_WALL = 0.05          # half thickness of interior walls
_DOOR_W, _DOOR_H = 0.5, 2.1   # half width, height of a doorway


def _room_centre(i: int, j: int) -> np.ndarray:
    return np.array([-4.0 + 4.0 * i, -2.5 + 5.0 * j, 0.0])


def _wall_slabs():
    """Interior walls of the 3 x 2 room grid as solid slabs, with a doorway
    on every room-centre line (x = -2, 2 at y = -2.5, 2.5; y = 0 at x = -4, 0, 4)."""
    slabs = []

    def wall_x(x, doors):
        # wall at x spanning y in [-5, 5], doors centred at `doors`
        edges = [-5.0] + [e for c in sorted(doors) for e in (c - _DOOR_W, c + _DOOR_W)] + [5.0]
        for a, b in zip(edges[0::2], edges[1::2]):
            slabs.append([x - _WALL, a, 0.0, x + _WALL, b, 3.0])
        for c in doors:
            slabs.append([x - _WALL, c - _DOOR_W, _DOOR_H, x + _WALL, c + _DOOR_W, 3.0])

    def wall_y(y, doors):
        edges = [-6.0] + [e for c in sorted(doors) for e in (c - _DOOR_W, c + _DOOR_W)] + [6.0]
        for a, b in zip(edges[0::2], edges[1::2]):
            slabs.append([a, y - _WALL, 0.0, b, y + _WALL, 3.0])
        for c in doors:
            slabs.append([c - _DOOR_W, y - _WALL, _DOOR_H, c + _DOOR_W, y + _WALL, 3.0])

    wall_x(-2.0, [-2.5, 2.5])
    wall_x(2.0, [-2.5, 2.5])
    wall_y(0.0, [-4.0, 0.0, 4.0])
    return slabs


# the walk: room centres in loop order (through the doorways between them)
_LOOP = [(0, 0), (1, 0), (2, 0), (2, 1), (1, 1), (0, 1), (0, 0)]


def _dist_to_path(x: float, y: float) -> float:
    best = np.inf
    for (i0, j0), (i1, j1) in zip(_LOOP[:-1], _LOOP[1:]):
        a, b = _room_centre(i0, j0)[:2], _room_centre(i1, j1)[:2]
        ab = b - a
        t = np.clip(np.dot(np.array([x, y]) - a, ab) / np.dot(ab, ab), 0.0, 1.0)
        best = min(best, float(np.linalg.norm(np.array([x, y]) - (a + t * ab))))
    return best


def floor_plan_scene(seed: int = 0, n_primitives: int = 40) -> Scene:
    """12 x 10 x 3 m floor plan: 6 rooms (3 x 2) separated by walls with
    doorways, and n_primitives random boxes and spheres inside the rooms,
    clear of the walls and of the walking path."""
    rng = np.random.default_rng(5000 + seed)
    sph, boxes = [], list(_wall_slabs())
    while len(sph) + len(boxes) - len(_wall_slabs()) < n_primitives:
        size = rng.uniform(0.1, 0.4)
        i, j = int(rng.integers(0, 3)), int(rng.integers(0, 2))
        c = _room_centre(i, j)
        x = c[0] + rng.uniform(-2.0 + _WALL + size + 0.2, 2.0 - _WALL - size - 0.2)
        y = c[1] + rng.uniform(-2.5 + _WALL + size + 0.2, 2.5 - _WALL - size - 0.2)
        if _dist_to_path(x, y) < size + 0.7:
            continue
        z = rng.uniform(size, 2.6 - size) if rng.random() < 0.4 else size
        if rng.random() < 0.5:
            sph.append([x, y, z, size])
        else:
            boxes.append([x - size, y - size, z - size, x + size, y + size, z + size])
    return Scene(PLAN_LO.copy(), PLAN_HI.copy(), np.array(sph, np.float64).reshape(-1, 4),
                 np.array(boxes, np.float64).reshape(-1, 6))


def floor_plan_walk(n: int, seed: int = 0, fps: float = 30.0, speed: float = 0.4) -> List[np.ndarray]:
    """n poses walking the room loop at `speed` m/s (<= 0.5), eye height about
    1.5 m, heading along the path (smoothed over +-0.6 m of arc) with a slow
    look-around of +-35 degrees and a slight downward pitch."""
    rng = np.random.default_rng(6000 + seed)
    pts = [_room_centre(i, j)[:2] for i, j in _LOOP]
    seg = [np.linalg.norm(b - a) for a, b in zip(pts[:-1], pts[1:])]
    total = float(sum(seg))

    def at(sarc):
        sarc = sarc % total
        for (a, b), L in zip(zip(pts[:-1], pts[1:]), seg):
            if sarc <= L:
                return a + (b - a) * (sarc / L)
            sarc -= L
        return pts[-1]

    ph1, ph2 = rng.uniform(0, 2 * math.pi, 2)
    poses = []
    for k in range(n):
        t = k / fps
        sarc = speed * t + 0.3
        p = at(sarc)
        dvec = at(sarc + 0.6) - at(sarc - 0.6)
        yaw = math.atan2(dvec[1], dvec[0]) + math.radians(35.0) * math.sin(2 * math.pi * t / 6.0 + ph1)
        z = 1.5 + 0.08 * math.sin(2 * math.pi * t / 4.0 + ph2)
        pos = np.array([p[0], p[1], z])
        target = pos + np.array([math.cos(yaw), math.sin(yaw), -0.18])
        poses.append(look_at(pos, target, roll=0.03 * math.sin(2 * math.pi * t / 5.0)))
    return poses


# ---------------------------------------------------------------- workloads

@dataclasses.dataclass
class Workload:
    name: str
    scene: Scene
    camera: Camera
    poses: List[np.ndarray]
    noise: dict
    seed: int

    def frame(self, i: int) -> np.ndarray:
        """Depth frame i as float32 (H, W) in metres (0 = missing)."""
        clean = render_depth(self.scene, self.camera, self.poses[i])
        rng = np.random.default_rng([self.seed, i])
        return add_noise(clean, rng, **self.noise).astype(np.float32)

    def pose(self, i: int) -> np.ndarray:
        return self.poses[i].astype(np.float32)


def small_circle(n_frames: int = 60, seed: int = 0) -> Workload:
    """Plain TSDF case: 320x240, fx=fy=262.5, circle r=1.2 m at 1.5 m height."""
    cam = Camera(320, 240, 262.5, 262.5, 159.5, 119.5)
    return Workload("room320_circle", room_scene(seed), cam, circle_trajectory(n_frames),
                    dict(sigma_coef=0.0012), seed)


def full_spline(n_frames: int = 500, seed: int = 0, width: int = 640, height: int = 480) -> Workload:
    """PSDF case: 640x480, fx=fy=525, spline path, outliers 5 %, zeros 2 %."""
    s = width / 640.0
    cam = Camera(width, height, 525.0 * s, 525.0 * s, (width - 1) / 2.0, (height - 1) / 2.0)
    return Workload(f"room{width}_spline", room_scene(seed, extra=6), cam,
                    spline_trajectory(n_frames, seed),
                    dict(sigma_coef=0.0012, outlier_frac=0.05, outlier_range=(0.3, 5.0),
                         zero_frac=0.02), seed)


def floor_plan(n_frames: int = 2000, seed: int = 0, width: int = 640, height: int = 480) -> Workload:
    """Large-scene streaming case: the 12 x 10 x 3 m floor plan walked at
    0.4 m/s, 640x480 (fx = fy = 525 at that width), noise as full_spline."""
    s = width / 640.0
    cam = Camera(width, height, 525.0 * s, 525.0 * s, (width - 1) / 2.0, (height - 1) / 2.0)
    return Workload(f"floorplan{width}_walk", floor_plan_scene(seed), cam, floor_plan_walk(n_frames, seed),
                    dict(sigma_coef=0.0012, outlier_frac=0.05, outlier_range=(0.3, 5.0), zero_frac=0.02), seed)
