"""Seeded synthetic scenes for the five benchmark workloads.

The reference measures on no dataset; these generators stand in for its
demo scenes (demo/src/circles.rs:67-138 builds circle layers the same way).
Every value comes from one u64 seed through a counter-based splitmix64, so a
scene is bit-identical on every machine and numpy version.

Workloads (sizes as named by the benchmark configurations):
  circles    1,000 circle layers (64-segment polygons) on 1024x1024
  mixed      100,000 star/convex polygon and closed-cubic layers, random
             affine per layer, 12 blend modes, NonZero/EvenOdd, 2560x1600
  glyphs     50,000 glyph-like layers (3-6 closed quad contours) in text rows,
             EvenOdd, opaque black on white, 3840x2160
  batch      256 scenes, log-uniform layer count in [10, 50,000], canvas side
             in {256, 512, 1024, 2048}, geometry from the mixed generator
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import abi

GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def _mix(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
    return z ^ (z >> np.uint64(31))


class Rng:
    """Counter-based splitmix64: value (row r, column k) of stream `tag` is
    mix(key_r + (k + 1) * GAMMA) with key_r = mix(seed ^ mix(tag) + r * GAMMA)."""

    def __init__(self, seed: int, tag: int):
        with np.errstate(over="ignore"):
            self.base = _mix(np.uint64(seed & 0xFFFFFFFFFFFFFFFF) ^ _mix(np.uint64(tag)))

    def u64(self, rows: int, cols: int):
        with np.errstate(over="ignore"):
            r = np.arange(rows, dtype=np.uint64)[:, None]
            k = np.arange(1, cols + 1, dtype=np.uint64)[None, :]
            keys = _mix(self.base + r * GAMMA)
            return _mix(keys + k * GAMMA)

    def uniform(self, rows: int, cols: int):
        """float64 in [0, 1) with 53 random bits."""
        return (self.u64(rows, cols) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


@dataclass
class Scene:
    name: str
    width: int
    height: int
    background: tuple
    wide: bool
    n_layers: int
    # paths (one or more per layer), in the layout of cgb_insert_paths
    path_layer: np.ndarray = None      # uint32 [n_paths]
    cmd_offsets: np.ndarray = None     # uint64 [n_paths + 1]
    kinds: np.ndarray = None           # uint32 [n_cmds]
    point_offsets: np.ndarray = None   # uint64 [n_paths + 1]
    points: np.ndarray = None          # float32 [n_floats]
    # per layer
    transforms: Optional[np.ndarray] = None  # float32 [n_layers, 6] (surpass affine) or None
    fill_rule: np.ndarray = None       # uint32 [n_layers]
    blend_mode: np.ndarray = None      # uint32 [n_layers]
    color: np.ndarray = None           # float32 [n_layers, 4]
    meta: dict = field(default_factory=dict)

    @property
    def n_paths(self):
        return len(self.path_layer)

    def path(self, k):
        """Commands of path k as (kinds, points) numpy views."""
        c0, c1 = int(self.cmd_offsets[k]), int(self.cmd_offsets[k + 1])
        p0, p1 = int(self.point_offsets[k]), int(self.point_offsets[k + 1])
        return self.kinds[c0:c1], self.points[p0:p1]


def _assemble(name, width, height, background, wide, n_layers, per_path_kinds, per_path_points, path_layer,
              transforms, fill_rule, blend_mode, color, meta=None):
    counts = np.array([len(k) for k in per_path_kinds], dtype=np.uint64)
    pcounts = np.array([len(p) for p in per_path_points], dtype=np.uint64)
    cmd_offsets = np.zeros(len(counts) + 1, np.uint64)
    cmd_offsets[1:] = np.cumsum(counts)
    point_offsets = np.zeros(len(pcounts) + 1, np.uint64)
    point_offsets[1:] = np.cumsum(pcounts)
    kinds = np.concatenate(per_path_kinds).astype(np.uint32) if per_path_kinds else np.zeros(0, np.uint32)
    points = np.concatenate(per_path_points).astype(np.float32) if per_path_points else np.zeros(0, np.float32)
    return Scene(name, width, height, background, wide, n_layers, np.asarray(path_layer, np.uint32), cmd_offsets,
                 kinds, point_offsets, points, transforms, np.asarray(fill_rule, np.uint32),
                 np.asarray(blend_mode, np.uint32), np.asarray(color, np.float32), meta or {})


def _flat_scene(name, width, height, wide, n_layers, geo, transforms, fill_rule, blend_mode, color):
    """A scene with one path per layer from already-flattened command arrays."""
    kinds, points, cmd_off, pt_off = geo
    return Scene(name, width, height, (1.0, 1.0, 1.0, 1.0), wide, n_layers, np.arange(n_layers, dtype=np.uint32),
                 cmd_off, kinds, pt_off, points, transforms, np.asarray(fill_rule, np.uint32),
                 np.asarray(blend_mode, np.uint32), np.asarray(color, np.float32))


def _polygon_path(xs, ys):
    """Closed polygon as LINE commands plus CLOSE."""
    n = len(xs)
    pts = np.empty((n, 4), np.float32)
    pts[:, 0] = xs
    pts[:, 1] = ys
    pts[:, 2] = np.roll(xs, -1)
    pts[:, 3] = np.roll(ys, -1)
    kinds = np.full(n + 1, abi.CMD_LINE, np.uint32)
    kinds[-1] = abi.CMD_CLOSE
    return kinds, pts.reshape(-1)


def circles(seed: int = 1, n_layers: int = 1000, size: int = 1024, segments: int = 64) -> Scene:
    """1,000 filled circles (closed 64-segment polygons) on 1024x1024 RGBA8:
    centres U[0,size)^2, radii U[4,64], RGB U[0,1], alpha U[0.5,1], NonZero,
    Over, identity transforms, white background."""
    u = Rng(seed, 1).uniform(n_layers, 8)
    cx, cy = u[:, 0] * size, u[:, 1] * size
    r = 4.0 + u[:, 2] * 60.0
    color = np.stack([u[:, 3], u[:, 4], u[:, 5], 0.5 + 0.5 * u[:, 6]], axis=1).astype(np.float32)
    ang = np.arange(segments, dtype=np.float64) * (2.0 * np.pi / segments)
    kinds, points = [], []
    for i in range(n_layers):
        k, p = _polygon_path((cx[i] + r[i] * np.cos(ang)).astype(np.float32),
                             (cy[i] + r[i] * np.sin(ang)).astype(np.float32))
        kinds.append(k)
        points.append(p)
    return _assemble("circles", size, size, (1.0, 1.0, 1.0, 1.0), False, n_layers, kinds, points,
                     np.arange(n_layers), None, np.zeros(n_layers), np.zeros(n_layers), color)


def _mixed_geometry(rng_tag_seed, n_layers, width, height):
    """Geometry of the mixed workload, in path space around the origin, plus
    the per-layer surpass affine that places it on the canvas."""
    seed = rng_tag_seed
    U = Rng(seed, 2).uniform(n_layers, 16)
    is_poly = U[:, 0] < 0.6
    # per-layer affine: rotation U[0,2pi), uniform scale U[0.5,2], translation in the canvas
    th = U[:, 1] * 2.0 * np.pi
    s = 0.5 + 1.5 * U[:, 2]
    tx, ty = U[:, 3] * width, U[:, 4] * height
    transforms = np.stack([s * np.cos(th), -s * np.sin(th), s * np.sin(th), s * np.cos(th), tx, ty],
                          axis=1).astype(np.float32)
    fill_rule = (U[:, 5] < 0.5).astype(np.uint32)
    blend = np.minimum((U[:, 6] * 12).astype(np.uint32), 11)
    color = np.stack([U[:, 7], U[:, 8], U[:, 9], 0.2 + 0.8 * U[:, 10]], axis=1).astype(np.float32)

    # polygons: 3..32 vertices, radius log-U[2, 200]; half convex, half star
    V = Rng(seed, 3).uniform(n_layers, 2 * 32 + 4)
    nv = 3 + np.minimum((V[:, 0] * 30).astype(np.int64), 29)
    radius = np.exp(np.log(2.0) + V[:, 1] * (np.log(200.0) - np.log(2.0)))
    star = V[:, 2] < 0.5
    inner = 0.3 + 0.4 * V[:, 3]
    # cubic loops: 4..12 cubics, control points in a box of side log-U[4, 300]
    C = Rng(seed, 4).uniform(n_layers, 2 + 12 * 6 + 12)
    nc = 4 + np.minimum((C[:, 0] * 9).astype(np.int64), 8)
    box = np.exp(np.log(4.0) + C[:, 1] * (np.log(300.0) - np.log(4.0)))

    # per-layer command / float counts, then every polygon and every cubic
    # loop written at its layer's offsets (padded to 32 vertices / 12 cubics)
    n_cmd = np.where(is_poly, nv + 1, nc + 1).astype(np.int64)
    n_flt = np.where(is_poly, nv * 4, nc * 8).astype(np.int64)
    cmd_off = np.concatenate([[0], np.cumsum(n_cmd)])
    pt_off = np.concatenate([[0], np.cumsum(n_flt)])
    kinds = np.empty(int(cmd_off[-1]), np.uint32)
    points = np.empty(int(pt_off[-1]), np.float32)

    P = np.nonzero(is_poly)[0]
    if len(P):
        n = nv[P][:, None]
        k = np.arange(32)[None, :]
        mask = k < n
        ang = (k + 0.8 * V[P, 4:36]) * (2.0 * np.pi / n)
        rr = radius[P][:, None] * np.where(star[P][:, None] & (k % 2 == 1), inner[P][:, None], 1.0)
        x = (rr * np.cos(ang)).astype(np.float32)
        y = (rr * np.sin(ang)).astype(np.float32)
        nxt = (k + 1) % n
        seg = np.stack([x, y, np.take_along_axis(x, nxt, 1), np.take_along_axis(y, nxt, 1)], -1)
        dst = (pt_off[P][:, None] + 4 * k)[mask]
        points[(dst[:, None] + np.arange(4)[None, :]).reshape(-1)] = seg[mask].reshape(-1)
        kinds[(cmd_off[P][:, None] + k)[mask]] = abi.CMD_LINE
        kinds[cmd_off[P] + nv[P]] = abi.CMD_CLOSE
    Q = np.nonzero(~is_poly)[0]
    if len(Q):
        n = nc[Q][:, None]
        k = np.arange(12)[None, :]
        mask = k < n
        half = (box[Q] / 2.0)[:, None]
        a_ang = (k + 0.5 * C[Q, 2:14]) * (2.0 * np.pi / n)
        a_r = half * (0.5 + 0.5 * C[Q, 14:26])
        ax, ay = a_r * np.cos(a_ang), a_r * np.sin(a_ang)
        ctl = (C[Q, 26:74].reshape(-1, 12, 4) * 2.0 - 1.0) * half[:, :, None]
        nxt = (k + 1) % n
        pts = np.empty((len(Q), 12, 8), np.float64)
        pts[..., 0], pts[..., 1] = ax, ay
        pts[..., 2:6] = ctl
        pts[..., 6], pts[..., 7] = np.take_along_axis(ax, nxt, 1), np.take_along_axis(ay, nxt, 1)
        pts = pts.astype(np.float32)
        dst = (pt_off[Q][:, None] + 8 * k)[mask]
        points[(dst[:, None] + np.arange(8)[None, :]).reshape(-1)] = pts[mask].reshape(-1)
        kinds[(cmd_off[Q][:, None] + k)[mask]] = abi.CMD_CUBIC
        kinds[cmd_off[Q] + nc[Q]] = abi.CMD_CLOSE
    geo = (kinds, points, cmd_off.astype(np.uint64), pt_off.astype(np.uint64))
    return geo, transforms, fill_rule, blend, color


def mixed(seed: int = 2, n_layers: int = 100_000, width: int = 2560, height: int = 1600) -> Scene:
    """The hot-path-at-scale workload: star/convex polygons (60%) and closed
    4-12-cubic paths (40%), random affine, NonZero/EvenOdd 50/50, blend mode
    uniform over the 12 modes, alpha U[0.2,1], white background.  More than
    65,536 layers selects the widened (17-bit layer) segment format."""
    geo, transforms, fr, bm, color = _mixed_geometry(seed, n_layers, width, height)
    return _flat_scene(f"mixed{n_layers}", width, height, n_layers > 65536, n_layers, geo, transforms, fr, bm, color)


def glyphs(seed: int = 3, n_layers: int = 50_000, width: int = 3840, height: int = 2160,
           pitch: Optional[float] = None) -> Scene:
    """Dense text-like scene: glyph layers of 3-6 closed contours of 4-10
    quadratic Beziers, heights U[8,24] px, laid out in rows; EvenOdd, Over,
    opaque black on white."""
    U = Rng(seed, 5).uniform(n_layers, 4)
    h = 8.0 + 16.0 * U[:, 0]
    adv = 0.62 * h + 1.0
    ncont = 3 + np.minimum((U[:, 1] * 4).astype(np.int64), 3)
    # lay glyphs out left to right, wrapping rows at the canvas width
    if pitch is None:
        total = float(adv.sum())
        rows = max(1.0, np.ceil(total / (width - 24.0)))
        pitch = max(8.0, (height - 24.0) / rows)
    xs = np.zeros(n_layers)
    ys = np.zeros(n_layers)
    x, y = 4.0, 4.0
    for i in range(n_layers):
        if x + adv[i] > width - 4.0:
            x = 4.0
            y += pitch
        xs[i], ys[i] = x, y
        x += adv[i]
    C = Rng(seed, 6).uniform(n_layers, 6 * (4 + 10 * 3))
    kinds, points, path_layer = [], [], []
    for i in range(n_layers):
        base = 0
        for c in range(int(ncont[i])):
            cc = C[i, base:base + 4 + 30]
            base += 4 + 30
            n = 4 + min(int(cc[0] * 7), 6)
            w = 0.55 * h[i]
            cxc = xs[i] + w * (0.2 + 0.6 * cc[1])
            cyc = ys[i] + h[i] * (0.2 + 0.6 * cc[2])
            rad = 0.5 * h[i] * (0.15 + 0.35 * cc[3])
            ang = (np.arange(n) + 0.3 * cc[4:4 + n]) * (2.0 * np.pi / n)
            ax, ay = cxc + rad * np.cos(ang), cyc + 1.3 * rad * np.sin(ang)
            mid = ang + np.pi / n
            cr = rad * (0.7 + 0.8 * cc[14:14 + n])
            qx, qy = cxc + cr * np.cos(mid), cyc + 1.3 * cr * np.sin(mid)
            pts = np.empty((n, 6), np.float64)
            pts[:, 0], pts[:, 1] = ax, ay
            pts[:, 2], pts[:, 3] = qx, qy
            pts[:, 4], pts[:, 5] = np.roll(ax, -1), np.roll(ay, -1)
            k = np.full(n + 1, abi.CMD_QUAD, np.uint32)
            k[-1] = abi.CMD_CLOSE
            kinds.append(k)
            points.append(pts.astype(np.float32).reshape(-1))
            path_layer.append(i)
    color = np.tile(np.array([[0.0, 0.0, 0.0, 1.0]], np.float32), (n_layers, 1))
    return _assemble("glyphs", width, height, (1.0, 1.0, 1.0, 1.0), False, n_layers, kinds, points, path_layer,
                     None, np.full(n_layers, abi.FILL_EVENODD), np.zeros(n_layers), color, {"pitch": pitch})


def batch(seed: int = 4, n_scenes: int = 256, max_layers: int = 50_000) -> List[Scene]:
    """Batched workload: per scene, layer count log-U[10, max_layers], canvas
    side in {256, 512, 1024, 2048}, geometry from the mixed generator."""
    U = Rng(seed, 7).uniform(n_scenes, 2)
    out = []
    for s in range(n_scenes):
        n = int(np.exp(np.log(10.0) + U[s, 0] * (np.log(max_layers) - np.log(10.0))))
        side = (256, 512, 1024, 2048)[min(int(U[s, 1] * 4), 3)]
        geo, tr, fr, bm, color = _mixed_geometry(seed * 1000003 + s, n, side, side)
        out.append(_flat_scene(f"batch{s}", side, side, False, n, geo, tr, fr, bm, color))
    return out


def load(scene: Scene, comp, unchecked=True):
    """Creates the scene's layers (ids 0..n-1, order = id) in a Composition
    (cassia_gb300.Composition or the oracle's) and sets props/transforms."""
    for i in range(scene.n_layers):
        lid = comp.create_layer()
        assert lid == i, (lid, i)
    comp.insert_paths(scene)
    comp.set_layers_solid(np.arange(scene.n_layers, dtype=np.uint32), scene.fill_rule, scene.blend_mode,
                          scene.color)
    if scene.transforms is not None:
        comp.set_transforms(np.arange(scene.n_layers, dtype=np.uint32), scene.transforms, unchecked=unchecked)
    return comp
