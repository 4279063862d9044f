"""GPU parity of the flattener's rational and perspective branches.

mold flattens rational quadratic and cubic Beziers with weighted lerps
(mold/src/path/segments.rs:169-210), and `insert_in_layer_transformed` takes a
3x3 transform that is divided by t22 and, when t6 or t7 is non-zero, turns
lines into projected lines and quads/cubics into rational curves
(mold/src/path/transform.rs:56-94).  These tests insert such paths through the
C ABI, flatten them on the GPU, and compare the sorted pixel segments and the
RGBA8 frame with the oracle bit for bit.
"""
import math

import numpy as np
import pytest

import oracle
from cassia_gb300.types import BlendMode, FillRule, Path, solid

pytestmark = pytest.mark.gpu


def _circle(x, y, r):
    """The reference demo's circle: four rational quads with weight sqrt(2)/2
    on the corner control points (demo/src/circles.rs:67-90)."""
    w = math.sqrt(2.0) / 2.0
    p = Path()
    p.rat_quad(((x + r, y), 1.0), ((x + r, y - r), w), ((x, y - r), 1.0))
    p.rat_quad(((x, y - r), 1.0), ((x - r, y - r), w), ((x - r, y), 1.0))
    p.rat_quad(((x - r, y), 1.0), ((x - r, y + r), w), ((x, y + r), 1.0))
    p.rat_quad(((x, y + r), 1.0), ((x + r, y + r), w), ((x + r, y), 1.0))
    return p


def _rat_cubic_blob(rng, cx, cy, size):
    """A closed path of 3-6 rational cubics with weights in [0.25, 4]."""
    n = int(rng.integers(3, 7))
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    rad = size * rng.uniform(0.4, 1.0, n)
    pts = [(cx + rad[i] * np.cos(ang[i]), cy + rad[i] * np.sin(ang[i])) for i in range(n)]
    p = Path()
    for i in range(n):
        a, b = pts[i], pts[(i + 1) % n]
        c1 = (a[0] + rng.uniform(-size, size), a[1] + rng.uniform(-size, size))
        c2 = (b[0] + rng.uniform(-size, size), b[1] + rng.uniform(-size, size))
        w = rng.uniform(0.25, 4.0, 2)
        p.rat_cubic((a, 1.0), (c1, float(w[0])), (c2, float(w[1])), (b, 1.0))
    return p.close()


def _poly_curves(rng, cx, cy, size):
    """A closed path mixing lines, quads and cubics (all become rational
    under a perspective transform)."""
    n = int(rng.integers(3, 7))
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    pts = [(cx + size * np.cos(a), cy + size * np.sin(a)) for a in ang]
    p = Path()
    for i in range(n):
        a, b = pts[i], pts[(i + 1) % n]
        k = i % 3
        if k == 0:
            p.line(a, b)
        elif k == 1:
            p.quad(a, (0.5 * (a[0] + b[0]) + rng.uniform(-size, size), 0.5 * (a[1] + b[1]) + rng.uniform(-size, size)), b)
        else:
            p.cubic(a, (a[0] + rng.uniform(-size, size), a[1] + rng.uniform(-size, size)),
                    (b[0] + rng.uniform(-size, size), b[1] + rng.uniform(-size, size)), b)
    return p.close()


def _perspective(rng, cx, cy, strength):
    """A 3x3 about (cx, cy): rotation, scale, translation back, t6/t7 of the
    given strength and t22 in [0.8, 1.25]."""
    th = rng.uniform(0, 2 * np.pi)
    s = rng.uniform(0.6, 1.6)
    t22 = float(np.exp(rng.uniform(np.log(0.8), np.log(1.25))))
    t6, t7 = rng.uniform(-strength, strength, 2)
    a, b = s * np.cos(th), -s * np.sin(th)
    c, d = s * np.sin(th), s * np.cos(th)
    tx = cx - (a * cx + b * cy)
    ty = cy - (c * cx + d * cy)
    # row-major [t00 t01 t02; t10 t11 t12; t20 t21 t22]
    return [a * t22, b * t22, tx * t22, c * t22, d * t22, ty * t22, float(t6), float(t7), t22]


def _build(comp, items):
    for path, t9, props in items:
        lid = comp.create_layer()
        comp.insert_in_layer(lid, path, t9)
        comp.set_props(lid, props)


def _compare(items, width, height, background=(1.0, 1.0, 1.0, 1.0)):
    from cassia_gb300 import Composition
    g = Composition()
    o = oracle.Composition()
    _build(g, items)
    _build(o, items)
    gs, gnone = g.pixel_segments(canonical=True)
    os_, onone = o.pixel_segments(threads=8)
    assert len(gs) > 0
    assert gnone == onone
    assert np.array_equal(gs, os_), f"{int(np.sum(gs != os_)) if len(gs) == len(os_) else 'count'} segments differ"
    a = np.zeros((height, width, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, width, background)
    o.render(b, width, background, threads=8)
    if not np.array_equal(a, b):
        diff = np.argwhere(np.any(a != b, axis=-1))
        y, x = diff[0]
        raise AssertionError(f"{len(diff)} pixels differ; first at (x={x}, y={y}): gpu={a[y, x]} oracle={b[y, x]}")
    g.close()
    return len(gs)


def test_demo_circles_of_rational_quads():
    rng = np.random.default_rng(101)
    items = []
    for _ in range(300):
        x, y = rng.uniform(0, 512, 2)
        r = rng.uniform(10, 50)
        color = (*rng.uniform(0, 1, 3), 0.5)  # the demo's alpha
        items.append((_circle(float(x), float(y), float(r)), None, solid(color)))
    assert _compare(items, 512, 512) > 10_000


def test_rational_cubics_both_fill_rules_and_modes():
    rng = np.random.default_rng(102)
    items = []
    for i in range(240):
        cx, cy = rng.uniform(0, 400, 2)
        path = _rat_cubic_blob(rng, float(cx), float(cy), float(rng.uniform(6, 60)))
        props = solid((*rng.uniform(0, 1, 3), rng.uniform(0.2, 1)), FillRule(i % 2), BlendMode(i % 12))
        items.append((path, None, props))
    _compare(items, 400, 320)


def test_affine_with_t22_not_one():
    """t22 != 1 without perspective: the transform is divided by t22 and the
    affine branch flattens in transformed space."""
    rng = np.random.default_rng(103)
    items = []
    for i in range(200):
        cx, cy = rng.uniform(0, 384, 2)
        t9 = _perspective(rng, float(cx), float(cy), 0.0)
        t9[6] = t9[7] = 0.0
        path = _poly_curves(rng, float(cx), float(cy), float(rng.uniform(5, 40)))
        items.append((path, t9, solid((*rng.uniform(0, 1, 3), rng.uniform(0.3, 1)), FillRule(i % 2))))
    _compare(items, 384, 384)


def test_perspective_lines_quads_cubics():
    """t6/t7 != 0: lines are projected point by point, quads and cubics become
    rational quads and cubics, rational curves stay rational."""
    rng = np.random.default_rng(104)
    items = []
    for i in range(200):
        cx, cy = rng.uniform(0, 384, 2)
        t9 = _perspective(rng, float(cx), float(cy), 4e-4)
        if i % 4 == 3:
            path = _rat_cubic_blob(rng, float(cx), float(cy), float(rng.uniform(5, 40)))
        elif i % 4 == 2:
            path = _circle(float(cx), float(cy), float(rng.uniform(5, 40)))
        else:
            path = _poly_curves(rng, float(cx), float(cy), float(rng.uniform(5, 40)))
        items.append((path, t9, solid((*rng.uniform(0, 1, 3), rng.uniform(0.3, 1)), FillRule(i % 2),
                                      BlendMode(i % 12))))
    _compare(items, 384, 384)


def test_seeded_scene_mixing_rational_and_perspective():
    """A scene of every branch at once: plain, rational and perspective
    layers interleaved, some layers holding several paths."""
    from cassia_gb300 import Composition
    rng = np.random.default_rng(105)
    W, H = 640, 400
    layers = []
    for i in range(400):
        paths = []
        for _ in range(int(rng.integers(1, 4))):
            cx, cy = float(rng.uniform(0, W)), float(rng.uniform(0, H))
            size = float(np.exp(rng.uniform(np.log(3), np.log(80))))
            kind = int(rng.integers(0, 4))
            path = (_circle(cx, cy, size) if kind == 0 else _rat_cubic_blob(rng, cx, cy, size) if kind == 1
                    else _poly_curves(rng, cx, cy, size))
            t9 = None
            mode = int(rng.integers(0, 3))
            if mode == 1:
                t9 = _perspective(rng, cx, cy, 0.0)
                t9[6] = t9[7] = 0.0
            elif mode == 2:
                t9 = _perspective(rng, cx, cy, 1e-3)
            paths.append((path, t9))
        props = solid((*rng.uniform(0, 1, 3), rng.uniform(0.2, 1)), FillRule(int(rng.integers(0, 2))),
                      BlendMode(int(rng.integers(0, 12))))
        layers.append((paths, props))

    def build(comp):
        for paths, props in layers:
            lid = comp.create_layer()
            for path, t9 in paths:
                comp.insert_in_layer(lid, path, t9)
            comp.set_props(lid, props)

    g = Composition()
    o = oracle.Composition()
    build(g)
    build(o)
    gs, gnone = g.pixel_segments(canonical=True)
    os_, onone = o.pixel_segments(threads=8)
    assert gnone == onone and np.array_equal(gs, os_)
    a = np.zeros((H, W, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, W, (0.9, 0.95, 1.0, 1.0))
    o.render(b, W, (0.9, 0.95, 1.0, 1.0), threads=8)
    assert np.array_equal(a, b), f"{int(np.sum(np.any(a != b, axis=-1)))} pixels differ"
    g.close()
