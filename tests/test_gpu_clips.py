"""Clip layers in the GPU painter (Func::Clip, Style::is_clipped;
layer_workbench.rs:224-308, painter/mod.rs:260-317, 402-416).

Clips with partial and full coverage, unused clips, clipped layers outside
any clip, a clip replaced while the previous one is still in range, clips
under opaque layers and with gradient fills, and a seeded scene with many
clips: RGBA8 must equal the oracle's, bit for bit.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes
from cassia_gb300.types import BlendMode, FillRule, Gradient, Path, Props, Style, solid

pytestmark = pytest.mark.gpu


def _rect(x0, y0, x1, y1):
    return Path().line((x0, y0), (x1, y0)).line((x1, y0), (x1, y1)).line((x1, y1), (x0, y1)).close()


def _tri(a, b, c):
    return Path().line(a, b).line(b, c).line(c, a).close()


def _layer(c, path, props):
    lid = c.create_layer()
    c.insert_in_layer(lid, path)
    c.set_props(lid, props)
    return lid


def _clipped(color, mode=BlendMode.Over, fr=FillRule.NonZero):
    return Props(fill_rule=fr, func=Style(fill=color, blend_mode=mode, is_clipped=True))


def _render_both(setup, w, h, bg=(1.0, 1.0, 1.0, 1.0)):
    from cassia_gb300 import Composition
    g, o = Composition(), oracle.Composition()
    setup(g)
    setup(o)
    a = np.zeros((h, w, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, w, bg)
    o.render(b, w, bg, threads=4)
    return a, b


def _assert_same(a, b):
    if not np.array_equal(a, b):
        d = np.argwhere(np.any(a != b, axis=-1))
        y, x = d[0]
        raise AssertionError(f"{len(d)} pixels differ; first at ({x}, {y}): gpu={a[y, x]} oracle={b[y, x]}")


def test_clip_layers_partial_full_unused_and_outside():
    def setup(c):
        _layer(c, _rect(0.0, 0.0, 64.0, 48.0), solid((0.9, 0.9, 0.9, 1.0)))           # opaque background layer
        _layer(c, _tri((4.0, 4.0), (60.0, 10.0), (20.0, 44.0)), Props(func=2))        # clips the next 2
        _layer(c, _rect(2.0, 2.0, 40.0, 40.0), _clipped((1.0, 0.0, 0.0, 0.8)))
        _layer(c, _rect(20.0, 6.0, 62.0, 30.0), _clipped((0.0, 0.0, 1.0, 0.6), BlendMode.Multiply))
        _layer(c, _rect(10.0, 30.0, 50.0, 46.0), _clipped((0.0, 1.0, 0.0, 1.0)))       # outside the clip's range
        _layer(c, _rect(-8.0, -8.0, 80.0, 70.0), Props(func=1))                       # full in inner tiles
        _layer(c, _tri((1.0, 47.0), (63.0, 40.0), (30.0, 1.0)), _clipped((0.5, 0.2, 0.7, 0.7), fr=FillRule.EvenOdd))
        _layer(c, _rect(30.0, 30.0, 34.0, 34.0), Props(func=3))                       # clips nothing clipped: unused
        _layer(c, _rect(5.0, 20.0, 25.0, 28.0), solid((0.2, 0.8, 0.2, 0.5)))
    a, b = _render_both(setup, 64, 48)
    _assert_same(a, b)


def test_clip_replaced_while_in_range_and_with_gradients():
    def setup(c):
        _layer(c, _tri((0.0, 0.0), (64.0, 8.0), (8.0, 48.0)), Props(func=4))
        _layer(c, _rect(4.0, 4.0, 60.0, 44.0), _clipped((0.8, 0.3, 0.1, 0.9)))
        _layer(c, _rect(30.0, 0.0, 64.0, 48.0), Props(fill_rule=FillRule.EvenOdd, func=3))  # a second clip in range
        g = Gradient(start=(0.0, 0.0), end=(64.0, 48.0), stops=[((0.0, 0.5, 1.0, 1.0), None), ((1.0, 0.5, 0.0, 0.5), None)])
        _layer(c, _rect(0.0, 10.0, 64.0, 40.0), Props(func=Style(fill=g, blend_mode=BlendMode.Screen, is_clipped=True)))
        _layer(c, _rect(10.0, 0.0, 50.0, 48.0), _clipped((0.1, 0.9, 0.4, 0.7), BlendMode.Overlay))
        _layer(c, _rect(12.0, 12.0, 52.0, 36.0), solid((0.0, 0.0, 0.0, 0.3)))
    a, b = _render_both(setup, 64, 48)
    _assert_same(a, b)


def test_seeded_scene_with_many_clips():
    sc = scenes.mixed(seed=61, n_layers=900, width=320, height=200)
    rng = np.random.default_rng(61)
    kinds = rng.integers(0, 10, size=sc.n_layers)

    def setup(c):
        scenes.load(sc, c)
        for k in range(sc.n_layers):
            fr = FillRule(int(sc.fill_rule[k]))
            if kinds[k] == 0:
                c.set_props(k, Props(fill_rule=fr, func=int(rng_n[k])))
            elif kinds[k] <= 3:
                col = tuple(float(v) for v in sc.color[k])
                c.set_props(k, Props(fill_rule=fr, func=Style(fill=col, blend_mode=BlendMode(int(sc.blend_mode[k])),
                                                              is_clipped=True)))
    rng_n = rng.integers(1, 12, size=sc.n_layers)
    a, b = _render_both(setup, sc.width, sc.height, sc.background)
    _assert_same(a, b)
