"""Gradient fills in the GPU painter (style.rs:29-175, painter/mod.rs:335-345).

Linear and radial gradients with evenly spread and explicit stops, stops at
equal positions, t outside [0, 1], every blend mode and both fill rules, a
gradient over a fully covered opaque layer (the Solid fold must give way to
the colour buffer), and a batch mixing gradient and solid scenes: RGBA8 must
equal the oracle's, bit for bit.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes
from cassia_gb300.types import BlendMode, FillRule, Gradient, GradientType, Path, Props, Style, solid

pytestmark = pytest.mark.gpu


def _rect(x0, y0, x1, y1):
    return Path().line((x0, y0), (x1, y0)).line((x1, y0), (x1, y1)).line((x1, y1), (x0, y1)).close()


def _tri(a, b, c):
    return Path().line(a, b).line(b, c).line(c, a).close()


def _gradients():
    return [
        Gradient(start=(0.0, 0.0), end=(60.0, 30.0), stops=[((1.0, 0.0, 0.0, 1.0), None), ((0.0, 0.0, 1.0, 0.5), None)]),
        Gradient(start=(50.0, 5.0), end=(5.0, 40.0),
                 stops=[((0.1, 0.9, 0.2, 0.9), 0.0), ((0.9, 0.9, 0.1, 0.4), 0.3), ((0.2, 0.1, 0.8, 1.0), 0.3),
                        ((0.5, 0.5, 0.5, 0.7), 1.0)]),
        Gradient(start=(30.0, 20.0), end=(55.0, 45.0), type=GradientType.Radial,
                 stops=[((0.0, 0.0, 0.0, 1.0), None), ((1.0, 1.0, 1.0, 1.0), None), ((0.3, 0.6, 0.9, 0.6), None)]),
        Gradient(start=(10.0, 10.0), end=(12.0, 11.0), type=GradientType.Radial,  # t far above 1
                 stops=[((0.8, 0.2, 0.4, 1.0), 0.2), ((0.1, 0.7, 0.3, 0.8), 0.6)]),
    ]


def _compose(c, k_shift=0):
    shapes = [_rect(2.5, 3.0, 57.0, 41.0), _tri((5.0, 44.0), (60.0, 2.0), (33.0, 47.5)),
              _rect(17.0, 9.0, 40.0, 30.0), _tri((1.0, 1.0), (63.0, 20.0), (10.0, 46.0))]
    for k, (path, g) in enumerate(zip(shapes, _gradients())):
        lid = c.create_layer()
        c.insert_in_layer(lid, path)
        mode = BlendMode((k * 5 + k_shift) % 12)
        fr = FillRule.EvenOdd if k % 2 else FillRule.NonZero
        c.set_props(lid, Props(fill_rule=fr, func=Style(fill=g, blend_mode=mode)))


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


def test_gradients_match_oracle():
    for shift in range(0, 12, 3):
        a, b = _render_both(lambda c: _compose(c, shift), 64, 48)
        assert np.array_equal(a, b), f"blend shift {shift}"


def test_gradient_over_opaque_solid_uses_the_color_buffer():
    def setup(c):
        lid = c.create_layer()
        c.insert_in_layer(lid, _rect(-4.0, -4.0, 70.0, 60.0))  # opaque, covers every tile
        c.set_props(lid, solid((0.2, 0.3, 0.4, 1.0)))
        lid = c.create_layer()
        c.insert_in_layer(lid, _rect(-2.0, -2.0, 68.0, 58.0))  # full gradient above it
        c.set_props(lid, Props(func=Style(fill=_gradients()[0], blend_mode=BlendMode.Multiply)))
        lid = c.create_layer()
        c.insert_in_layer(lid, _rect(8.0, 8.0, 30.0, 30.0))  # a solid on top
        c.set_props(lid, solid((0.9, 0.1, 0.1, 0.5)))
    a, b = _render_both(setup, 64, 48)
    assert np.array_equal(a, b)


def test_gradients_in_a_mixed_scene_and_batch():
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    sc = scenes.mixed(seed=51, n_layers=700, width=300, height=200)
    gs = _gradients()

    def setup(c):
        scenes.load(sc, c)
        for k in range(0, sc.n_layers, 5):  # every fifth layer gets a gradient
            g = gs[k % len(gs)]
            g2 = Gradient(start=(g.start[0] * 4, g.start[1] * 3), end=(g.end[0] * 4, g.end[1] * 3), stops=g.stops,
                          type=g.type)
            c.set_props(k, Props(fill_rule=FillRule(int(sc.fill_rule[k])),
                                 func=Style(fill=g2, blend_mode=BlendMode(int(sc.blend_mode[k])))))
    a, b = _render_both(setup, sc.width, sc.height, sc.background)
    assert np.array_equal(a, b)
    # batched with a solid-only scene
    g, plain = Composition(), Composition()
    setup(g)
    other = scenes.mixed(seed=52, n_layers=300, width=120, height=90)
    scenes.load(other, plain)
    outs = [np.zeros((sc.height, sc.width, 4), np.uint8), np.zeros((other.height, other.width, 4), np.uint8)]
    render_batch(Composition(), [g, plain], outs, [sc.width, other.width], [sc.background, other.background])
    assert np.array_equal(outs[0], b)
    alone = np.zeros_like(outs[1])
    plain.render(alone, other.width, other.background)
    assert np.array_equal(outs[1], alone)
