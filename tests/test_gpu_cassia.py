"""The cassia-format consumer (cassia_render, cassia/src/Cassia.h:25-41).

Segments from the oracle's pixel_segments (the reference's CompactSegment
stream), shuffled and with NONE slots mixed in, painted with stylings built
from the same Solid props as the demo does (demo/src/circles.rs:117-131),
must give the oracle's own render of the composition, bit for bit.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes

pytestmark = pytest.mark.gpu

NONE = np.uint64(1) << np.uint64(63)


def _stylings(sc):
    return [(tuple(float(v) for v in sc.color[k]), int(sc.fill_rule[k]), int(sc.blend_mode[k]))
            for k in range(sc.n_layers)]


@pytest.mark.parametrize("name", ["circles", "mixed"])
def test_cassia_render_matches_oracle_render(name):
    from cassia_gb300 import Composition
    sc = (scenes.circles(seed=71, n_layers=400, size=256) if name == "circles"
          else scenes.mixed(seed=72, n_layers=1500, width=400, height=300))
    o = oracle.Composition(wide=sc.wide)
    scenes.load(sc, o)
    segs, _ = o.pixel_segments(threads=4)
    want = np.zeros((sc.height, sc.width, 4), np.uint8)
    o.render(want, sc.width, sc.background, threads=4)
    rng = np.random.default_rng(7)
    mixed = np.concatenate([segs, np.full(len(segs) // 10, NONE, np.uint64)])
    rng.shuffle(mixed)
    ctx = Composition(wide=sc.wide)
    got = np.zeros_like(want)
    ctx.cassia_render(mixed, _stylings(sc), got, sc.width, sc.background)
    assert np.array_equal(got, want)
    # the handle still renders its own layers afterwards
    scenes.load(sc, ctx)
    again = np.zeros_like(want)
    ctx.render(again, sc.width, sc.background)
    assert np.array_equal(again, want)


def test_cassia_render_drops_orders_without_styling(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.circles(seed=73, n_layers=60, size=128)
    o = oracle.Composition()
    scenes.load(sc, o)
    segs, _ = o.pixel_segments(threads=2)
    # keep the stylings of the first 30 orders: the others' segments are dropped,
    # as removing those layers from the composition would
    ctx = Composition()
    got = np.zeros((sc.height, sc.width, 4), np.uint8)
    ctx.cassia_render(segs, _stylings(sc)[:30], got, sc.width, sc.background)
    o2 = oracle.Composition()
    scenes.load(sc, o2)
    for k in range(30, 60):
        o2.set_enabled(k, False)
    want = np.zeros_like(got)
    o2.render(want, sc.width, sc.background, threads=2)
    assert np.array_equal(got, want)
