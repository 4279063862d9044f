"""The segment sort skips its order passes only when that changes nothing.

Segments are sorted tile-major (tile row, tile column, layer order).  When
every scene's lines are in non-decreasing layer order, the rasterizer's
segments already come in that order within each tile, so the sort's stable
passes over the order digits would move no segment and the frame skips them
(cgb_stats.sort_passes_skipped); any line out of order makes the frame run
them.  Either way the pixels equal the oracle's: scenes loaded in layer
order, orders reversed, a layer given more lines after the others, a
disabled layer between, digit widths that skip an odd number of passes,
frames replayed from a frame graph, and a batch whose scenes differ.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes
from cassia_gb300.types import Path

pytestmark = pytest.mark.gpu


def _pair(sc):
    from cassia_gb300 import Composition
    g = Composition(wide=sc.wide)
    scenes.load(sc, g)
    o = oracle.Composition(wide=sc.wide)
    scenes.load(sc, o)
    return g, o


def _render(c, sc, **kw):
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    c.render(img, sc.width, sc.background, **kw)
    return img


def _check(g, o, sc, what):
    a = _render(g, sc)
    b = np.zeros_like(a)
    o.render(b, sc.width, sc.background, threads=8)
    if not np.array_equal(a, b):
        n = int(np.count_nonzero(np.any(a != b, axis=-1)))
        raise AssertionError(f"{what}: {n} pixels differ from the oracle")
    return g.stats()


def _square(x, y, s):
    p = Path()
    p.line((x, y), (x + s, y))
    p.line((x + s, y), (x + s, y + s))
    p.line((x + s, y + s), (x, y + s))
    p.line((x, y + s), (x, y))
    return p


def test_skip_in_layer_order_and_not_otherwise(gpu_lib):
    sc = scenes.mixed(seed=71, n_layers=3000, width=640, height=400)
    g, o = _pair(sc)
    st = _check(g, o, sc, "layer order")
    assert st["sort_passes_skipped"] > 0, st
    # reversed orders: the lines now run in decreasing order
    n = sc.n_layers
    for i in range(n):
        g.set_order(i, n - 1 - i)
        o.set_order(i, n - 1 - i)
    st = _check(g, o, sc, "reversed orders")
    assert st["sort_passes_skipped"] == 0, st
    # back in order, then layer 0 (the lowest order) gets lines after all the others
    for i in range(n):
        g.set_order(i, i)
        o.set_order(i, i)
    assert _check(g, o, sc, "restored")["sort_passes_skipped"] > 0
    for c in (g, o):
        c.insert_in_layer(0, _square(100.5, 90.25, 180.0))
    st = _check(g, o, sc, "late lines of a low order")
    assert st["sort_passes_skipped"] == 0, st


def test_disabled_layer_and_graph_replay(gpu_lib):
    sc = scenes.mixed(seed=72, n_layers=2000, width=520, height=300)
    g, o = _pair(sc)
    g.set_graph_mode(True)
    for c in (g, o):
        c.set_enabled(700, False)
    for k in range(3):  # staged, captured, replayed
        st = _check(g, o, sc, f"frame {k}")
        assert st["sort_passes_skipped"] > 0, st
    assert st["graph_replayed"] == 1
    # an order change under the same frame graph: the replay runs the passes
    for c in (g, o):
        c.set_order(5, 1999)
        c.set_order(1999, 5)
    for k in range(2):
        st = _check(g, o, sc, f"swapped orders {k}")
        assert st["sort_passes_skipped"] == 0, st


@pytest.mark.parametrize("bits", [4, 5, 8])
def test_digit_widths(gpu_lib, bits):
    # 2,000 layers: an 11-bit order field, 3 passes of 4 bits (odd: the last
    # skipped pass copies the keys across), 3 of 5 bits, 2 of 8 bits
    sc = scenes.mixed(seed=73, n_layers=2000, width=520, height=300)
    g, o = _pair(sc)
    g.set_tuning(radix_bits=bits)
    st = _check(g, o, sc, f"{bits}-bit digits")
    assert st["sort_passes_skipped"] == -(-11 // bits), st


def test_batch_with_one_scene_out_of_order(gpu_lib):
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    sset = [scenes.mixed(seed=80 + k, n_layers=600 + 300 * k, width=256 + 64 * k, height=200) for k in range(3)]
    comps, refs = [], []
    for k, sc in enumerate(sset):
        g, o = _pair(sc)
        if k == 1:
            for c in (g, o):
                c.set_order(3, sc.n_layers - 1)
                c.set_order(sc.n_layers - 1, 3)
        comps.append(g)
        b = np.zeros((sc.height, sc.width, 4), np.uint8)
        o.render(b, sc.width, sc.background, threads=8)
        refs.append(b)
    outs = [np.zeros((sc.height, sc.width, 4), np.uint8) for sc in sset]
    ctx = Composition()
    render_batch(ctx, comps, outs, [sc.width for sc in sset], [sc.background for sc in sset])
    assert ctx.stats()["sort_passes_skipped"] == 0
    for k in range(3):
        assert np.array_equal(outs[k], refs[k]), f"scene {k}"
    comps[1].set_order(3, 3)
    comps[1].set_order(sset[1].n_layers - 1, sset[1].n_layers - 1)
    render_batch(ctx, comps, outs, [sc.width for sc in sset], [sc.background for sc in sset])
    assert ctx.stats()["sort_passes_skipped"] > 0
