"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer and byte results must be bit-exact: sorted pixel segments (canonical
full-u64 order and the reference's key order), NONE counts and RGBA8 pixels.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes
from cassia_gb300.types import BlendMode, FillRule, Path, Props, Style, solid

from . import test_oracle_kats as kats

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[False, True], ids=["u16", "wide"])
def gpu_comp(request, gpu_lib):
    from cassia_gb300 import Composition
    c = Composition(wide=request.param)
    yield c
    c.close()


# ---- the reference's render KATs, through the GPU ----------------------------------

KAT_NAMES = ["background_color_clear", "one_pixel", "two_pixels_same_layer", "one_pixel_translated",
             "one_pixel_rotated", "remove_and_resize", "remove_twice", "render_change_layers_only",
             "clear_emptied_tiles", "separate_layer_caches", "even_odd"]


def _make_kat(name):
    fn = getattr(kats, "test_" + name)

    def t(gpu_comp):
        fn(gpu_comp)

    t.__name__ = "test_gpu_kat_" + name
    return t


for _n in KAT_NAMES:
    globals()["test_gpu_kat_" + _n] = _make_kat(_n)


# ---- seeded scenes -------------------------------------------------------------------------

def _load_both(scene, wide=None):
    from cassia_gb300 import Composition
    wide = scene.wide if wide is None else wide
    g = Composition(wide=wide)
    o = oracle.Composition(wide=wide)
    scenes.load(scene, g)
    scenes.load(scene, o)
    return g, o


def _assert_same_image(a, b):
    if not np.array_equal(a, b):
        diff = np.argwhere(np.any(a != b, axis=-1))
        y, x = diff[0]
        raise AssertionError(f"{len(diff)} pixels differ; first at (x={x}, y={y}): gpu={a[y, x]} oracle={b[y, x]}")


def _render_both(scene, g, o, **kw):
    img_g = np.zeros((scene.height, scene.width, 4), np.uint8)
    img_o = np.zeros_like(img_g)
    g.render(img_g, scene.width, scene.background, **kw)
    o.render(img_o, scene.width, scene.background, threads=8, **kw)
    return img_g, img_o


SMALL_SCENES = {
    "circles": lambda: scenes.circles(seed=11, n_layers=300, size=256),
    "mixed": lambda: scenes.mixed(seed=12, n_layers=400, width=320, height=200),
    "glyphs": lambda: scenes.glyphs(seed=13, n_layers=600, width=480, height=270),
}


@pytest.mark.parametrize("name", list(SMALL_SCENES))
def test_pixel_segments_bit_exact(name):
    sc = SMALL_SCENES[name]()
    g, o = _load_both(sc)
    gs, gnone = g.pixel_segments(canonical=True)
    os_, onone = o.pixel_segments(threads=8)
    assert gnone == onone
    assert len(gs) == len(os_)
    assert np.array_equal(gs, os_)


@pytest.mark.parametrize("name", list(SMALL_SCENES))
def test_pixel_segments_key_order(name):
    # CGB_SORT_KEY: the reference's order (u64 >> 22), a permutation of the same multiset
    sc = SMALL_SCENES[name]()
    g, o = _load_both(sc)
    gs, _ = g.pixel_segments(canonical=False)
    os_, _ = o.pixel_segments(threads=8)
    keys = gs >> np.uint64(22)
    assert np.all(keys[1:] >= keys[:-1])
    assert np.array_equal(np.sort(gs), os_)


@pytest.mark.parametrize("name", list(SMALL_SCENES))
def test_render_bit_exact(name):
    sc = SMALL_SCENES[name]()
    g, o = _load_both(sc)
    a, b = _render_both(sc, g, o)
    _assert_same_image(a, b)


def test_render_wide_format_matches_u16():
    sc = SMALL_SCENES["mixed"]()
    g, o = _load_both(sc, wide=True)
    a, b = _render_both(sc, g, o)
    _assert_same_image(a, b)
    g2, _ = _load_both(sc, wide=False)
    c = np.zeros_like(a)
    g2.render(c, sc.width, sc.background)
    _assert_same_image(a, c)


def test_render_all_blend_modes_and_fill_rules():
    sc = scenes.mixed(seed=21, n_layers=600, width=256, height=160)
    sc.blend_mode[:] = np.arange(sc.n_layers) % 12
    sc.fill_rule[:] = (np.arange(sc.n_layers) // 12) % 2
    g, o = _load_both(sc)
    a, b = _render_both(sc, g, o)
    _assert_same_image(a, b)


def test_render_opaque_layers_cull_and_solid_tiles():
    # opaque Over layers exercise skip_fully_covered_layers and the Solid path
    sc = scenes.mixed(seed=22, n_layers=500, width=256, height=256)
    sc.blend_mode[:] = np.where(np.arange(sc.n_layers) % 3 == 0, 0, sc.blend_mode)
    sc.color[::2, 3] = 1.0
    sc.blend_mode[::2] = BlendMode.Over
    g, o = _load_both(sc)
    a, b = _render_both(sc, g, o)
    _assert_same_image(a, b)


@pytest.mark.parametrize("w,h", [(250, 131), (9, 9), (1, 1), (7, 300)])
def test_render_partial_tiles(w, h):
    sc = scenes.mixed(seed=23, n_layers=200, width=w, height=h)
    g, o = _load_both(sc)
    a, b = _render_both(sc, g, o)
    _assert_same_image(a, b)


def test_render_stride_and_crop():
    sc = scenes.mixed(seed=24, n_layers=300, width=200, height=120)
    g, o = _load_both(sc)
    stride = 232
    a = np.full((sc.height, stride, 4), 7, np.uint8)
    b = a.copy()
    g.render(a, sc.width, sc.background, width_stride=stride)
    o.render(b, sc.width, sc.background, width_stride=stride, threads=4)
    _assert_same_image(a, b)
    a[...] = 9
    b[...] = 9
    crop = (37, 150, 20, 90)
    g.render(a, sc.width, sc.background, width_stride=stride, crop=crop)
    o.render(b, sc.width, sc.background, width_stride=stride, crop=crop, threads=4)
    _assert_same_image(a, b)


def test_render_empty_and_offcanvas():
    from cassia_gb300 import Composition
    g, o = Composition(), oracle.Composition()
    for c in (g, o):
        # a layer entirely left of the canvas (its covers cancel per row) and one above it
        lid = c.create_layer()
        c.insert_in_layer(lid, kats.pixel_path(-20, 3))
        c.set_props(lid, solid((1.0, 0.0, 0.0, 0.5)))
        lid = c.create_layer()
        c.insert_in_layer(lid, kats.pixel_path(3, -40))
        c.set_props(lid, solid((0.0, 0.0, 1.0, 1.0)))
    a = np.zeros((20, 24, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, 24, (0.25, 0.5, 0.75, 1.0))
    o.render(b, 24, (0.25, 0.5, 0.75, 1.0))
    _assert_same_image(a, b)


def test_render_left_of_canvas_carry():
    # shapes that straddle the left edge: their left-of-canvas covers seed the row's carry
    from cassia_gb300 import Composition
    g, o = Composition(), oracle.Composition()
    for c in (g, o):
        for k, (x, fr) in enumerate([(-30, FillRule.NonZero), (-9, FillRule.EvenOdd), (-1, FillRule.NonZero)]):
            lid = c.create_layer()
            p = Path().line((x, 2 + k), (x + 40.3, 5 + k)).line((x + 40.3, 5 + k), (x + 12.0, 19.7 + k)).close()
            c.insert_in_layer(lid, p)
            c.set_props(lid, Props(fill_rule=fr, func=Style(fill=(0.2 * k, 0.5, 1.0 - 0.2 * k, 0.8))))
    a = np.zeros((32, 40, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, 40, (1.0, 1.0, 1.0, 1.0))
    o.render(b, 40, (1.0, 1.0, 1.0, 1.0))
    _assert_same_image(a, b)


def test_render_layer_cache_sequence():
    sc = scenes.mixed(seed=25, n_layers=150, width=160, height=96)
    g, o = _load_both(sc)
    cg, co = g.create_buffer_layer_cache(), o.create_buffer_layer_cache()
    a = np.zeros((sc.height, sc.width, 4), np.uint8)
    b = np.zeros_like(a)
    rng = np.random.default_rng(5)
    for frame in range(4):
        ids = rng.choice(sc.n_layers, size=10, replace=False).astype(np.uint32)
        t = sc.transforms[ids].copy()
        t[:, 4] += rng.uniform(-5, 5, size=len(ids)).astype(np.float32)
        for c in (g, o):
            c.set_transforms(ids, t)
        a[...] = 3
        b[...] = 3
        g.render(a, sc.width, sc.background, layer_cache=cg)
        o.render(b, sc.width, sc.background, layer_cache=co, threads=4)
        _assert_same_image(a, b)


def test_disable_and_gc_matches_oracle():
    sc = scenes.mixed(seed=26, n_layers=200, width=128, height=128)
    g, o = _load_both(sc)
    for c in (g, o):
        for lid in range(0, 200, 3):
            c.set_enabled(lid, False)
    a, b = _render_both(sc, g, o)
    _assert_same_image(a, b)
    assert g.lens() == o.lens()


def test_render_tile_layer_longer_than_scan_blocks():
    # one layer zigzags inside a single tile: its tile-layer group holds
    # thousands of segments, so whole blocks of the group scan hold no group
    # head and the group's cover sum crosses several blocks
    from cassia_gb300 import Composition
    g, o = Composition(), oracle.Composition()
    for c in (g, o):
        for k, (fr, x0) in enumerate([(FillRule.NonZero, 8.0), (FillRule.EvenOdd, 24.0)]):
            lid = c.create_layer()
            p = Path()
            pts = [(x0 + 0.2 + 0.0047 * i, 8.2 if i % 2 == 0 else 15.8) for i in range(1300)]
            for a, b in zip(pts, pts[1:] + pts[:1]):
                p.line(a, b)
            c.insert_in_layer(lid, p.close())
            c.set_props(lid, Props(fill_rule=fr, func=Style(fill=(0.9, 0.3 * k, 0.1, 0.7))))
        lid = c.create_layer()  # a plain shape across the same rows
        c.insert_in_layer(lid, Path().line((1.5, 3.0), (38.0, 12.5)).line((38.0, 12.5), (5.0, 22.0)).close())
        c.set_props(lid, solid((0.1, 0.2, 0.9, 0.6)))
    a = np.zeros((32, 40, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, 40, (1.0, 1.0, 1.0, 1.0))
    o.render(b, 40, (1.0, 1.0, 1.0, 1.0))
    stats_segments = g.stats()["segments"]
    assert stats_segments > 3 * 2048
    _assert_same_image(a, b)


def test_lines_across_rasterizer_blocks():
    """Lines longer than a rasterizer block's 2,048 pixel steps, with runs of
    culled lines (no steps in a render frame) before, between and after them,
    so that blocks start and end inside long lines and next to empty ones; the
    same layers rasterized whole by pixel_segments; and an incremental frame,
    whose sparse rasterizer walks mostly empty lines."""
    from cassia_gb300 import Composition
    W, H = 2600, 48
    g, o = Composition(), oracle.Composition()
    for c in (g, o):
        for k in range(40):
            lid = c.create_layer()
            if k % 4 == 3:  # a long thin triangle across the canvas
                y = 1.5 + k
                p = Path().line((-3.5, y), (W + 2.5, y + 2.7)).line((W + 2.5, y + 2.7), (W / 2, y + 6.1)).close()
                props = Props(fill_rule=FillRule(int(k % 8 == 3)), func=Style(fill=(0.2, 0.6, 0.9, 0.7)))
            else:  # above the canvas
                x = 10.0 * k
                p = Path().line((x, -300.0), (x + 900.0, -280.0)).line((x + 900.0, -280.0), (x, -250.0)).close()
                props = solid((1.0, 0.0, 0.0, 1.0))
            c.insert_in_layer(lid, p)
            c.set_props(lid, props)
    g.set_incremental(True)
    bg = (1.0, 1.0, 1.0, 1.0)
    a = np.zeros((H, W, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, W, bg)
    o.render(b, W, bg, threads=8)
    _assert_same_image(a, b)
    assert g.stats()["steps"] > 8 * 2048
    t = np.array([[0.999, -0.02, 0.02, 0.999, 1.25, -0.5]], np.float32)
    for c in (g, o):
        c.set_transforms(np.array([7], np.uint32), t)
    g.render(a, W, bg)
    o.render(b, W, bg, threads=8)
    _assert_same_image(a, b)
    assert g.stats()["incremental_form"] in (1, 2)
    gs, gnone = g.pixel_segments(canonical=True)
    os_, onone = o.pixel_segments(threads=8)
    assert gnone == onone
    assert np.array_equal(gs, os_)


def test_many_transforms_in_one_call():
    """20,000 layer transforms in one call (split over host threads) render as
    the same update made in calls of 1,000 layers and as the oracle; an
    invalid transform in the middle of a call leaves the layers before it
    moved and the rest as they were, as one call per layer would."""
    from cassia_gb300 import Composition
    from cassia_gb300.abi import CassiaError
    sc = scenes.mixed(seed=27, n_layers=20_000, width=256, height=192)
    g1, o = _load_both(sc)
    g2 = Composition(wide=sc.wide)
    scenes.load(sc, g2)
    ids = np.arange(sc.n_layers, dtype=np.uint32)
    t = sc.transforms.copy()
    t[:, 4] += 0.75
    t[:, 5] -= 0.5

    def chunked(c, tt, unchecked=True):
        for k in range(0, len(ids), 1000):
            c.set_transforms(ids[k:k + 1000], tt[k:k + 1000], unchecked=unchecked)

    g1.set_transforms(ids, t)
    chunked(g2, t)
    o.set_transforms(ids, t)
    a, b = _render_both(sc, g1, o)
    _assert_same_image(a, b)
    c2 = np.zeros_like(a)
    g2.render(c2, sc.width, sc.background)
    _assert_same_image(c2, a)
    t2 = t.copy()
    t2[:, 4] -= 2.0
    t2[15_000, 0] = 1.5  # scale above 1
    with pytest.raises(CassiaError):
        g1.set_transforms(ids, t2, unchecked=False)
    with pytest.raises(CassiaError):
        chunked(g2, t2, unchecked=False)
    g1.render(a, sc.width, sc.background)
    g2.render(c2, sc.width, sc.background)
    _assert_same_image(c2, a)


def test_render_many_small_tile_layer_groups():
    # 20,000 squares of 0.4-2 px, packed on a 256x256 canvas: a group of a
    # tile and a layer holds 2-8 segments, so many warps of the tile-layer
    # scan hold more groups than its shared-memory stage (they write their
    # groups directly) and others fewer; pixels and segments equal the oracle's.
    from cassia_gb300 import Composition
    rng = np.random.default_rng(913)
    n, size = 20000, 256
    g, o = Composition(), oracle.Composition()
    for c in (g, o):
        for _ in range(n):
            c.create_layer()
    x = rng.uniform(-1, size + 1, n).astype(np.float32)
    y = rng.uniform(-1, size + 1, n).astype(np.float32)
    s = rng.uniform(0.4, 2.0, n).astype(np.float32)
    for i in range(n):
        a, b, e = float(x[i]), float(y[i]), float(s[i])
        segs = [[a, b, a + e, b], [a + e, b, a + e, b + e], [a + e, b + e, a, b + e], [a, b + e, a, b]]
        for c in (g, o):
            c.insert_lines(i, segs)
    ids = np.arange(n, dtype=np.uint32)
    fr = rng.integers(0, 2, n).astype(np.uint32)
    bm = rng.integers(0, 12, n).astype(np.uint32)
    col = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    col[:, 3] = rng.uniform(0.2, 1, n)
    for c in (g, o):
        c.set_layers_solid(ids, fr, bm, col)
    a = np.zeros((size, size, 4), np.uint8)
    g.render(a, size, (1.0, 1.0, 1.0, 1.0))
    b = np.zeros_like(a)
    o.render(b, size, (1.0, 1.0, 1.0, 1.0), threads=8)
    assert np.array_equal(a, b)
    st = g.stats()
    assert st["painted_segments"] < 4 * st["tile_layers"]  # groups of a few segments
    gs, gn = g.pixel_segments()
    os_, on = o.pixel_segments(threads=8)
    assert gn == on and np.array_equal(gs, os_)
