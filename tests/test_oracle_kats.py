"""Pins the CPU oracle to the reference's own known-answer tests.

Each test restates one test of the reference (cited file:line) with the
reference's expected values; tile sizes are read as the current 8x8
(surpass/src/lib.rs:27-33) where a test was written for the removed TILE_SIZE.
"""
import math

import numpy as np
import pytest

import oracle
from cassia_gb300.types import BlendMode, FillRule, Gradient, GradientType, Path, Props, Style, solid

F32_EPS = np.float32(np.finfo(np.float32).eps)


def approx(a, b):
    assert abs(np.float32(a) - np.float32(b)) <= F32_EPS, (a, b)


# ---- surpass/src/segment.rs:304-538 -------------------------------------------

START_X, START_Y = 2.0, 3.0

OCTANT_CASES = [
    # (dx, dy, start, slope, octant, (coord used for the y check), expected)
    (3.0, 2.0, START_X, 2.0 / 3.0, 0),
    (2.0, 3.0, START_Y, 2.0 / 3.0, 1),
    (-2.0, 3.0, START_Y, -2.0 / 3.0, 2),
    (-3.0, 2.0, START_X - 3.0, -2.0 / 3.0, 3),
    (-3.0, -2.0, START_X - 3.0, 2.0 / 3.0, 4),
    (-2.0, -3.0, START_Y - 3.0, 2.0 / 3.0, 5),
    (2.0, -3.0, START_Y - 3.0, -2.0 / 3.0, 6),
    (3.0, -2.0, START_X, -2.0 / 3.0, 7),
]


@pytest.mark.parametrize("dx,dy,start,slope,octant", OCTANT_CASES)
def test_line_octants(dx, dy, start, slope, octant):
    # line_octant_1..8 (surpass/src/segment.rs:322-512)
    l = oracle.build_lines([[START_X, START_Y, START_X + dx, START_Y + dy]])
    assert l["starts"][0] == int(start)
    assert l["lengths"][0] == 3
    approx(l["slopes"][0], slope)
    approx(l["slopes_recip"][0], 1.0 / slope)
    assert l["octants"][0] == octant
    s, sr = np.float32(l["slopes"][0]), np.float32(l["slopes_recip"][0])
    b, br = np.float32(l["py_slope_pxs"][0]), np.float32(l["px_slope_recip_pys"][0])
    x_major = abs(dx) > abs(dy)
    if x_major:
        sx = 1.0 if dx > 0 else -1.0
        sy = 1.0 if dy > 0 else -1.0
        y = s * np.float32(START_X + sx * 1.5) + b
        approx(y, START_Y + sy * 1.0)
        x = sr * np.float32(START_Y + sy * 1.0) + br
        approx(x, START_X + sx * 1.5)
    else:
        sx = 1.0 if dx > 0 else -1.0
        sy = 1.0 if dy > 0 else -1.0
        x = s * np.float32(START_Y + sy * 1.5) + b
        approx(x, START_X + sx * 1.0)
        y = sr * np.float32(START_X + sx * 1.0) + br
        approx(y, START_Y + sy * 1.5)


def test_octant_borders():
    # surpass/src/segment.rs:514-529
    segs = [[0, 0, x, y] for x in (-10.0, 0.0, 10.0) for y in (-10.0, 0.0, 10.0) if x != 0.0 and y != 0.0]
    l = oracle.build_lines(segs)
    assert all(v == 10 for v in l["lengths"])


def test_empty_segment():
    # surpass/src/segment.rs:531-538
    l = oracle.build_lines([[2.0, 2.0, 2.0, 2.0]])
    assert list(l["lengths"]) == [0]


# ---- surpass/src/painter/style.rs:469-642 ------------------------------------------

@pytest.mark.parametrize("mode", list(BlendMode))
def test_blend_mode_scalar_equals_vector(mode):
    # test_blend_mode (style.rs:469-490): blend_fn == blend_function! on a 9x9 grid
    vals = [0.0, 0.125, 0.25, 0.375, 0.5, 0.625, 0.75, 0.875, 1.0]
    for d in vals:
        for s in vals:
            vec = oracle.blend_vector(mode, [d, d, d], [s, s, s])
            # blend() with alpha 1 and dst alpha 0 isolates f(dst, src): c = fma(dst, 0, f*1)
            sc = oracle.blend_scalar(mode, [d, d, d, 0.0], [s, s, s, 1.0])
            for c in range(3):
                assert np.float32(vec[c]) == np.float32(sc[c]), (mode, d, s, vec, sc)


def _color_eq(c):
    assert c[0] == c[1] == c[2] == c[3]
    return c[0]


def test_linear_gradient():
    # style.rs:492-530
    g = Gradient(start=(0.0, 7.0), end=(7.0, 0.0),
                 stops=[((0.25,) * 4, None), ((0.75,) * 4, None), ((0.25,) * 4, None), ((0.75,) * 4, None),
                        ((0.25,) * 4, None)])
    props = Props(func=Style(fill=g))
    col = oracle.gradient_color_at(props, 0.0, 0.0)
    assert col[0] == (0.25,) * 4
    assert _color_eq(col[1]) < _color_eq(col[2])
    assert _color_eq(col[2]) < _color_eq(col[3])
    assert _color_eq(col[4]) > _color_eq(col[5])
    assert _color_eq(col[5]) > _color_eq(col[6])
    assert col[7] == (0.25,) * 4
    col = oracle.gradient_color_at(props, 3.0, 0.0)
    assert _color_eq(col[0]) < 0.75
    assert _color_eq(col[1]) > _color_eq(col[2])
    assert _color_eq(col[2]) > _color_eq(col[3])
    assert col[3] == (0.25,) * 4
    assert _color_eq(col[3]) < _color_eq(col[4])
    assert _color_eq(col[4]) < _color_eq(col[5])
    assert _color_eq(col[5]) < _color_eq(col[6])
    assert _color_eq(col[7]) < 0.75
    col = oracle.gradient_color_at(props, 7.0, 0.0)
    assert col[0] == (0.25,) * 4
    assert _color_eq(col[1]) < _color_eq(col[2])
    assert _color_eq(col[2]) < _color_eq(col[3])
    assert _color_eq(col[4]) > _color_eq(col[5])
    assert _color_eq(col[5]) > _color_eq(col[6])
    assert col[7] == (0.25,) * 4


def test_radial_gradient():
    # style.rs:532-582
    r = 7.0 * (1.0 / math.sqrt(2.0))
    r = float(np.float32(7.0) * (np.float32(1.0) / np.float32(math.sqrt(2.0))))
    g = Gradient(start=(0.0, 0.0), end=(r, r), stops=[((0.25,) * 4, None), ((0.75,) * 4, None)],
                 type=GradientType.Radial)
    props = Props(func=Style(fill=g))
    col = oracle.gradient_color_at(props, 0.0, 0.0)
    assert col[0] == (0.25,) * 4
    for k in range(1, 6):
        assert _color_eq(col[k]) < _color_eq(col[k + 1])
    assert col[7] == (0.75,) * 4
    col = oracle.gradient_color_at(props, 3.0, 0.0)
    for k in range(0, 6):
        assert _color_eq(col[k]) < _color_eq(col[k + 1])
    assert col[7] == (0.75,) * 4
    col = oracle.gradient_color_at(props, 4.0, 0.0)
    for k in range(0, 5):
        assert _color_eq(col[k]) < _color_eq(col[k + 1])
    assert col[6] == (0.75,) * 4 and col[7] == (0.75,) * 4
    col = oracle.gradient_color_at(props, 7.0, 0.0)
    assert all(c == (0.75,) * 4 for c in col)


# ---- mold/src/path/mod.rs:181-403 ------------------------------------------------------

def segs_list(a):
    return [tuple(float(v) for v in row) for row in a]


def test_close_open_path():
    p = Path().line((0, 0), (1, 1)).line((1, 1), (2, 0)).close()
    assert segs_list(oracle.flatten(p)) == [(0, 0, 1, 1), (1, 1, 2, 0), (2, 0, 0, 0)]


def test_close_closed_path():
    p = Path().line((0, 0), (1, 1)).line((1, 1), (2, 0)).line((2, 0), (0, 0)).close()
    assert segs_list(oracle.flatten(p)) == [(0, 0, 1, 1), (1, 1, 2, 0), (2, 0, 0, 0)]


def test_scale_translate():
    # scale_translate_quad + scale_translate (mold/src/path/mod.rs:287-321)
    p = Path().quad((0, 0), (1, 1), (2, 0))
    s = oracle.flatten(p, [2.0, 0.0, 2.0, 0.0, 2.0, 2.0, 0.0, 0.0, 1.0])
    assert tuple(s[0][:2]) == (2.0, 2.0)
    assert tuple(s[-1][2:]) == (6.0, 2.0)


def test_scale_translate_t22_not_1():
    # mold/src/path/mod.rs:323-334
    p = Path().quad((0, 0), (1, 1), (2, 0))
    s = oracle.flatten(p, [2.0, 0.0, 2.0, 0.0, 2.0, 2.0, 0.0, 0.0, 2.0])
    assert tuple(s[0][:2]) == (1.0, 1.0)
    assert tuple(s[-1][2:]) == (3.0, 1.0)


def test_perspective_transform_quad():
    # perspective_transform_quad (mold/src/path/mod.rs:300-314): the quad becomes
    # RatQuad [(0,0),1], [(1,1),1.5], [(2,0),2]; its end points are (0,0) and (1,0).
    p = Path().quad((0, 0), (1, 1), (2, 0))
    s = oracle.flatten(p, [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.5, 0.0, 1.0])
    r = Path().rat_quad(((0, 0), 1.0), ((1.0 / 1.5, 1.0 / 1.5), 1.5), ((1.0, 0.0), 2.0))
    assert tuple(s[0][:2]) == (0.0, 0.0)
    assert tuple(s[-1][2:]) == (1.0, 0.0)
    assert len(s) == len(oracle.flatten(r))


def test_rational_bezier_with_weights_1():
    # mold/src/path/mod.rs:336-358
    a = Path().quad((2, 0), (2, 2), (0, 2))
    b = Path().rat_quad(((2, 0), 1.0), ((2, 2), 1.0), ((0, 2), 1.0))
    assert segs_list(oracle.flatten(a)) == segs_list(oracle.flatten(b))


def test_circle_rational_bezier():
    # mold/src/path/mod.rs:360-385
    R = 10.0
    w = float(np.float32(math.sqrt(2.0)) / np.float32(2.0))
    p = Path().rat_quad(((R, 0.0), 1.0), ((R * w, R * w), w), ((0.0, R), 1.0))
    s = oracle.flatten(p)
    for row in s[1:]:
        for (x, y) in ((row[0], row[1]), (row[2], row[3])):
            assert np.float32(x) * np.float32(x) + np.float32(y) * np.float32(y) - np.float32(R * R) < 1e-4


def test_quad_split_into_segments():
    # mold/src/path/mod.rs:387-403
    assert len(oracle.flatten(Path().quad((0, 0), (1, 1), (2, 0)))) == 3


# ---- surpass/src/rasterizer/mod.rs:293-699 (historic, commented tables) ----------

NONE = np.uint64(1 << 63)


def decode(seg):
    seg = int(seg)
    if seg == int(NONE):
        return None

    def sext(v, b):
        v &= (1 << b) - 1
        return v - (1 << b) if v >> (b - 1) else v

    return {
        "tile_j": sext(seg >> 51, 12), "tile_i": sext(seg >> 38, 13), "layer": (seg >> 22) & 0xFFFF,
        "tile_y": (seg >> 19) & 7, "tile_x": (seg >> 16) & 7, "area": sext(seg >> 6, 10), "cover": sext(seg, 6),
    }


def areas_and_covers(p0, p1):
    out = []
    for s in oracle.rasterize_lines([[*p0, *p1]]):
        d = decode(s)
        out.append(None if d is None else (d["area"], d["cover"]))
    return out


AC = [
    ((3.0, 2.0), [(11 * 16 // 2, 11), None, (5 * 8 // 2 + 5 * 8, 5), (5 * 8 // 2, 5), (11 * 16 // 2, 11), None]),
    ((2.0, 3.0), [(16 * 11 // 2 + 16 * 5, 16), None, (8 * 5 // 2, 8), (8 * 5 // 2 + 8 * 11, 8), (16 * 11 // 2, 16), None]),
    ((-2.0, 3.0), [(16 * 11 // 2, 16), None, (8 * 5 // 2 + 8 * 11, 8), (8 * 5 // 2, 8), (16 * 11 // 2 + 16 * 5, 16), None]),
    ((-3.0, 2.0), [(11 * 16 // 2, 11), None, (5 * 8 // 2 + 5 * 8, 5), (5 * 8 // 2, 5), (11 * 16 // 2, 11), None]),
    ((-3.0, -2.0), [(-(11 * 16 // 2), -11), None, (-(5 * 8 // 2 + 5 * 8), -5), (-(5 * 8 // 2), -5), (-(11 * 16 // 2), -11), None]),
    ((-2.0, -3.0), [(-(16 * 11 // 2 + 16 * 5), -16), None, (-(8 * 5 // 2), -8), (-(8 * 5 // 2 + 8 * 11), -8), (-(16 * 11 // 2), -16), None]),
    ((2.0, -3.0), [(-(16 * 11 // 2), -16), None, (-(8 * 5 // 2 + 8 * 11), -8), (-(8 * 5 // 2), -8), (-(16 * 11 // 2 + 16 * 5), -16), None]),
    ((3.0, -2.0), [(-(11 * 16 // 2), -11), None, (-(5 * 8 // 2 + 5 * 8), -5), (-(5 * 8 // 2), -5), (-(11 * 16 // 2), -11), None]),
    ((1.0, 0.0), []),
    ((1.0, 1.0), [(16 * 16 // 2, 16), None]),
    ((0.0, 1.0), [(16 * 16, 16), None]),
    ((-1.0, 1.0), [(16 * 16 // 2, 16), None]),
    ((-1.0, 0.0), []),
    ((-1.0, -1.0), [(-(16 * 16 // 2), -16), None]),
    ((0.0, -1.0), [(-(16 * 16), -16), None]),
]


@pytest.mark.parametrize("p1,expected", AC)
def test_area_cover(p1, expected):
    # area_cover_octant_1..8 and area_cover_axis_* (rasterizer/mod.rs:342-524)
    assert areas_and_covers((0.0, 0.0), p1) == expected


def test_start_and_end_not_on_pixel_border():
    # rasterizer/mod.rs:685-698
    assert areas_and_covers((0.5, 0.25), (4.0, 2.0))[0] == (4 * 8 // 2, 4)
    assert areas_and_covers((0.0, 0.0), (3.5, 1.75))[6] == (4 * 8 // 2 + 4 * 8, 4)


T = 8  # TILE_SIZE read as the current TILE_WIDTH = TILE_HEIGHT


def tiles(p0, p1):
    out = []
    for s in oracle.rasterize_lines([[*p0, *p1]]):
        d = decode(s)
        # the rasterizer stores max(tile_i, -1) + 256 (rasterizer/mod.rs:188)
        out.append(None if d is None else (d["tile_i"] - 256, d["tile_j"], d["tile_x"], d["tile_y"]))
    return out


TILE_CASES = [
    ((T, T), (T + 3.0, T + 2.0), [(1, 1, 0, 0), None, (1, 1, 1, 0), (1, 1, 1, 1), (1, 1, 2, 1), None]),
    ((T, T), (T + 2.0, T + 3.0), [(1, 1, 0, 0), None, (1, 1, 0, 1), (1, 1, 1, 1), (1, 1, 1, 2), None]),
    ((-T, T), (-T - 2.0, T + 3.0), [(-1, 1, T - 1, 0), None, (-1, 1, T - 1, 1), (-1, 1, T - 2, 1), (-1, 1, T - 2, 2), None]),
    ((-T, T), (-T - 3.0, T + 2.0), [(-1, 1, T - 3, 1), None, (-1, 1, T - 2, 1), (-1, 1, T - 2, 0), (-1, 1, T - 1, 0), None]),
    ((-T, -T), (-T - 3.0, -T - 2.0), [(-1, -2, T - 3, T - 2), None, (-1, -2, T - 2, T - 2), (-1, -2, T - 2, T - 1), (-1, -2, T - 1, T - 1), None]),
    ((-T, -T), (-T - 2.0, -T - 3.0), [(-1, -2, T - 2, T - 3), None, (-1, -2, T - 2, T - 2), (-1, -2, T - 1, T - 2), (-1, -2, T - 1, T - 1), None]),
    ((T, -T), (T + 2.0, -T - 3.0), [(1, -2, 1, T - 3), None, (1, -2, 1, T - 2), (1, -2, 0, T - 2), (1, -2, 0, T - 1), None]),
    ((T, -T), (T + 3.0, -T - 2.0), [(1, -2, 0, T - 1), None, (1, -2, 1, T - 1), (1, -2, 1, T - 2), (1, -2, 2, T - 2), None]),
]


@pytest.mark.parametrize("p0,p1,expected", TILE_CASES)
def test_tiles(p0, p1, expected):
    # tile_octant_1..8 (rasterizer/mod.rs:526-683) with 8x8 tiles; tile_i -2 is
    # stored clamped to -1 (left of canvas).
    assert tiles(p0, p1) == expected


# ---- mold/src/composition.rs:331-799 (render KATs, TILE_SIZE read as 8) ---------------

BLACK = (0x00, 0x00, 0x00, 0xFF)
BLACKF = (0.0, 0.0, 0.0, 1.0)
RED = (0xFF, 0x00, 0x00, 0xFF)
REDF = (1.0, 0.0, 0.0, 1.0)
GREEN = (0x00, 0xFF, 0x00, 0xFF)
GREENF = (0.0, 1.0, 0.0, 1.0)
RED_GREEN_50 = (0xBB, 0xBB, 0x00, 0xFF)


def pixel_path(x, y):
    return (Path().line((x, y), (x, y + 1)).line((x, y + 1), (x + 1, y + 1))
            .line((x + 1, y + 1), (x + 1, y)).line((x + 1, y), (x, y)))


def buf(n, color, width=None):
    a = np.zeros((1 if width is None else n // width, n if width is None else width, 4), np.uint8)
    a[...] = color
    return a


def px(a, i):
    return tuple(int(v) for v in a.reshape(-1, 4)[i])


def render(comp, b, width, bg, cache=-1):
    return comp.render(b, width, bg, layer_cache=cache)


@pytest.fixture(params=[False, True], ids=["u16", "wide"])
def comp(request):
    return oracle.Composition(wide=request.param)


def test_background_color_clear(comp):
    b = buf(1, GREEN)
    render(comp, b, 1, REDF)
    assert px(b, 0) == RED


def test_one_pixel(comp):
    b = buf(3, GREEN)
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(1, 0))
    comp.set_props(lid, solid(REDF))
    render(comp, b, 3, GREENF)
    assert [px(b, i) for i in range(3)] == [GREEN, RED, GREEN]


def test_two_pixels_same_layer(comp):
    b = buf(3, GREEN)
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(1, 0))
    comp.set_props(lid, solid(REDF))
    comp.insert_in_layer(lid, pixel_path(2, 0))
    render(comp, b, 3, GREENF)
    assert [px(b, i) for i in range(3)] == [GREEN, RED, RED]


def test_one_pixel_translated(comp):
    b = buf(3, GREEN)
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(1, 0))
    comp.set_props(lid, solid(REDF))
    comp.set_transform(lid, [1.0, 0.0, 0.0, 1.0, 0.5, 0.0])
    render(comp, b, 3, GREENF)
    assert [px(b, i) for i in range(3)] == [GREEN, RED_GREEN_50, RED_GREEN_50]


def test_one_pixel_rotated(comp):
    b = buf(3, GREEN)
    a = np.float32(-math.pi / 2.0)
    c, s = float(np.cos(a, dtype=np.float32)), float(np.sin(a, dtype=np.float32))
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(-1, 1))
    comp.set_props(lid, solid(REDF))
    comp.set_transform(lid, [c, -s, s, c, 0.0, 0.0])
    render(comp, b, 3, GREENF)
    assert [px(b, i) for i in range(3)] == [GREEN, RED, GREEN]


def test_remove_and_resize(comp):
    # mold/src/composition.rs:434-484.  The reference caches the BufferLayout
    # per buffer (ptr, len) (composition.rs:238-241), so the later renders keep
    # the first render's 4-pixel width.
    b = buf(4, GREEN)
    ids = [comp.create_layer() for _ in range(3)]
    comp.insert_in_layer(ids[0], pixel_path(0, 0))
    comp.set_props(ids[0], solid(REDF))
    comp.insert_in_layer(ids[1], pixel_path(1, 0))
    comp.set_props(ids[1], solid(REDF))
    comp.insert_in_layer(ids[2], pixel_path(2, 0))
    comp.set_props(ids[2], solid(REDF))
    comp.insert_in_layer(ids[2], pixel_path(3, 0))
    comp.set_props(ids[2], solid(REDF))
    render(comp, b, 4, GREENF)
    assert [px(b, i) for i in range(4)] == [RED] * 4
    assert comp.lens() == (16, 16)
    b[...] = GREEN
    comp.set_enabled(ids[0], False)
    render(comp, b, 4, GREENF)
    assert [px(b, i) for i in range(4)] == [GREEN, RED, RED, RED]
    assert comp.lens() == (16, 12)
    b[...] = GREEN
    comp.set_enabled(ids[2], False)
    render(comp, b, 4, GREENF)
    assert [px(b, i) for i in range(4)] == [GREEN, RED, GREEN, GREEN]
    assert comp.lens() == (4, 4)


def test_remove_twice(comp):
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(0, 0))
    comp.set_props(lid, solid(REDF))
    assert comp.lens()[1] == 4
    comp.set_enabled(lid, False)
    assert comp.lens()[1] == 0
    comp.set_enabled(lid, False)
    assert comp.lens()[1] == 0


def test_render_change_layers_only(comp):
    b = buf(3 * T * T, BLACK, width=3 * T)
    cache = comp.create_buffer_layer_cache()
    l0 = comp.create_layer()
    comp.insert_in_layer(l0, pixel_path(0, 0))
    comp.set_props(l0, solid(REDF))
    comp.insert_in_layer(l0, pixel_path(T, 0))
    l1 = comp.create_layer()
    comp.insert_in_layer(l1, pixel_path(T + 1, 0))
    comp.set_props(l1, solid(GREENF))
    comp.insert_in_layer(l1, pixel_path(2 * T, 0))
    render(comp, b, 3 * T, BLACKF, cache)
    assert px(b, 0) == RED and px(b, T) == RED and px(b, T + 1) == GREEN and px(b, 2 * T) == GREEN
    b[...] = BLACK
    comp.set_props(l1, solid(REDF))
    render(comp, b, 3 * T, BLACKF, cache)
    assert px(b, 0) == BLACK and px(b, T) == RED and px(b, T + 1) == RED and px(b, 2 * T) == RED


def test_clear_emptied_tiles(comp):
    # mold/src/composition.rs:581-664; the layout stays 2*T wide (cached per buffer).
    b = buf(2 * T * T, BLACK, width=2 * T)
    cache = comp.create_buffer_layer_cache()
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(0, 0))
    comp.set_props(lid, solid(REDF))
    comp.insert_in_layer(lid, pixel_path(T, 0))
    render(comp, b, 2 * T, BLACKF, cache)
    assert px(b, 0) == RED
    comp.set_transform(lid, [1.0, 0.0, 0.0, 1.0, float(T), 0.0])
    render(comp, b, 2 * T, BLACKF, cache)
    assert px(b, 0) == BLACK
    comp.set_transform(lid, [1.0, 0.0, 0.0, 1.0, -float(T), 0.0])
    render(comp, b, 2 * T, BLACKF, cache)
    assert px(b, 0) == RED
    comp.set_transform(lid, [1.0, 0.0, 0.0, 1.0, 0.0, float(T)])
    render(comp, b, 2 * T, BLACKF, cache)
    assert px(b, 0) == BLACK


def test_separate_layer_caches(comp):
    b = buf(T * T, BLACK, width=T)
    c0 = comp.create_buffer_layer_cache()
    c1 = comp.create_buffer_layer_cache()
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(0, 0))
    comp.set_props(lid, solid(REDF))
    render(comp, b, T, BLACKF, c0)
    assert px(b, 0) == RED
    b[...] = BLACK
    render(comp, b, T, BLACKF, c0)
    assert px(b, 0) == BLACK
    render(comp, b, T, BLACKF, c1)
    assert px(b, 0) == RED
    comp.set_transform(lid, [1.0, 0.0, 0.0, 1.0, 1.0, 0.0])
    render(comp, b, T, BLACKF, c0)
    assert px(b, 0) == BLACK and px(b, 1) == RED
    b[...] = BLACK
    render(comp, b, T, BLACKF, c1)
    assert px(b, 0) == BLACK and px(b, 1) == RED


def test_even_odd(comp):
    p = (Path().line((0, 0), (0, T)).line((0, T), (3 * T, T)).line((3 * T, T), (3 * T, 0))
         .line((3 * T, 0), (T, 0)).line((T, 0), (T, T)).line((T, T), (2 * T, T)).line((2 * T, T), (2 * T, 0))
         .line((2 * T, 0), (0, 0)))
    b = buf(3 * T * T, BLACK, width=3 * T)
    lid = comp.create_layer()
    comp.insert_in_layer(lid, p)
    comp.set_props(lid, Props(fill_rule=FillRule.EvenOdd, func=Style(fill=REDF)))
    render(comp, b, 3 * T, BLACKF)
    assert px(b, 0) == RED and px(b, T) == BLACK and px(b, 2 * T) == RED


def test_set_transform_scale_check():
    # mold/src/layer.rs:186-190 panics; the C ABI reports CGB_ERR_SCALE unless
    # the caller opts into surpass's unchecked affine (D4).
    comp = oracle.Composition()
    lid = comp.create_layer()
    comp.insert_in_layer(lid, pixel_path(0, 0))
    with pytest.raises(Exception):
        comp.set_transform(lid, [2.0, 0.0, 0.0, 2.0, 0.0, 0.0])
    comp.set_transform(lid, [2.0, 0.0, 0.0, 2.0, 0.0, 0.0], unchecked=True)
