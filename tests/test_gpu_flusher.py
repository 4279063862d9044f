"""mold Buffer::flusher (mold/src/buffer.rs:19-25; painter/mod.rs:483-492).

The flusher sees each row slice (at most 8 pixels) of every tile the render
wrote, after the tile is painted, and may change it: the frame must equal the
oracle's render with the same flush applied to those slices.  Tiles outside
a crop, and tiles left unchanged by a layer cache, are not flushed.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes

pytestmark = pytest.mark.gpu


def _flush_like(img, w, h, tiles):
    for j, i in tiles:
        for y in range(j * 8, min(j * 8 + 8, h)):
            s = img[y, i * 8:min(i * 8 + 8, w)]
            s[:, [0, 2]] = s[:, [2, 0]]  # swap red and blue
            s[:, 1] = 255 - s[:, 1]


def test_flusher_sees_every_written_tile_and_crop(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=81, n_layers=300, width=203, height=117)
    g, o = Composition(), oracle.Composition()
    scenes.load(sc, g)
    scenes.load(sc, o)
    calls = []

    def flusher(view):
        calls.append(len(view))
        view[:, [0, 2]] = view[:, [2, 0]].copy()
        view[:, 1] = 255 - view[:, 1]

    a = np.zeros((sc.height, sc.width, 4), np.uint8)
    g.render(a, sc.width, sc.background, flusher=flusher)
    b = np.zeros_like(a)
    o.render(b, sc.width, sc.background, threads=4)
    rows, cols = (sc.height + 7) // 8, (sc.width + 7) // 8
    _flush_like(b, sc.width, sc.height, [(j, i) for j in range(rows) for i in range(cols)])
    assert np.array_equal(a, b)
    assert len(calls) == sc.height * cols and max(calls) == 8 and min(calls) == sc.width % 8
    # with a crop only the crop's tiles are written and flushed
    crop = (40, 130, 16, 90)
    a2 = np.full_like(a, 3)
    calls.clear()
    g.render(a2, sc.width, sc.background, crop=crop, flusher=flusher)
    b2 = np.full_like(a2, 3)
    o.render(b2, sc.width, sc.background, crop=crop, threads=4)
    _flush_like(b2, sc.width, sc.height, [(j, i) for j in range(2, 12) for i in range(5, 17)])
    assert np.array_equal(a2, b2)


def test_unchanged_tiles_are_not_flushed(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=82, n_layers=100, width=96, height=64)
    g = Composition()
    scenes.load(sc, g)
    cache = g.create_buffer_layer_cache()
    a = np.zeros((sc.height, sc.width, 4), np.uint8)
    g.render(a, sc.width, sc.background, layer_cache=cache)
    calls = []
    g.render(a, sc.width, sc.background, layer_cache=cache, flusher=lambda v: calls.append(1))
    assert calls == []  # nothing changed: every tile is TileWriteOp::None
