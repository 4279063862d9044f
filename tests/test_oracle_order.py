"""The oracle's pixel segments come in the canonical order the GPU parity
tests compare against: ascending by the full 64-bit segment, which refines the
reference's unstable sort by `u64 >> 22` (surpass/src/rasterizer/mod.rs:287-290),
so the array is also monotone in that key; the count of NONE slots is
reported apart (none are returned); and the oracle's thread count changes
nothing.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes

CASES = {
    "circles": lambda: scenes.circles(seed=5, n_layers=200, size=256),
    "mixed": lambda: scenes.mixed(seed=6, n_layers=400, width=320, height=200),
    "glyphs": lambda: scenes.glyphs(seed=7, n_layers=300, width=384, height=216),
}


@pytest.mark.parametrize("name", list(CASES))
def test_canonical_order(name):
    sc = CASES[name]()
    o = oracle.Composition(wide=sc.wide)
    scenes.load(sc, o)
    a, none_a = o.pixel_segments(threads=1)
    b, none_b = o.pixel_segments(threads=8)
    assert len(a) > 1000
    assert np.array_equal(a, b) and none_a == none_b
    assert np.all(a[1:] >= a[:-1])
    k = a >> np.uint64(22)
    assert np.all(k[1:] >= k[:-1])
    # the top bit of the reference layout marks NONE (raster_segment.rs:13-160)
    assert not np.any(a >> np.uint64(63))
