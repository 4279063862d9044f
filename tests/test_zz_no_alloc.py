"""The allocation-free sort entry point (cgb_sort_keys_noalloc) against the
existing pipeline's sort.

Callers that cannot allocate device memory while they run (a render loop with
its memory reserved up front, or a process whose device memory belongs to
another allocator) use cgb_sort_keys_noalloc, whose scratch is a static
device array.  Its output must equal the canonical pixel_segments order of
the ordinary entry point, bit for bit, on two calls in a row (the second call
must not see the first call's leftover scratch).  This file is collected last
so that a run stopping at its first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 24


def _sort_noalloc(lib, keys_u64, bit_lo=0, bit_hi=64):
    import torch
    n = len(keys_u64)
    keys = torch.from_numpy(keys_u64.view(np.int64).copy()).cuda()
    out = torch.empty_like(keys)
    torch.cuda.synchronize()
    st = lib.cgb_sort_keys_noalloc(ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(out.data_ptr()), n,
                                   bit_lo, bit_hi, None)
    torch.cuda.synchronize()
    return st, out.cpu().numpy().view(np.uint64)


def _reference_sorted(scene):
    from cassia_gb300 import Composition, scenes
    c = Composition(wide=scene.wide)
    scenes.load(scene, c)
    segs, _ = c.pixel_segments(canonical=True)  # the existing entry point (cgb_pixel_segments)
    c.close()
    return segs


def test_noalloc_sort_matches_pipeline_sort_twice(gpu_lib):
    from cassia_gb300 import abi, scenes
    lib = abi.load_library()
    rng = np.random.default_rng(1234)
    for scene in (scenes.mixed(seed=31, n_layers=3000, width=640, height=400),
                  scenes.circles(seed=32, n_layers=500, size=512)):
        expected = _reference_sorted(scene)
        shuffled = expected[rng.permutation(len(expected))]
        st, got = _sort_noalloc(lib, shuffled)
        assert st == abi.OK, abi.STATUS_NAMES.get(st)
        assert np.array_equal(got, expected)


def test_noalloc_sort_key_bits_and_limits(gpu_lib):
    from cassia_gb300 import abi, scenes
    lib = abi.load_library()
    expected = _reference_sorted(scenes.circles(seed=33, n_layers=300, size=256))
    shuffled = expected[np.random.default_rng(7).permutation(len(expected))]
    st, got = _sort_noalloc(lib, shuffled, 22, 64)  # the reference's key: u64 >> 22
    assert st == abi.OK
    keys = got >> np.uint64(22)
    assert np.all(keys[1:] >= keys[:-1])
    assert np.array_equal(np.sort(got), expected)
    # sizes beyond the stated maximum are rejected before any device work
    assert lib.cgb_sort_keys_noalloc(None, None, MAX_KEYS + 1, 0, 64, None) == abi.ERR_CAPACITY


SORT_TILE = 7168  # keys one onesweep tile ranks


@pytest.mark.parametrize("n", [1, SORT_TILE + 1, MAX_KEYS])
def test_noalloc_sort_sizes_twice(gpu_lib, n):
    """One key, one key past a tile, and the stated maximum (where the
    look-back table uses every tile of the static array), each twice in a row
    with different keys, against numpy's sort."""
    from cassia_gb300 import abi
    lib = abi.load_library()
    rng = np.random.default_rng(n)
    for _ in range(2):
        keys = rng.integers(0, np.iinfo(np.uint64).max, size=n, dtype=np.uint64, endpoint=True)
        st, got = _sort_noalloc(lib, keys)
        assert st == abi.OK, abi.STATUS_NAMES.get(st)
        assert np.array_equal(got, np.sort(keys))


def test_noalloc_sort_rejects_overlap_and_capture(gpu_lib):
    """Overlapping buffers and a capturing stream are refused before any work;
    the next ordinary call still sorts."""
    import torch
    from cassia_gb300 import abi
    lib = abi.load_library()
    n = 5000
    buf = torch.zeros(2 * n, dtype=torch.int64, device="cuda")
    base = buf.data_ptr()
    assert lib.cgb_sort_keys_noalloc(ctypes.c_void_p(base), ctypes.c_void_p(base + 8 * (n // 2)), n, 0, 64,
                                     None) == abi.ERR_INVALID_ARG
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        buf.add_(1)  # something to capture
        st = lib.cgb_sort_keys_noalloc(ctypes.c_void_p(base), ctypes.c_void_p(base + 8 * n), n, 0, 64,
                                       ctypes.c_void_p(side.cuda_stream))
    assert st == abi.ERR_INVALID_ARG
    keys = np.random.default_rng(5).integers(0, 1 << 62, size=n, dtype=np.uint64)
    st, got = _sort_noalloc(lib, keys)
    assert st == abi.OK
    assert np.array_equal(got, np.sort(keys))
