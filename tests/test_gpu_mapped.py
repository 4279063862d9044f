"""Output buffers in page-locked host memory that the painter writes directly
(CGB_MEMORY_HOST_MAPPED): the same pixels as a host buffer (staged on the
device and copied back) and the oracle, with crops, layer caches, flushers,
frame graphs and batches; pageable memory is refused."""
import numpy as np
import pytest

import oracle
from cassia_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _pinned(shape, fill=0):
    import torch
    a = torch.zeros(shape, dtype=torch.uint8).pin_memory().numpy()
    a[...] = fill
    return a


def test_mapped_equals_host_and_oracle(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=91, n_layers=400, width=203, height=157)
    g, o = Composition(), oracle.Composition()
    scenes.load(sc, g)
    scenes.load(sc, o)
    ref = np.zeros((sc.height, sc.width, 4), np.uint8)
    o.render(ref, sc.width, sc.background, threads=4)
    m = _pinned(ref.shape)
    g.render(m, sc.width, sc.background, mapped=True)
    assert np.array_equal(m, ref)
    # frames replayed from a frame graph write the caller's pages too
    g.set_graph_mode(True)
    for _ in range(3):
        m[...] = 7
        g.render(m, sc.width, sc.background, mapped=True)
        assert np.array_equal(m, ref)
    assert g.stats()["graph_replayed"] == 1


def test_mapped_crop_cache_and_flusher(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=92, n_layers=200, width=120, height=96)
    g = Composition()
    scenes.load(sc, g)
    crop = (16, 90, 8, 70)
    h = np.full((sc.height, sc.width, 4), 5, np.uint8)
    m = _pinned(h.shape, 5)
    g.render(h, sc.width, sc.background, crop=crop)
    g.render(m, sc.width, sc.background, crop=crop, mapped=True)
    assert np.array_equal(m, h)  # outside the crop the caller's pixels stay
    calls_h, calls_m = [], []
    h2, m2 = np.zeros_like(h), _pinned(h.shape)
    g.render(h2, sc.width, sc.background, flusher=lambda v: calls_h.append(v.copy()))
    g.render(m2, sc.width, sc.background, flusher=lambda v: calls_m.append(v.copy()), mapped=True)
    assert np.array_equal(m2, h2) and len(calls_h) == len(calls_m)
    assert all(np.array_equal(x, y) for x, y in zip(calls_h, calls_m))
    # a layer cache: unchanged tiles are not written, so the caller's pixels stay
    cache = g.create_buffer_layer_cache()
    m3 = _pinned(h.shape)
    g.render(m3, sc.width, sc.background, layer_cache=cache, mapped=True)
    m3[:8, :8] = 200  # a tile no layer changes keeps what the caller wrote
    g.render(m3, sc.width, sc.background, layer_cache=cache, mapped=True)
    h3 = np.zeros_like(h)
    g2 = Composition()
    scenes.load(sc, g2)
    cache2 = g2.create_buffer_layer_cache()
    g2.render(h3, sc.width, sc.background, layer_cache=cache2)
    h3[:8, :8] = 200
    g2.render(h3, sc.width, sc.background, layer_cache=cache2)
    assert np.array_equal(m3, h3)


def test_mapped_batch(gpu_lib):
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    sset = [scenes.mixed(seed=93 + k, n_layers=150, width=64 + 40 * k, height=48 + 24 * k) for k in range(3)]
    comps = []
    for sc in sset:
        c = Composition()
        scenes.load(sc, c)
        comps.append(c)
    ctx = Composition()
    mapped = [_pinned((sc.height, sc.width, 4)) for sc in sset]
    render_batch(ctx, comps, mapped, [sc.width for sc in sset], [sc.background for sc in sset], mapped=True)
    for c, sc, m in zip(comps, sset, mapped):
        h = np.zeros_like(m)
        c.render(h, sc.width, sc.background)
        assert np.array_equal(m, h)


def test_pageable_memory_is_refused(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=97, n_layers=20, width=64, height=64)
    g = Composition()
    scenes.load(sc, g)
    pageable = np.zeros((sc.height, sc.width, 4), np.uint8)
    with pytest.raises(abi.CassiaError) as ex:
        g.render(pageable, sc.width, sc.background, mapped=True)
    assert ex.value.status == abi.ERR_INVALID_ARG
    g.render(pageable, sc.width, sc.background)  # the same buffer as a host buffer still renders
    assert pageable.any()


def test_mapped_from_another_thread(gpu_lib):
    """A render call from a thread that has made no CUDA call yet (the
    device addresses of page-locked memory are those of a current context)."""
    import threading
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=98, n_layers=60, width=80, height=64)
    g = Composition()
    scenes.load(sc, g)
    h = np.zeros((sc.height, sc.width, 4), np.uint8)
    g.render(h, sc.width, sc.background)
    m = _pinned(h.shape)
    errors = []

    def run():
        try:
            g.render(m, sc.width, sc.background, mapped=True)
        except BaseException as e:
            errors.append(e)

    t = threading.Thread(target=run)
    t.start()
    t.join()
    assert not errors, errors
    assert np.array_equal(m, h)
