"""Batched rendering: many compositions in one pipeline (cgb_render_batch).

Each scene's pixels from the batched frame must equal its own single-scene
render and the oracle's, bit for bit.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scene_set():
    out = []
    for k, (n, side) in enumerate([(12, 256), (300, 512), (40, 256), (1500, 1024), (7, 64), (900, 512)]):
        sc = scenes.mixed(seed=100 + k, n_layers=n, width=side, height=side)
        out.append(sc)
    out.append(scenes.circles(seed=110, n_layers=150, size=320))
    out.append(scenes.glyphs(seed=111, n_layers=200, width=400, height=120))
    w = scenes.mixed(seed=112, n_layers=500, width=200, height=130)  # non-multiple-of-8 canvas
    out.append(w)
    return out


def _render_single(sc):
    from cassia_gb300 import Composition
    c = Composition(wide=sc.wide)
    scenes.load(sc, c)
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    c.render(img, sc.width, sc.background)
    return c, img


def test_batch_equals_single_and_oracle(gpu_lib):
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    sset = _scene_set()
    comps, singles = [], []
    for sc in sset:
        c, img = _render_single(sc)
        comps.append(c)
        singles.append(img)
    ctx = Composition()
    outs = [np.zeros((sc.height, sc.width, 4), np.uint8) for sc in sset]
    render_batch(ctx, comps, outs, [sc.width for sc in sset], [sc.background for sc in sset])
    for k, sc in enumerate(sset):
        assert np.array_equal(outs[k], singles[k]), f"scene {k} batched != single"
        o = oracle.Composition(wide=sc.wide)
        scenes.load(sc, o)
        ref = np.zeros_like(outs[k])
        o.render(ref, sc.width, sc.background, threads=4)
        assert np.array_equal(outs[k], ref), f"scene {k} batched != oracle"
    # a second batched frame after a few transform changes still matches
    rng = np.random.default_rng(3)
    for k, sc in enumerate(sset):
        if sc.transforms is None:
            continue
        ids = rng.choice(sc.n_layers, size=max(1, sc.n_layers // 5), replace=False).astype(np.uint32)
        t = sc.transforms[ids].copy()
        t[:, 4] += rng.uniform(-9, 9, size=len(ids)).astype(np.float32)
        comps[k].set_transforms(ids, t)
    outs2 = [np.zeros_like(x) for x in outs]
    render_batch(comps[0], comps, outs2, [sc.width for sc in sset], [sc.background for sc in sset])
    for k, sc in enumerate(sset):
        single = np.zeros_like(outs2[k])
        comps[k].render(single, sc.width, sc.background)
        assert np.array_equal(outs2[k], single), f"frame 2 scene {k}"


def test_batch_with_crops_caches_and_empty_scene(gpu_lib):
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    a = scenes.mixed(seed=120, n_layers=200, width=160, height=96)
    b = scenes.mixed(seed=121, n_layers=100, width=96, height=64)
    ca, cb_, ce = Composition(), Composition(), Composition()
    scenes.load(a, ca)
    scenes.load(b, cb_)
    oa, ob = oracle.Composition(), oracle.Composition()
    scenes.load(a, oa)
    scenes.load(b, ob)
    cache_g, cache_o = ca.create_buffer_layer_cache(), oa.create_buffer_layer_cache()
    crop_b = (13, 70, 9, 50)
    for frame in range(3):
        ga = np.full((a.height, a.width, 4), 5 + frame, np.uint8)
        gb = np.full((b.height, b.width, 4), 9, np.uint8)
        ge = np.full((16, 24, 4), 1, np.uint8)
        ra, rb = ga.copy(), gb.copy()
        render_batch(ca, [ca, cb_, ce], [ga, gb, ge], [a.width, b.width, 24],
                     [a.background, b.background, (0.5, 0.25, 0.125, 1.0)],
                     crops=[(0, a.width, 0, a.height), crop_b, (0, 24, 0, 16)], layer_caches=[cache_g, -1, -1])
        oa.render(ra, a.width, a.background, crop=(0, a.width, 0, a.height), layer_cache=cache_o, threads=4)
        ob.render(rb, b.width, b.background, crop=crop_b, threads=4)
        assert np.array_equal(ga, ra)
        assert np.array_equal(gb, rb)
        re = np.full_like(ge, 1)
        oracle.Composition().render(re, 24, (0.5, 0.25, 0.125, 1.0))
        assert np.array_equal(ge, re)
        ids = np.arange(0, a.n_layers, 7, dtype=np.uint32)
        t = a.transforms[ids].copy()
        t[:, 5] += np.float32(1.5 * (frame + 1))
        ca.set_transforms(ids, t)
        oa.set_transforms(ids, t)
