"""Incremental frames (cgb_set_incremental): a composition that keeps its last
frame's sorted segments on the device and rasterizes only changed layers
renders every frame bit-exact with a composition that rasterizes everything.

Frames change 20% of the layers' transforms, remove and add layers (the
serving workload's seeded updates), swap layer orders, disable and re-enable
layers and change the canvas; single renders, batched renders and the oracle;
and with layer caches, crops, gradient fills and clip layers in the painter.
"""
from types import SimpleNamespace

import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes, serving
from cassia_gb300.types import BlendMode, FillRule, Gradient, Props, Style

pytestmark = pytest.mark.gpu


def _pair(sc, pool, wide=False):
    from cassia_gb300 import Composition
    out = []
    for inc in (True, False):
        c = Composition(wide=wide)
        scenes.load(sc, c)
        if inc:
            c.set_incremental(True)
        out.append(serving.Client(c, sc, None, np.ones(sc.n_layers, bool), sc.transforms.copy(), pool=pool))
    return out


def _render(c, sc, width=None, height=None):
    w, h = width or sc.width, height or sc.height
    img = np.zeros((h, w, 4), np.uint8)
    c.render(img, w, sc.background)
    return img


def _assert_same(a, b, what):
    if not np.array_equal(a, b):
        d = np.argwhere(np.any(a != b, axis=-1))
        y, x = d[0]
        raise AssertionError(f"{what}: {len(d)} pixels differ; first at ({x}, {y}): {a[y, x]} vs {b[y, x]}")


def test_incremental_frames_match_full_frames_and_oracle(gpu_lib):
    sc = scenes.mixed(seed=95, n_layers=3000, width=640, height=400)
    pool = scenes.mixed(seed=96, n_layers=64, width=640, height=400)
    cg, cr = _pair(sc, pool)
    o = oracle.Composition()
    scenes.load(sc, o)
    co = serving.Client(o, sc, None, np.ones(sc.n_layers, bool), sc.transforms.copy(), pool=pool)
    rasterized = []

    def frame(what):
        a, b = _render(cg.comp, sc), _render(cr.comp, sc)
        _assert_same(a, b, what)
        sg, sr = cg.comp.stats(), cr.comp.stats()
        for key in ("painted_segments", "tile_layers", "work_items"):
            assert sg[key] == sr[key], (what, key)
        rasterized.append((sg["segments"], sr["segments"]))
        return a

    for seq in range(9):
        if seq:
            for cl in (cg, cr, co):
                serving.apply_update(cl, 0, seq, changed=0.2, churn=0.02)
        a = frame(f"frame {seq}")
        live = np.flatnonzero(cr.enabled).astype(np.uint32)
        if seq == 4:  # two layers exchange their orders (orders default to the ids)
            x, y = int(live[10]), int(live[-10])
            for cl in (cg, cr, co):
                cl.comp.set_order(x, y)
                cl.comp.set_order(y, x)
            a = frame("orders exchanged")
        if seq == 6:  # layers off, then back on before the next update collects them
            ids = live[100:140]
            for cl in (cg, cr, co):
                cl.comp.set_enabled_many(ids, np.zeros(len(ids), np.uint8))
            frame("layers disabled")
            for cl in (cg, cr, co):
                cl.comp.set_enabled_many(ids, np.ones(len(ids), np.uint8))
            a = frame("layers enabled again")
    # after the first frame only the changed layers' segments are rasterized
    assert rasterized[0][0] == rasterized[0][1]
    assert all(g < r for g, r in rasterized[1:])
    ref = np.zeros_like(a)
    o.render(ref, sc.width, sc.background, threads=8)
    _assert_same(a, ref, "oracle")


def test_unchanged_frame_and_canvas_change(gpu_lib):
    sc = scenes.mixed(seed=97, n_layers=1500, width=300, height=200)
    pool = scenes.mixed(seed=98, n_layers=32, width=300, height=200)
    cg, cr = _pair(sc, pool)
    want = _render(cr.comp, sc)
    _assert_same(_render(cg.comp, sc), want, "first")
    _assert_same(_render(cg.comp, sc), want, "nothing changed")
    assert cg.comp.stats()["segments"] == 0
    # another canvas: every line again, then incremental on the new canvas
    for k in range(3):
        if k:
            for cl in (cg, cr):
                serving.apply_update(cl, 1, k)
        _assert_same(_render(cg.comp, sc, 333, 150), _render(cr.comp, sc, 333, 150), f"canvas frame {k}")
    # cleared and rebuilt
    for cl in (cg, cr):
        cl.comp.clear()
        scenes.load(sc, cl.comp)
    _assert_same(_render(cg.comp, sc), _render(cr.comp, sc), "after clear")


@pytest.mark.parametrize("wide", [False, True])
def test_incremental_batch(gpu_lib, wide):
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    sizes = [(300, 256), (1500, 512), (40, 128), (800, 384)]
    pairs, scs = [], []
    for k, (n, w) in enumerate(sizes):
        sc = scenes.mixed(seed=300 + k, n_layers=n, width=w, height=w)
        pool = scenes.mixed(seed=400 + k, n_layers=32, width=w, height=w)
        pairs.append(_pair(sc, pool, wide=wide))
        scs.append(sc)
    ctx = Composition()
    for seq in range(6):
        if seq:
            for k, (cg, cr) in enumerate(pairs):
                if (seq + k) % 3:  # some scenes change, some do not
                    for cl in (cg, cr):
                        serving.apply_update(cl, k, seq)
        outs = [np.zeros((sc.height, sc.width, 4), np.uint8) for sc in scs]
        render_batch(ctx, [cg.comp for cg, _ in pairs], outs, [sc.width for sc in scs],
                     [sc.background for sc in scs])
        for k, ((cg, cr), sc) in enumerate(zip(pairs, scs)):
            _assert_same(outs[k], _render(cr.comp, sc), f"frame {seq}, scene {k}")
            # and the same composition rendered alone, incrementally
            _assert_same(_render(cg.comp, sc), outs[k], f"frame {seq}, scene {k} alone")


def test_incremental_with_caches_crops_gradients_and_clips(gpu_lib):
    sc = scenes.mixed(seed=99, n_layers=1200, width=320, height=200)
    pool = scenes.mixed(seed=100, n_layers=32, width=320, height=200)
    cg, cr = _pair(sc, pool)
    rng = np.random.default_rng(99)
    kinds = rng.integers(0, 10, size=sc.n_layers)
    clip_n = rng.integers(1, 12, size=sc.n_layers)
    grad = Gradient(start=(20.0, 10.0), end=(250.0, 180.0),
                    stops=[((1.0, 0.2, 0.0, 1.0), None), ((0.0, 0.4, 1.0, 0.6), None)])
    for cl in (cg, cr):
        for k in range(sc.n_layers):
            fr = FillRule(int(sc.fill_rule[k]))
            mode = BlendMode(int(sc.blend_mode[k]))
            if kinds[k] == 0:
                cl.comp.set_props(k, Props(fill_rule=fr, func=int(clip_n[k])))
            elif kinds[k] == 1:
                col = tuple(float(v) for v in sc.color[k])
                cl.comp.set_props(k, Props(fill_rule=fr, func=Style(fill=col, blend_mode=mode, is_clipped=True)))
            elif kinds[k] == 2:
                cl.comp.set_props(k, Props(fill_rule=fr, func=Style(fill=grad, blend_mode=mode)))
    caches = [cl.comp.create_buffer_layer_cache() for cl in (cg, cr)]
    crop = (24, 290, 16, 170)
    imgs = [np.zeros((sc.height, sc.width, 4), np.uint8) for _ in range(2)]
    for seq in range(6):
        if seq:
            for cl in (cg, cr):
                serving.apply_update(cl, 3, seq, changed=0.1, churn=0.02)
        for cl, cache, img in zip((cg, cr), caches, imgs):
            cl.comp.render(img, sc.width, sc.background, crop=crop if seq % 2 else None, layer_cache=cache)
        _assert_same(imgs[0], imgs[1], f"frame {seq}")


def test_incremental_full_size(gpu_lib):
    """Config 2a (65,535 layers, 2560x1600, ~42M segments per frame): incremental
    frames equal full frames through seeded transform updates of 20% of the
    layers (no layers added: the 16-bit format has no free ids left)."""
    import torch
    sc = scenes.mixed(seed=2, n_layers=65_535, width=2560, height=1600)
    pool = scenes.mixed(seed=3, n_layers=256, width=2560, height=1600)
    cg, cr = _pair(sc, pool)
    outs = [torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda") for _ in range(2)]
    for seq in range(4):
        if seq:
            for cl in (cg, cr):
                serving.apply_update(cl, 5, seq, changed=0.2, churn=0.0)
        for cl, out in zip((cg, cr), outs):
            cl.comp.render(out.data_ptr(), sc.width, sc.background, height=sc.height)
        assert torch.equal(outs[0], outs[1]), f"frame {seq}"
        sg, sr = cg.comp.stats(), cr.comp.stats()
        assert sg["painted_segments"] == sr["painted_segments"] > 40_000_000
        if seq:
            assert sg["segments"] < sr["segments"] // 3


def test_sync_free_incremental_frames_and_overflow(gpu_lib):
    """Incremental frames of a composition on its own handle run without
    host synchronization once an earlier incremental frame sized the
    buffers (incremental_form 2); an update larger than the capacities
    paints nothing and is rendered again stage by stage (form 1), which
    sizes the buffers for the next ones."""
    sc = scenes.mixed(seed=101, n_layers=2000, width=512, height=384)
    pool = scenes.mixed(seed=102, n_layers=32, width=512, height=384)
    cg, cr = _pair(sc, pool)
    forms = []
    for seq, frac in enumerate([0.0, 0.02, 0.02, 0.02, 0.6, 0.6, 0.02]):
        if seq:
            for cl in (cg, cr):
                serving.apply_update(cl, 7, seq, changed=frac, churn=0.0)
        _assert_same(_render(cg.comp, sc), _render(cr.comp, sc), f"frame {seq}")
        sg, sr = cg.comp.stats(), cr.comp.stats()
        for key in ("painted_segments", "tile_layers", "work_items"):
            assert sg[key] == sr[key], (seq, key)
        forms.append(sg["incremental_form"])
        assert sr["incremental_form"] == 0
    assert forms == [1, 1, 2, 2, 1, 2, 2], forms


def test_switching_between_incremental_and_graph_frames(gpu_lib):
    """One composition switched between incremental and full frames: every
    frame equals a composition that always renders full frames, and the
    frame form it reports is the form that frame ran in (a replayed graph
    is a full frame, form 0)."""
    sc = scenes.mixed(seed=103, n_layers=1200, width=384, height=256)
    pool = scenes.mixed(seed=104, n_layers=32, width=384, height=256)
    cg, cr = _pair(sc, pool)
    cg.comp.set_graph_mode(True)
    plan = [True, True, True, True, False, False, False, True, True, True]
    for seq, inc in enumerate(plan):
        if seq:
            for cl in (cg, cr):
                serving.apply_update(cl, 9, seq, changed=0.05, churn=0.0)
        cg.comp.set_incremental(inc)
        _assert_same(_render(cg.comp, sc), _render(cr.comp, sc), f"frame {seq}")
        st = cg.comp.stats()
        if not inc:
            assert st["incremental_form"] == 0, (seq, st["incremental_form"])
        else:
            assert st["incremental_form"] in (1, 2), (seq, st["incremental_form"])
        if not inc and seq == 6:  # the third full frame in a row replays its graph
            assert st["graph_replayed"] == 1


def test_more_new_than_resident_segments(gpu_lib):
    # A frame whose new segments outnumber the kept ones twenty to one, and
    # the frames around it with few new segments: every frame equals a
    # composition rendered in full and the oracle.
    from cassia_gb300 import Composition
    big = scenes.mixed(seed=131, n_layers=1200, width=480, height=320)
    few = 60
    comps = []
    for inc in (True, False):
        c = Composition()
        for _ in range(big.n_layers):
            c.create_layer()
        if inc:
            c.set_incremental(True)
        comps.append(c)
    o = oracle.Composition()
    for _ in range(big.n_layers):
        o.create_layer()

    def load(lo, hi):
        # the paths of layers [lo, hi) (a scene lists its paths layer by layer)
        k = np.flatnonzero((big.path_layer >= lo) & (big.path_layer < hi))
        k0, k1 = int(k[0]), int(k[-1]) + 1
        assert k1 - k0 == len(k)
        c0, c1 = int(big.cmd_offsets[k0]), int(big.cmd_offsets[k1])
        p0, p1 = int(big.point_offsets[k0]), int(big.point_offsets[k1])
        part = SimpleNamespace(n_paths=k1 - k0, path_layer=np.ascontiguousarray(big.path_layer[k0:k1]),
                               cmd_offsets=np.ascontiguousarray(big.cmd_offsets[k0:k1 + 1] - np.uint64(c0)),
                               kinds=np.ascontiguousarray(big.kinds[c0:c1]),
                               point_offsets=np.ascontiguousarray(big.point_offsets[k0:k1 + 1] - np.uint64(p0)),
                               points=np.ascontiguousarray(big.points[p0:p1]))
        ids = np.arange(lo, hi, dtype=np.uint32)
        for c in comps + [o]:
            c.insert_paths(part)
            c.set_layers_solid(ids, big.fill_rule[lo:hi], big.blend_mode[lo:hi], big.color[lo:hi])
            c.set_transforms(ids, big.transforms[lo:hi], unchecked=True)

    def frame(what):
        a, b = _render(comps[0], big), _render(comps[1], big)
        _assert_same(a, b, what)
        ref = np.zeros_like(a)
        o.render(ref, big.width, big.background, threads=8)
        _assert_same(a, ref, what + " (oracle)")
        return comps[0].stats()

    load(0, few)
    frame("few layers")
    frame("unchanged")
    load(few, big.n_layers)  # twenty times the layers: mostly new segments
    st = frame("many layers added")
    assert st["incremental_form"] >= 1
    ids = np.arange(0, big.n_layers, 7, dtype=np.uint32)
    t = big.transforms[ids].copy()
    t[:, 4] += 3.25
    for c in comps + [o]:
        c.set_transforms(ids, t, unchecked=True)
    frame("one layer in seven moved")
