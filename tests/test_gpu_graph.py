"""Frame graphs (cgb_set_graph_mode): a frame replayed from a CUDA graph equals
the same frame rendered stage by stage, bit for bit.

A replayed frame keeps S, P, G and W on the device and its buffers are sized
with headroom above the counts of the frame the graph was captured after.
Covered: capture then replay (and the oracle), transforms that change between
frames so that the counts move inside and past the capacities (headroom 0
forces the overflow path: nothing painted, the frame rendered again stage by
stage), host buffers with a flusher and a layer cache, batched groups with
one graph per group, and clip and gradient scenes (the full painter).
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes
from cassia_gb300.types import BlendMode, FillRule, Gradient, Props, Style

pytestmark = pytest.mark.gpu


def _pair(sc, headroom=0.125, wide=False):
    from cassia_gb300 import Composition
    g, ref = Composition(wide=wide), Composition(wide=wide)
    g.set_graph_mode(True, headroom)
    scenes.load(sc, g)
    scenes.load(sc, ref)
    return g, ref


def _render(c, sc, **kw):
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    c.render(img, sc.width, sc.background, **kw)
    return img


def test_replay_equals_staged_and_oracle(gpu_lib):
    import torch
    from cassia_gb300.composition import kernel_launches
    sc = scenes.mixed(seed=91, n_layers=3000, width=640, height=400)
    g, ref = _pair(sc)
    out = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
    want = _render(ref, sc)
    replayed = []
    for k in range(4):
        out.zero_()
        l0 = kernel_launches()
        g.render(out.data_ptr(), sc.width, sc.background, height=sc.height)
        st = g.stats()
        replayed.append(st["graph_replayed"])
        assert kernel_launches() > l0
        assert np.array_equal(out.cpu().numpy(), want), f"frame {k}"
    assert replayed == [0, 1, 1, 1]
    assert st["graphs_cached"] == 1
    rs = ref.stats()
    for key in ("steps", "segments", "painted_segments", "tile_layers", "work_items"):
        assert st[key] == rs[key], key
    o = oracle.Composition()
    scenes.load(sc, o)
    b = np.zeros_like(want)
    o.render(b, sc.width, sc.background, threads=8)
    assert np.array_equal(want, b)


@pytest.mark.parametrize("headroom", [0.125, 0.0])
def test_changing_transforms_inside_and_past_capacity(gpu_lib, headroom):
    sc = scenes.mixed(seed=92, n_layers=2500, width=512, height=384)
    g, ref = _pair(sc, headroom)
    ids = np.arange(sc.n_layers, dtype=np.uint32)
    base = sc.transforms.astype(np.float32).copy()
    replayed = []
    # grow, then shrink: counts pass the capacities of the graph captured
    # after the first frame, then fall back inside them
    for k, s in enumerate([1.0, 1.0, 1.15, 1.3, 1.3, 0.9, 0.9, 1.02]):
        tr = base.copy()
        tr[:, :4] *= np.float32(s)
        tr[:, 4] += np.float32(0.37 * k)
        g.set_transforms(ids, tr)
        ref.set_transforms(ids, tr)
        a = _render(g, sc)
        replayed.append(g.stats()["graph_replayed"])
        assert np.array_equal(a, _render(ref, sc)), f"frame {k} (scale {s})"
    assert replayed[0] == 0 and replayed[1] == 1
    if headroom == 0.0:
        assert replayed[2] == 0  # 15% more segments than the graph holds: rendered stage by stage
    assert sum(replayed) >= 3


def test_host_buffer_flusher_and_layer_cache(gpu_lib):
    sc = scenes.mixed(seed=93, n_layers=800, width=203, height=117)
    g, ref = _pair(sc)
    cg, cr = g.create_buffer_layer_cache(), ref.create_buffer_layer_cache()
    seen = []

    def flusher(view):
        seen.append(len(view))
        view[:, 1] = 255 - view[:, 1]

    a = np.zeros((sc.height, sc.width, 4), np.uint8)
    b = np.zeros_like(a)
    for k in range(4):
        if k == 2:  # one layer moves: the cache repaints only its tiles
            t = sc.transforms[5].copy()
            t[4] += 9.0
            g.set_transform(5, t, unchecked=True)
            ref.set_transform(5, t, unchecked=True)
        n0 = len(seen)
        g.render(a, sc.width, sc.background, layer_cache=cg, flusher=flusher)
        n_g = len(seen) - n0
        ref.render(b, sc.width, sc.background, layer_cache=cr, flusher=flusher)
        assert np.array_equal(a, b), f"frame {k}"
        assert n_g == len(seen) - n0 - n_g  # the same row slices were flushed
        assert g.stats()["graph_replayed"] == (1 if k else 0)


def test_batched_groups_replay(gpu_lib):
    from cassia_gb300 import Composition
    from cassia_gb300.composition import render_batch
    groups = [[scenes.mixed(seed=200 + k, n_layers=n, width=w, height=w) for k, (n, w) in enumerate(grp)]
              for grp in ([(40, 256), (900, 512), (7, 64)], [(300, 512), (1200, 384)])]
    ctx = Composition()
    ctx.set_graph_mode(True)
    comps, alone = [], []
    for grp in groups:
        cs, outs = [], []
        for sc in grp:
            c = Composition()
            scenes.load(sc, c)
            cs.append(c)
            outs.append(_render(c, sc))
        comps.append(cs)
        alone.append(outs)
    # the groups share the handle's buffers: a capture that grows them makes
    # the other group's graph stale (recaptured on its next frame) until the
    # sizes settle
    for rep in range(5):
        for grp, cs, want in zip(groups, comps, alone):
            outs = [np.zeros((sc.height, sc.width, 4), np.uint8) for sc in grp]
            render_batch(ctx, cs, outs, [sc.width for sc in grp], [sc.background for sc in grp])
            if rep == 0:
                assert ctx.stats()["graph_replayed"] == 0
            if rep == 4:
                assert ctx.stats()["graph_replayed"] == 1
            for o, w in zip(outs, want):
                assert np.array_equal(o, w)
    assert ctx.stats()["graphs_cached"] == 2


def test_clips_and_gradients_replay(gpu_lib):
    sc = scenes.mixed(seed=94, n_layers=900, width=320, height=200)
    rng = np.random.default_rng(94)
    kinds = rng.integers(0, 10, size=sc.n_layers)
    clip_n = rng.integers(1, 12, size=sc.n_layers)
    grad = Gradient(start=(20.0, 10.0), end=(250.0, 180.0),
                    stops=[((1.0, 0.2, 0.0, 1.0), None), ((0.0, 0.4, 1.0, 0.6), None)])
    g, ref = _pair(sc)
    for c in (g, ref):
        for k in range(sc.n_layers):
            fr = FillRule(int(sc.fill_rule[k]))
            mode = BlendMode(int(sc.blend_mode[k]))
            if kinds[k] == 0:
                c.set_props(k, Props(fill_rule=fr, func=int(clip_n[k])))
            elif kinds[k] <= 2:
                col = tuple(float(v) for v in sc.color[k])
                c.set_props(k, Props(fill_rule=fr, func=Style(fill=col, blend_mode=mode, is_clipped=True)))
            elif kinds[k] == 3:
                c.set_props(k, Props(fill_rule=fr, func=Style(fill=grad, blend_mode=mode)))
    want = _render(ref, sc)
    for k in range(3):
        assert np.array_equal(_render(g, sc), want), f"frame {k}"
    assert g.stats()["graph_replayed"] == 1
    o = oracle.Composition()
    scenes.load(sc, o)
    for k in range(sc.n_layers):
        fr = FillRule(int(sc.fill_rule[k]))
        mode = BlendMode(int(sc.blend_mode[k]))
        if kinds[k] == 0:
            o.set_props(k, Props(fill_rule=fr, func=int(clip_n[k])))
        elif kinds[k] <= 2:
            col = tuple(float(v) for v in sc.color[k])
            o.set_props(k, Props(fill_rule=fr, func=Style(fill=col, blend_mode=mode, is_clipped=True)))
        elif kinds[k] == 3:
            o.set_props(k, Props(fill_rule=fr, func=Style(fill=grad, blend_mode=mode)))
    b = np.zeros_like(want)
    o.render(b, sc.width, sc.background, threads=8)
    assert np.array_equal(want, b)
