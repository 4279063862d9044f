"""The render server: continuous batching over resident compositions.

After a run under Poisson arrivals, every client's last frame must equal the
same state rendered alone and the oracle's render after replaying the same
seeded updates, bit for bit.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _oracle_replay(cl, client_id, last_seq):
    from cassia_gb300 import scenes, serving
    sc = cl.scene
    o = oracle.Composition(wide=cl.comp.wide)
    scenes.load(sc, o)
    shadow = serving.Client(o, sc, None, np.ones(sc.n_layers, bool), sc.transforms.copy(), pool=cl.pool)
    for seq in range(last_seq + 1):
        serving.apply_update(shadow, client_id, seq)
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    o.render(img, sc.width, sc.background, threads=4)
    return img


@pytest.mark.parametrize("mode,incremental", [("batched", False), ("plain", False), ("batched", True)])
def test_server_results_match_alone_and_oracle(gpu_lib, mode, incremental):
    import torch
    from cassia_gb300 import serving
    clients = serving.make_clients(6, seed=42, device_out=True, max_layers=400, incremental=incremental)
    reqs = serving.poisson_arrivals(rate=400.0, n_clients=len(clients), duration=0.25, seed=1)
    srv = serving.Server(clients, mode=mode, workers=2, max_batch=4)
    done = srv.run(reqs)
    assert all(r.t_done >= r.arrival for r in done)
    for r in done:  # per-client frames completed in order
        assert r.t_done > 0
    for k, cl in enumerate(clients):
        got = cl.out.cpu().numpy()
        alone = torch.zeros_like(cl.out)
        cl.comp.render(alone.data_ptr(), cl.scene.width, cl.scene.background, height=cl.scene.height)
        assert np.array_equal(got, alone.cpu().numpy()), f"client {k}: mix != alone"
        if cl.done_seq >= 0:
            ref = _oracle_replay(cl, k, cl.done_seq)
            assert np.array_equal(got, ref), f"client {k}: != oracle after {cl.done_seq + 1} frames"
    summary = serving.latency_summary(done, 0.25)
    assert summary["p99_ms"] >= summary["p50_ms"] > 0


def test_admission_respects_budget(gpu_lib):
    from cassia_gb300 import serving
    clients = serving.make_clients(4, seed=43, device_out=True, max_layers=200)
    reqs = serving.poisson_arrivals(rate=500.0, n_clients=len(clients), duration=0.1, seed=2)
    # a budget that fits one client's frame at a time forces batches of one
    srv = serving.Server(clients, mode="batched", workers=2, max_batch=8, hbm_budget=1)
    done = srv.run(reqs)
    assert max(r.batch_size for r in done) == 1


def _alone(cl):
    import torch
    img = torch.zeros_like(cl.out)
    cl.comp.render(img.data_ptr(), cl.scene.width, cl.scene.background, height=cl.scene.height)
    return img


def test_library_refuses_an_over_budget_batch(gpu_lib):
    """The worker contexts' HBM budget is enforced by the library: a batch
    whose frame buffers do not fit is refused with CGB_ERR_OVER_BUDGET, and
    the server then renders it in halves; every result still equals the
    client's frame rendered alone."""
    import torch
    from cassia_gb300 import Composition, abi, serving
    from cassia_gb300.composition import render_batch
    clients = serving.make_clients(4, seed=44, device_out=True, max_layers=300)
    # the largest single client's frame buffers on a batch context
    single = 0
    for cl in clients:
        ctx = Composition()
        render_batch(ctx, [cl.comp], [cl.out.data_ptr()], [cl.scene.width], [cl.scene.background],
                     heights=[cl.scene.height])
        single = max(single, ctx.device_bytes())
        ctx.close()
    share = int(1.3 * single)
    # the library itself refuses the four together
    ctx = Composition(hbm_budget=share)
    with pytest.raises(abi.CassiaError) as ex:
        render_batch(ctx, [cl.comp for cl in clients], [cl.out.data_ptr() for cl in clients],
                     [cl.scene.width for cl in clients], [cl.scene.background for cl in clients],
                     heights=[cl.scene.height for cl in clients])
    assert ex.value.status == abi.ERR_OVER_BUDGET
    ctx.close()
    # a server whose estimates admit whole batches: the library's refusal splits them
    resident = sum(cl.comp.device_bytes() + cl.pool_comp.device_bytes() for cl in clients)
    for cl in clients:
        cl.est_bytes = 1
    srv = serving.Server(clients, mode="batched", workers=1, max_batch=4, hbm_budget=resident + share)
    assert srv.ctx_budget == share
    reqs = serving.poisson_arrivals(rate=2000.0, n_clients=len(clients), duration=0.02, seed=3)
    srv.run(reqs)
    assert srv.refused_batches > 0
    assert srv.ctx[0].device_bytes() <= share
    for k, cl in enumerate(clients):
        assert torch.equal(cl.out, _alone(cl)), f"client {k}: mix != alone"


def test_added_layers_copy_pool_lines(gpu_lib):
    """insert_layer_copies gives the same lines, segments and pixels as
    inserting (and flattening) the same paths."""
    from cassia_gb300 import Composition, scenes
    pool = scenes.mixed(seed=45, n_layers=64, width=256, height=256)
    src = Composition()
    src.create_layers(pool.n_layers)
    src.insert_paths(pool)
    picks = np.array([5, 0, 63, 17, 17, 40], np.uint32)
    a, b = Composition(), Composition()
    ids_a = a.create_layers(len(picks))
    ids_b = b.create_layers(len(picks))
    a.insert_layer_copies(ids_a, src, picks)
    co = np.diff(pool.cmd_offsets)[picks]
    po = np.diff(pool.point_offsets)[picks]
    sub = scenes.Scene("sub", pool.width, pool.height, pool.background, False, len(picks), ids_b,
                       np.concatenate([[0], np.cumsum(co)]).astype(np.uint64),
                       np.concatenate([pool.kinds[pool.cmd_offsets[p]:pool.cmd_offsets[p + 1]] for p in picks]),
                       np.concatenate([[0], np.cumsum(po)]).astype(np.uint64),
                       np.concatenate([pool.points[pool.point_offsets[p]:pool.point_offsets[p + 1]] for p in picks]))
    b.insert_paths(sub)
    for c, ids in ((a, ids_a), (b, ids_b)):
        c.set_layers_solid(ids, pool.fill_rule[picks], pool.blend_mode[picks], pool.color[picks])
        c.set_transforms(ids, pool.transforms[picks])
    assert a.lens() == b.lens()
    sa, na = a.pixel_segments()
    sb, nb = b.pixel_segments()
    assert na == nb and np.array_equal(sa, sb)
    ia = np.zeros((256, 256, 4), np.uint8)
    ib = np.zeros_like(ia)
    a.render(ia, 256, (1.0, 1.0, 1.0, 1.0))
    b.render(ib, 256, (1.0, 1.0, 1.0, 1.0))
    assert np.array_equal(ia, ib)
    # a layer whose lines are no longer one run is refused as a source
    a.insert_layer_copies(ids_a[:1], src, picks[:1])
    with pytest.raises(Exception):
        b.insert_layer_copies(ids_b[:1], a, ids_a[:1])


def test_update_layers_equals_separate_calls(gpu_lib):
    """cgb_update_layers applies each composition's transforms, removals
    (with remove_disabled) and added copies exactly as the separate calls
    do: same new ids, same lines, same pixels."""
    from cassia_gb300 import Composition, scenes
    from cassia_gb300.composition import solid_props, update_layers
    sc = scenes.mixed(seed=46, n_layers=120, width=256, height=192)
    pool = scenes.mixed(seed=47, n_layers=32, width=256, height=192)
    src = Composition()
    src.create_layers(pool.n_layers)
    src.insert_paths(pool)
    a, b = Composition(), Composition()
    for c in (a, b):
        scenes.load(sc, c)
    rng = np.random.default_rng(48)
    live = np.arange(sc.n_layers, dtype=np.uint32)
    for step in range(3):
        pick = rng.permutation(len(live))
        ids = np.sort(live[pick[:25]])
        gone = np.sort(live[pick[25:31 + 20 * step]])
        t = np.tile(np.array([[1.0, 0.0, 0.0, 1.0, 0.0, 0.0]], np.float32), (len(ids), 1))
        t[:, 0] = t[:, 3] = rng.uniform(0.8, 1.2, len(ids)).astype(np.float32)
        t[:, 4:] = rng.uniform(-20, 20, (len(ids), 2)).astype(np.float32)
        picks = rng.integers(0, pool.n_layers, len(gone)).astype(np.uint32)
        props = solid_props(pool.fill_rule[picks], pool.blend_mode[picks], pool.color[picks])
        new_a = update_layers([{"comp": a, "transform_ids": ids, "transforms": t, "removed_ids": gone,
                                "added_from": src, "added_from_ids": picks, "added_props": props,
                                "added_transforms": pool.transforms[picks]}])[0]
        b.set_transforms(ids, t)
        b.set_enabled_many(gone, np.zeros(len(gone), np.uint8))
        b.remove_disabled()
        new_b = b.create_layers(len(gone))
        b.insert_layer_copies(new_b, src, picks)
        b.set_layers_solid(new_b, pool.fill_rule[picks], pool.blend_mode[picks], pool.color[picks])
        b.set_transforms(new_b, pool.transforms[picks])
        live = np.concatenate([np.setdiff1d(live, gone), new_b]).astype(np.uint32)
        assert np.array_equal(new_a, new_b)
        assert a.lens() == b.lens()
        ia = np.zeros((sc.height, sc.width, 4), np.uint8)
        ib = np.zeros_like(ia)
        a.render(ia, sc.width, sc.background)
        b.render(ib, sc.width, sc.background)
        assert np.array_equal(ia, ib), f"step {step}"


def test_copies_refused_after_compaction(gpu_lib):
    """remove_disabled's garbage collection moves the kept lines, after which
    a source layer's lines are no longer known to be one run."""
    from cassia_gb300 import Composition, abi, scenes
    pool = scenes.mixed(seed=49, n_layers=20, width=128, height=128)
    src = Composition()
    src.create_layers(pool.n_layers)
    src.insert_paths(pool)
    dst = Composition()
    ids = dst.create_layers(2)
    last = np.array([pool.n_layers - 1], np.uint32)
    dst.insert_layer_copies(ids[:1], src, last)  # one run: accepted
    before = src.lens()[0]
    src.set_enabled_many(np.arange(pool.n_layers - 1, dtype=np.uint32), np.zeros(pool.n_layers - 1, np.uint8))
    src.remove_disabled()  # more than half the lines are garbage: compaction
    assert src.lens()[0] < before
    with pytest.raises(abi.CassiaError) as ex:
        dst.insert_layer_copies(ids[1:], src, last)
    assert ex.value.status == abi.ERR_INVALID_ARG
