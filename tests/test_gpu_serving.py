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
