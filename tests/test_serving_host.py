"""The serving loop's host logic without a GPU: the seeded scene updates of a
batch are the same as the same updates drawn one client at a time (the
server draws a batch's updates together; the oracle replays them one by
one)."""
import numpy as np

from cassia_gb300 import serving


class _Calls:
    """Records the library calls of an update in place of a composition."""

    def __init__(self):
        self.log = []

    def set_transforms(self, ids, t):
        self.log.append(("t", np.array(ids).tolist(), np.array(t).tobytes()))

    def set_enabled_many(self, ids, en):
        self.log.append(("e", np.array(ids).tolist()))

    def remove_disabled(self):
        self.log.append(("gc",))


def _client(n, seed):
    rng = np.random.default_rng(seed)
    return serving.Client(_Calls(), None, None, np.ones(n, bool), rng.standard_normal((n, 6)).astype(np.float32))


def test_batched_updates_equal_one_at_a_time(monkeypatch):
    added = []
    monkeypatch.setattr(serving, "add_layers", lambda cl, n: added.append((id(cl), n)))
    sizes = [1, 10, 500, 3000, 77, 40_000]
    a = [_client(n, k) for k, n in enumerate(sizes)]
    b = [_client(n, k) for k, n in enumerate(sizes)]
    for seq in range(3):
        serving.apply_updates([(cl, k, seq) for k, cl in enumerate(a)])
        for k, cl in enumerate(b):
            serving.apply_update(cl, k, seq)
    for x, y in zip(a, b):
        assert np.array_equal(x.transforms, y.transforms)
        assert np.array_equal(x.enabled, y.enabled)
        assert x.comp.log == y.comp.log
    # about 20% of the layers change per frame and 1% are removed
    big = a[-1]
    assert 0.18 < len(big.comp.log[0][1]) / 40_000 < 0.22
    assert 0.5 < (40_000 - big.enabled.sum()) / (3 * 400) < 1.5
    assert sum(n for _, n in added) > 0


def test_update_rotation_is_a_rotation():
    cl = _client(2000, 9)
    cl.transforms[:] = np.array([1, 0, 0, 1, 0, 0], np.float32)
    serving.apply_updates([(cl, 3, 0)], churn=0.0)
    t = cl.transforms[cl.transforms[:, 1] != 0]
    det = t[:, 0] * t[:, 3] - t[:, 1] * t[:, 2]
    assert len(t) > 300 and np.allclose(det, 1.0, atol=1e-6)
    assert np.all(np.abs(t[:, 1]) < 0.051)
