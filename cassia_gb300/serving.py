"""A render server with continuous batching over resident compositions.

Each client owns a Composition whose lines, layer table and styles stay
resident on the GPU between frames.  A request asks for a client's next
frame after a seeded update of its scene (new affine transforms for a share
of its layers, a few layers added or removed).  Worker threads form batches
of ready requests -- at most one per client, oldest first, admitted while the
estimated device memory of the batch fits the HBM budget -- and render each
batch in one pipeline (cgb_render_batch) on the worker's own stream, so a
batch that arrives while another is on the GPU overlaps it on the device.

The reference renders one Composition per call and has no server
(mold/src/composition.rs:212-329); this module is the serving pattern built
on the batched pipeline.  `mode="plain"` serves the same requests one render
call at a time for comparison.
"""
import collections
import threading
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import scenes
from .composition import Composition, render_batch, solid_props, update_layers


@dataclass
class Request:
    client: int
    seq: int
    arrival: float  # seconds after the start of the run
    t_start: float = 0.0
    t_render: float = 0.0  # render call start (after the scene update)
    t_done: float = 0.0
    batch_size: int = 0


@dataclass
class Client:
    comp: Composition
    scene: scenes.Scene
    out: object                 # device RGBA8 tensor (torch) or host numpy array
    enabled: np.ndarray         # bool per layer id
    transforms: np.ndarray      # float32 [n, 6]
    est_bytes: int = 0          # estimated frame scratch of the last frame
    done_seq: int = -1
    pool: Optional[scenes.Scene] = None  # shapes new layers are drawn from
    pool_next: int = 0
    pool_comp: Optional[Composition] = None  # the pool's shapes flattened once, layer k = shape k


def poisson_arrivals(rate: float, n_clients: int, duration: float, seed: int = 0) -> List[Request]:
    """Poisson arrivals at `rate` requests/s over `duration` seconds, each for a
    uniformly chosen client; per-client sequence numbers in arrival order."""
    rng = np.random.default_rng(seed)
    t, out, seq = 0.0, [], collections.Counter()
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        c = int(rng.integers(n_clients))
        out.append(Request(c, seq[c], t))
        seq[c] += 1
    return out


def make_clients(n_clients: int, seed: int, device_out: bool = True, max_layers: int = 50_000,
                 incremental: bool = False):
    """Clients with compositions drawn from the batched-workload distribution.
    incremental: each composition keeps its last frame's sorted segments on
    the device and re-rasterizes only the layers an update changed."""
    import torch
    sset = scenes.batch(seed=seed, n_scenes=n_clients, max_layers=max_layers)
    clients = []
    for k, sc in enumerate(sset):
        # churn needs fresh layer ids until the lines garbage collection of
        # remove_disabled frees the removed ones (at 50% garbage): large
        # clients use the widened 17-bit layer format
        c = Composition(wide=sc.wide or sc.n_layers > 30_000, priority="high")
        scenes.load(sc, c)
        if incremental:
            c.set_incremental(True)
        if device_out:
            out = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
        else:
            out = np.zeros((sc.height, sc.width, 4), np.uint8)
        pool = scenes.mixed(seed=seed * 7919 + k, n_layers=256, width=sc.width, height=sc.height)
        # the pool's shapes flattened once on the device: an added layer takes
        # a copy of its shape's lines instead of flattening the path again
        pool_comp = Composition()
        pool_comp.create_layers(pool.n_layers)
        pool_comp.insert_paths(pool)
        clients.append(Client(c, sc, out, np.ones(sc.n_layers, bool), sc.transforms.copy(), pool=pool,
                              pool_comp=pool_comp))
    return clients


def _mix64(ids: np.ndarray, salt) -> np.ndarray:
    """splitmix64 of each id and a salt (a scalar or one per id), vectorized
    (array integer arithmetic wraps silently)."""
    salt = np.asarray(salt, np.uint64) if np.ndim(salt) else np.uint64(salt & 0xFFFFFFFFFFFFFFFF)
    z = ids.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15) + salt
    z ^= z >> np.uint64(30)
    z *= np.uint64(0xBF58476D1CE4E5B9)
    z ^= z >> np.uint64(27)
    z *= np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(31)
    return z


def _bits01(z: np.ndarray, shift: int, bits: int) -> np.ndarray:
    """Uniform [0, 1) from `bits` bits of z starting at `shift`."""
    return ((z >> np.uint64(shift)) & np.uint64((1 << bits) - 1)).astype(np.float64) * (1.0 / (1 << bits))


def _u01(ids: np.ndarray, salt: int) -> np.ndarray:
    """Seeded uniform [0, 1) per id (splitmix64 of id and salt)."""
    return _bits01(_mix64(ids, salt), 11, 53)


def _salt(client_id: int, seq: int) -> int:
    return ((client_id << 40) ^ (seq * 0x9E3779B1)) & 0xFFFFFFFFFFFFFFFF


def apply_update(cl: Client, client_id: int, seq: int, changed: float = 0.2, churn: float = 0.01):
    """The scene update of frame `seq` of one client (apply_updates of one)."""
    apply_updates([(cl, client_id, seq)], changed, churn)


def apply_updates(items, changed: float = 0.2, churn: float = 0.01):
    """The scene updates of a batch, one (client, client id, frame seq) per
    distinct client: each enabled layer gets a new affine with probability
    `changed` and is removed with probability `churn` (seeded per client and
    frame); as many layers as were removed are added.  The random draws of
    the whole batch are made by a few array operations over all its clients
    (integer hashing and IEEE float32 arithmetic only, so each client's
    update is the same whether it is drawn alone or in a batch); then each
    client's calls are made."""
    assert len({id(cl) for cl, _, _ in items}) == len(items), "one update per client"
    lives = [np.flatnonzero(cl.enabled).astype(np.uint32) for cl, _, _ in items]
    items = [it for it, live in zip(items, lives) if len(live)]
    lives = [live for live in lives if len(live)]
    if not items:
        return
    lens = np.array([len(x) for x in lives])
    salts = np.array([_salt(cid, seq) for _, cid, seq in items], np.uint64)
    # one hash per live layer: 24 bits decide the new affine, 24 others the removal
    z = _mix64(np.concatenate(lives), np.repeat(salts, lens))
    chg = _bits01(z, 40, 24) < changed
    rem = _bits01(z, 16, 24) < churn
    offs = np.concatenate([[0], np.cumsum(lens)])
    ids = []
    for k, live in enumerate(lives):
        sel = live[chg[offs[k]:offs[k + 1]]]
        ids.append(sel if len(sel) else live[:1])
    # one hash per changed layer: a rotation by 2 atan(u), u U[-0.025, 0.025),
    # as the rational (1 - u^2, 2u) / (1 + u^2), and a shift U[-3, 3)^2
    nid = np.array([len(x) for x in ids])
    w = _mix64(np.concatenate(ids), np.repeat(salts ^ np.uint64(0x2545F4914F6CDD1D), nid))
    u = ((_bits01(w, 42, 21) - 0.5) * 0.05).astype(np.float32)
    uu = u * u
    den = np.float32(1.0) + uu
    c = (np.float32(1.0) - uu) / den
    s = (np.float32(2.0) * u) / den
    t = np.concatenate([cl.transforms[x] for (cl, _, _), x in zip(items, ids)])
    a, b, cc, d = t[:, 0].copy(), t[:, 1].copy(), t[:, 2].copy(), t[:, 3].copy()
    t[:, 0], t[:, 1] = c * a - s * cc, c * b - s * d
    t[:, 2], t[:, 3] = s * a + c * cc, s * b + c * d
    t[:, 4] += ((_bits01(w, 21, 21) - 0.5) * 6.0).astype(np.float32)
    t[:, 5] += ((_bits01(w, 0, 21) - 0.5) * 6.0).astype(np.float32)
    toff = np.concatenate([[0], np.cumsum(nid)])
    batch = []  # clients whose calls go to the library in one cgb_update_layers
    for k, (cl, _, _) in enumerate(items):
        tk = t[toff[k]:toff[k + 1]]
        cl.transforms[ids[k]] = tk
        gone = lives[k][rem[offs[k]:offs[k + 1]]]
        if cl.pool_comp is not None and isinstance(cl.comp, Composition):
            u = {"comp": cl.comp, "transform_ids": ids[k], "transforms": tk}
            if len(gone):
                cl.enabled[gone] = False
                picks = _pool_picks(cl, len(gone))
                p = cl.pool
                u.update(removed_ids=gone, added_from=cl.pool_comp, added_from_ids=picks.astype(np.uint32),
                         added_props=solid_props(p.fill_rule[picks], p.blend_mode[picks], p.color[picks]),
                         added_transforms=p.transforms[picks])
            batch.append((cl, u))
            continue
        cl.comp.set_transforms(ids[k], tk)
        if len(gone):
            cl.comp.set_enabled_many(gone, np.zeros(len(gone), np.uint8))
            cl.enabled[gone] = False
            cl.comp.remove_disabled()  # mold's GC: drops the disabled layers at 50% garbage
            add_layers(cl, len(gone))
    if batch:
        # the same calls in the same order, in one library call for the batch
        for (cl, u), new_ids in zip(batch, update_layers([u for _, u in batch])):
            if len(new_ids):
                _note_added(cl, new_ids, u["added_from_ids"])


def _pool_runs(start: int, n: int, size: int):
    """[a, b) runs of pool indices start, start + 1, ... (n of them, mod size)."""
    runs, a = [], start % size
    while n > 0:
        b = min(size, a + n)
        runs.append((a, b))
        n -= b - a
        a = 0
    return runs


def _pool_picks(cl: Client, n: int) -> np.ndarray:
    """The next n shapes of the client's pool (taken in turn)."""
    runs = _pool_runs(cl.pool_next, n, cl.pool.n_layers)
    cl.pool_next += n
    return np.concatenate([np.arange(a, b) for a, b in runs])


def add_layers(cl: Client, n: int):
    """Adds n layers drawn in turn from the client's shape pool (one path
    per pool layer), with one insert call: copies of the shapes' lines from
    the pool's composition when the client has one, else the paths (the
    same lines: the flattening is deterministic)."""
    p = cl.pool
    ids = cl.comp.create_layers(n)
    picks = _pool_picks(cl, n)
    if cl.pool_comp is not None:
        cl.comp.insert_layer_copies(ids, cl.pool_comp, picks.astype(np.uint32))
    else:
        _insert_pool_paths(cl, ids, picks)
    cl.comp.set_layers_solid(ids, p.fill_rule[picks], p.blend_mode[picks], p.color[picks])
    cl.comp.set_transforms(ids, p.transforms[picks])
    _note_added(cl, ids, picks)


def _note_added(cl: Client, ids, picks):
    """The client's mirror of its new layers: enabled, with their transforms."""
    p = cl.pool
    top = int(ids.max()) + 1
    if top > len(cl.enabled):
        grow = top - len(cl.enabled)
        cl.enabled = np.concatenate([cl.enabled, np.zeros(grow, bool)])
        cl.transforms = np.concatenate([cl.transforms, np.zeros((grow, 6), np.float32)])
    cl.enabled[ids] = True
    cl.transforms[ids] = p.transforms[picks]


def _insert_pool_paths(cl: Client, ids, picks):
    p = cl.pool
    kinds = [p.kinds[int(p.cmd_offsets[k]):int(p.cmd_offsets[k + 1])] for k in picks]
    pts = [p.points[int(p.point_offsets[k]):int(p.point_offsets[k + 1])] for k in picks]
    co = np.concatenate([[0], np.cumsum(np.diff(p.cmd_offsets)[picks])]).astype(np.uint64)
    po = np.concatenate([[0], np.cumsum(np.diff(p.point_offsets)[picks])]).astype(np.uint64)
    sub = scenes.Scene("add", p.width, p.height, p.background, p.wide, len(ids), ids, co,
                       np.concatenate(kinds).astype(np.uint32), po, np.concatenate(pts).astype(np.float32))
    cl.comp.insert_paths(sub)


def frame_bytes(st: dict) -> int:
    """Device scratch a frame of this size holds (segments, groups, items)."""
    return int(16 * st.get("segments", 0) + 36 * st.get("tile_layers", 0) + 16 * st.get("work_items", 0) +
               40 * st.get("lines", 0))


class Server:
    """The HBM budget covers the clients' resident device memory (their lines,
    layer tables and resident segments) and the frame buffers of the batches
    in flight.  What the clients hold when the server starts is set aside;
    each worker's batch context gets an equal share of the rest as its
    library budget, so the library refuses (CGB_ERR_OVER_BUDGET) a batch
    whose frame would not fit: the worker then renders the batch in halves,
    and a single request that fits no share on the client's own handle
    (counted in `refused_alone`).  Requests are first admitted by an estimate
    of their frame size, kept current from the sizes of the frames rendered."""

    def __init__(self, clients: List[Client], mode: str = "batched", workers: int = 2, max_batch: int = 16,
                 hbm_budget: float = 40e9):
        assert mode in ("batched", "plain")
        self.clients = clients
        self.mode = mode
        self.workers = 1 if mode == "plain" else workers
        self.max_batch = 1 if mode == "plain" else max_batch
        self.budget = hbm_budget
        resident = sum(cl.comp.device_bytes() + (cl.pool_comp.device_bytes() if cl.pool_comp else 0)
                       for cl in clients)
        # at least what a handle holds when it is created (a budget of 0
        # would mean "unlimited" to the library)
        self.ctx_budget = max(1 << 20, int((hbm_budget - resident) // self.workers))
        # batch renders run at low priority so that the clients' small update
        # kernels are not queued behind them
        self.ctx = ([Composition(priority="low", hbm_budget=self.ctx_budget) for _ in range(self.workers)]
                    if mode == "batched" else [])
        self.refused_batches = 0  # batches the library refused for the budget (then split)
        self.refused_alone = 0    # single requests rendered on their own handle
        self.cv = threading.Condition()
        self.pending: Dict[int, collections.deque] = collections.defaultdict(collections.deque)
        self.busy = set()
        self.inflight_bytes = 0
        self.errors: List[BaseException] = []

    def _ready_batch(self, now):
        """Oldest-first ready requests, one per idle client, within the budget."""
        heads = [(q[0].arrival, c) for c, q in self.pending.items() if q and c not in self.busy and q[0].arrival <= now]
        heads.sort()
        batch, mem = [], 0
        for _, c in heads:
            est = max(self.clients[c].est_bytes, 1 << 20)
            # admit while the batch fits beside the batches in flight; a
            # request that fits nowhere runs alone once nothing is in flight
            if self.inflight_bytes + mem + est > self.budget and (batch or self.inflight_bytes > 0):
                continue
            batch.append(self.pending[c].popleft())
            mem += est
            if len(batch) >= self.max_batch:
                break
        return batch, mem

    def _worker(self, wid, t0, total):
        while True:
            with self.cv:
                while True:
                    if self.completed >= total or self.errors:
                        return
                    now = time.perf_counter() - t0
                    batch, mem = self._ready_batch(now)
                    if batch:
                        for r in batch:
                            self.busy.add(r.client)
                        self.inflight_bytes += mem
                        break
                    # arrivals and finished batches notify; the timeout is a safety net
                    self.cv.wait(timeout=0.05)
            try:
                ts = time.perf_counter() - t0
                for r in batch:
                    r.t_start = ts
                apply_updates([(self.clients[r.client], r.client, r.seq) for r in batch])
                tr = time.perf_counter() - t0
                for r in batch:
                    r.t_render = tr
                if self.mode == "plain":
                    r = batch[0]
                    cl = self.clients[r.client]
                    _render_one(cl)
                else:
                    cls = [self.clients[r.client] for r in batch]
                    self._render_within_budget(self.ctx[wid], cls)
                td = time.perf_counter() - t0
                for r in batch:
                    r.t_done = td
                    r.batch_size = len(batch)
                    cl = self.clients[r.client]
                    cl.done_seq = r.seq
                    if self.mode == "plain":
                        cl.est_bytes = frame_bytes(cl.comp.stats())
            except BaseException as e:  # surface to the caller
                with self.cv:
                    self.errors.append(e)
                    self.cv.notify_all()
                return
            with self.cv:
                for r in batch:
                    self.busy.discard(r.client)
                self.inflight_bytes -= mem
                self.completed += len(batch)
                self.cv.notify_all()

    def _render_within_budget(self, ctx: Composition, cls: List[Client]):
        """Renders a batch on `ctx`; a batch the library refuses for the
        budget is rendered in halves, a single client on its own handle."""
        from .abi import ERR_OVER_BUDGET, CassiaError
        try:
            _render_many(ctx, cls)
        except CassiaError as e:
            if e.status != ERR_OVER_BUDGET:
                raise
            with self.cv:
                self.refused_batches += 1
            if len(cls) == 1:
                with self.cv:
                    self.refused_alone += 1
                _render_one(cls[0])
                return
            h = len(cls) // 2
            self._render_within_budget(ctx, cls[:h])
            self._render_within_budget(ctx, cls[h:])
            return
        # size estimates from this frame: its buffers per line, times each client's lines
        st = ctx.stats()
        if st.get("lines", 0) > 0:
            per_line = frame_bytes(st) / st["lines"]
            for cl in cls:
                cl.est_bytes = int(per_line * cl.comp.lens()[0])

    def run(self, requests: List[Request]) -> List[Request]:
        """Serves `requests` (sorted by arrival) in real time; returns them
        with start / completion times filled in."""
        self._requests = requests
        self._cursor = 0
        self.completed = 0
        for cl in self.clients:  # size estimates from one frame each
            if cl.est_bytes == 0:
                _render_one(cl)
                cl.est_bytes = frame_bytes(cl.comp.stats())
        t0 = time.perf_counter()
        threads = [threading.Thread(target=self._worker, args=(w, t0, len(requests)), daemon=True)
                   for w in range(self.workers)]
        for th in threads:
            th.start()
        # feed arrivals in real time
        while self._cursor < len(requests):
            now = time.perf_counter() - t0
            with self.cv:
                fed = 0
                while self._cursor < len(requests) and requests[self._cursor].arrival <= now:
                    r = requests[self._cursor]
                    self.pending[r.client].append(r)
                    self._cursor += 1
                    fed += 1
                if fed:  # wake the workers only when there is new work
                    self.cv.notify_all()
                if self.errors:
                    break
            if self._cursor < len(requests):
                time.sleep(max(0.0, min(0.001, requests[self._cursor].arrival - now)))
        for th in threads:
            th.join()
        if self.errors:
            raise self.errors[0]
        return requests


def _render_one(cl: Client):
    sc = cl.scene
    if isinstance(cl.out, np.ndarray):
        cl.comp.render(cl.out, sc.width, sc.background)
    else:
        cl.comp.render(cl.out.data_ptr(), sc.width, sc.background, height=sc.height)


def _render_many(ctx: Composition, cls: List[Client]):
    outs = [cl.out if isinstance(cl.out, np.ndarray) else cl.out.data_ptr() for cl in cls]
    render_batch(ctx, [cl.comp for cl in cls], outs, [cl.scene.width for cl in cls],
                 [cl.scene.background for cl in cls], heights=[cl.scene.height for cl in cls])


def latency_summary(reqs: List[Request], duration: float) -> dict:
    lat = np.array([r.t_done - r.arrival for r in reqs]) * 1e3
    span = max(r.t_done for r in reqs) - min(r.arrival for r in reqs)
    render = np.array([r.t_done - r.t_render for r in reqs]) * 1e3
    update = np.array([r.t_render - r.t_start for r in reqs]) * 1e3
    return {"requests": len(reqs), "frames_per_s": len(reqs) / span, "p50_ms": float(np.percentile(lat, 50)),
            "render_call_ms_mean": float(render.mean()), "update_ms_mean": float(update.mean()),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "mean_batch": float(np.mean([r.batch_size for r in reqs])), "offered_s": duration}
