#!/usr/bin/env python3
"""Benchmark: Msegments/s of the surpass/mold rasterize -> sort -> paint frame.

Workload (default): the mixed 100,000-layer scene on a 2560x1600 canvas
(star/convex polygons and closed cubic paths, random affine per layer, 12
blend modes, NonZero/EvenOdd; ~7.6M lines, ~65M pixel segments), seeded and
synthetic.  Lines are flattened once on the GPU and stay resident in HBM; one
step is one frame: LinesBuilder::build -> rasterize -> sort -> paint into an
RGBA8 device buffer.  value = pixel segments / second over all ranks.  By
default frames are replayed from a captured CUDA graph (the library's graph
mode: counts stay on the device); --frame-mode staged enqueues each stage and
reads the counts back between stages.

The default run (mixed100k) then measures the batched form (the 256-scene
batch workload: one pipeline per group of scenes against one render call per
scene) and the served form (64 clients, Poisson arrivals, continuous batching
against one full render per request) and reports them as the "batched" and
"served" sub-objects of the same JSON line (--no-forms skips them).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--frame-mode staged|graph]

--impl reference times the CPU restatement of the reference path (the
oracle, std::thread-parallel over the host cores) on the same workload,
each step a bounded sample of it.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "mixed100k": dict(kind="mixed", n_layers=100_000, width=2560, height=1600, seed=2),
    "mixed65k": dict(kind="mixed", n_layers=65_535, width=2560, height=1600, seed=2),
    "mixed20k": dict(kind="mixed", n_layers=20_000, width=2560, height=1600, seed=2),
    "circles": dict(kind="circles", n_layers=1000, width=1024, height=1024, seed=1),
    "glyphs": dict(kind="glyphs", n_layers=50_000, width=3840, height=2160, seed=3),
    "batch256": dict(kind="batch", n_scenes=256, seed=4),
    "serve": dict(kind="serve", n_clients=64, rate=2000.0, duration=3.0, seed=5),
}


def make_scene(name):
    from cassia_gb300 import scenes
    w = WORKLOADS[name]
    if w["kind"] == "batch":
        raise ValueError("the batch workload has no single scene")
    if w["kind"] == "mixed":
        return scenes.mixed(seed=w["seed"], n_layers=w["n_layers"], width=w["width"], height=w["height"])
    if w["kind"] == "circles":
        return scenes.circles(seed=w["seed"], n_layers=w["n_layers"], size=w["width"])
    return scenes.glyphs(seed=w["seed"], n_layers=w["n_layers"], width=w["width"], height=w["height"])


def measure_frames(name, steps, warmup, local):
    """Device time per frame of one seeded scene, replayed from its frame
    graph (CUDA events on the library's stream), with its counts and stage
    times: the single-frame configurations beside the headline one."""
    import torch
    from cassia_gb300 import Composition, scenes
    scene = make_scene(name)
    comp = Composition(wide=scene.wide)
    scenes.load(scene, comp)
    ref_segments, _ = comp.count_segments()
    comp.set_graph_mode(True)
    H, W = scene.height, scene.width
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.ExternalStream(comp.stream())
    for _ in range(warmup):
        comp.render(out.data_ptr(), W, scene.background, height=H)
    comp.synchronize()
    torch.cuda.synchronize()
    stats = []
    with ClockSampler(local) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            comp.render(out.data_ptr(), W, scene.background, height=H)
            stats.append(comp.stats())
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    st = stats[-1]
    comp.close()
    config = scene_config(name, scene, 1)
    # line records and the sorted segment arrays against the 129 MB L2
    if st["lines"] * 52 + st["painted_segments"] * 16 < 129e6:
        config["l2"] = "inputs within L2 (not flushed between frames)"
    return {"metric": "Msegments/s", "value": ref_segments / (ms / 1e3) / 1e6, "unit": "Msegments/s",
            "ms_per_step": ms, "steps": steps, "warmup": warmup, "config": config,
            "frame_counts": {"lines": st["lines"], "segments_per_frame": ref_segments,
                             "painted_segments": st["painted_segments"], "tile_layers": st["tile_layers"],
                             "work_items": st["work_items"]},
            "stage_ms": {k: statistics.mean(x[k + "_ms"] for x in stats) for k in
                         ("build", "rasterize", "sort", "carry", "paint", "total")},
            "sort_passes": int(st["sort_passes"]), "sort_passes_skipped": int(st["sort_passes_skipped"]),
            "graph_replayed": int(st["graph_replayed"]), "clocks": clk.summary()}


def over_ranks(x, op="max"):
    """x reduced over the replicas of a multi-process run ("max" for times,
    "sum" for counts); x itself without a process group.  NCCL groups reduce
    on the current CUDA device, gloo groups on the host."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []  # (time, line)
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is producing samples
            deadline = time.time() + 3.0
            while not self.lines and time.time() < deadline:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        self.t0 = time.time()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def __exit__(self, *a):
        self.t1 = time.time()
        if self.proc:
            time.sleep(0.12)  # the sample in flight when the region ended
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        """Median SM clock and the throttle reasons of the samples taken
        inside the timed region (and the one that was in flight at its end)."""
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0 = self.t0 if self.t0 is not None else 0.0
        t1 = (self.t1 if self.t1 is not None else time.time()) + 0.11
        for t, ln in self.lines:
            if t < t0 or t > t1:
                continue
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def stage_bytes(st, scene):
    """Algorithmic bytes per stage: each stage reads its input once and
    writes its output once; one sort pass is one read + one write; the
    painter reads each segment, work item and tile-layer record (first
    segment, cover, carry) once, each layer style once and writes the frame."""
    L, P, N = st["lines"], st["segments"], scene.n_layers  # rasterized segments
    return {
        "rasterize": 18 * L + 8 * P,
        "sort": 16 * st["painted_segments"],
        "paint": (8 * st["painted_segments"] + 8 * st["work_items"] + 20 * st["tile_layers"] + 32 * N +
                  4 * scene.width * scene.height),
    }


def read_traffic(workload, stage):
    """DRAM bytes per launch of the stage's dominant kernel from the table in
    profiles/traffic.md (one ncu capture), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) == 5 and cells[0] == workload and cells[1] == stage:
                try:
                    return int(cells[3])
                except ValueError:
                    return None
    return None


STAGE_KERNELS = {
    "build": "k_build_lines + scan",
    "rasterize": "k_rasterize + k_gather_hist",
    "sort": "k_onesweep (one launch per digit pass)",
    "carry": "k_tl_scan + k_tl_carry + k_items_* + item sort",
    "paint": "k_paint",
}

# What bounds each stage's dominant kernel, from the ncu captures summarised
# in profiles/kernels_mixed20k.md.
STAGE_LIMITERS = {
    "rasterize": "fixed-point step arithmetic (70% issue active) and the latency of its line loads",
    "sort": "instruction issue of the onesweep tile's ranking and scatter (53-57% issue active, "
            "2.3 TB/s per pass)",
    "paint": "instruction issue and dependent-instruction latency (74% of issue slots, fixed-latency "
             "waits the top stall; not occupancy: more resident warps did not help); its DRAM traffic "
             "equals its algorithmic input",
}


def cpu_reference(scene, steps, warmup, budget_s=150.0):
    """Times the oracle's full frame (build, rasterize, sort, paint) on the
    host cores.  Each step renders a bounded sample: the first fraction of the
    scene's layers, sized so that all steps fit the time budget."""
    import oracle
    from cassia_gb300 import scenes as sc_mod
    threads = os.cpu_count() or 1

    def sub_scene(frac):
        n = max(1, int(scene.n_layers * frac))
        k = int(np.searchsorted(scene.path_layer, n))
        s = sc_mod.Scene(scene.name, scene.width, scene.height, scene.background, scene.wide, n,
                         scene.path_layer[:k], scene.cmd_offsets[:k + 1], scene.kinds[:int(scene.cmd_offsets[k])],
                         scene.point_offsets[:k + 1], scene.points[:int(scene.point_offsets[k])],
                         None if scene.transforms is None else scene.transforms[:n], scene.fill_rule[:n],
                         scene.blend_mode[:n], scene.color[:n])
        return s

    def frame(s, comp, img):
        t0 = time.perf_counter()
        comp.render(img, s.width, s.background, threads=threads)
        dt = time.perf_counter() - t0
        return dt, comp.stats()["segments"]

    img = np.zeros((scene.height, scene.width, 4), np.uint8)
    # calibrate on 5% of the layers
    s = sub_scene(0.05)
    comp = oracle.Composition(wide=scene.wide)
    sc_mod.load(s, comp)
    dt, _ = frame(s, comp, img)
    per_step = budget_s / max(1, steps + warmup)
    frac = min(1.0, 0.05 * per_step / max(dt, 1e-3))
    if frac < 1.0:
        s = sub_scene(frac)
    else:
        s = scene
    comp = oracle.Composition(wide=scene.wide)
    sc_mod.load(s, comp)
    for _ in range(warmup):
        frame(s, comp, img)
    times, segs = [], 0
    for _ in range(steps):
        dt, segs = frame(s, comp, img)
        times.append(dt)
    t = sum(times) / len(times)
    sample = (f"{s.n_layers} of {scene.n_layers} layers ({100.0 * s.n_layers / scene.n_layers:.1f}%), "
              f"full {scene.width}x{scene.height} canvas, {segs} segments per frame")
    return {"value": segs / t / 1e6, "unit": "Msegments/s", "cores": threads, "kind": "port", "sample": sample,
            "ms_per_step": t * 1e3, "frames_per_s": 1.0 / t}


def _bits(v):
    """Bits that hold values in [0, v] (at least 1)."""
    return max(1, int(v).bit_length())


def group_scenes(comps, sset, line_budget=16_000_000, key_bits=36):
    """Consecutive scenes whose lines fit one frame's budget and whose
    batched segment key -- the tile rows of all of them, the largest order,
    the widest tile row -- stays within key_bits (4 radix passes of 9 bits;
    one more bit would cost a fifth pass over every segment of the group)."""
    groups, cur, lines, rows, orders, cols = [], [], 0, 0, 1, 1
    for k, (c, sc) in enumerate(zip(comps, sset)):
        n = c.lens()[0]
        r, cl, o = (sc.height + 7) // 8, (sc.width + 7) // 8, max(1, sc.n_layers)
        nrows, nord, ncol = rows + r, max(orders, o), max(cols, cl)
        if cur and (lines + n > line_budget or _bits(nrows - 1) + _bits(nord - 1) + _bits(ncol) > key_bits):
            groups.append(cur)
            cur, lines = [], 0
            nrows, nord, ncol = r, o, cl
        cur.append(k)
        lines += n
        rows, orders, cols = nrows, nord, ncol
    if cur:
        groups.append(cur)
    return groups


def run_batch(args, rank, world, local):
    """Batched workload: 256 independent scenes (layer count log-U[10, 50,000],
    canvas side in {256, 512, 1024, 2048}).  Batched = the scenes rendered
    together, a few pipelines per pass (grouped by a line budget), the groups
    on --batch-streams contexts at once; plain = one render call per scene.
    Outputs are compared bit for bit."""
    import torch
    from cassia_gb300 import Composition, scenes
    from cassia_gb300.composition import kernel_launches, render_batch
    w = WORKLOADS[args.workload]
    t0 = time.time()
    sset = scenes.batch(seed=w["seed"] + rank, n_scenes=w["n_scenes"])
    gen_s = time.time() - t0
    comps = []
    for sc in sset:
        c = Composition(wide=sc.wide)
        scenes.load(sc, c)
        comps.append(c)
    outs_b = [torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda") for sc in sset]
    outs_p = [torch.zeros_like(o) for o in outs_b]
    ctx = Composition()
    groups = group_scenes(comps, sset)
    # groups are rendered on args.batch_streams contexts at once (one stream and
    # one host thread each), so that one group's tail overlaps the next group
    ctxs = [ctx] + [Composition() for _ in range(max(1, args.batch_streams) - 1)]

    def render_groups(contexts, outs, with_heights=True, mapped=False):
        def part(j):
            for gi, g in enumerate(groups):
                if gi % len(contexts) == j:
                    render_batch(contexts[j], [comps[k] for k in g], [outs[k] for k in g], [sset[k].width for k in g],
                                 [sset[k].background for k in g],
                                 heights=[sset[k].height for k in g] if with_heights else None, mapped=mapped)
        if len(contexts) == 1:
            part(0)
            return
        errors = []

        def guarded(j):
            try:
                part(j)
            except BaseException as e:  # re-raised below: a failed group must fail the run
                errors.append(e)

        threads = [threading.Thread(target=guarded, args=(j,)) for j in range(len(contexts))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]

    ptrs_b = [o.data_ptr() for o in outs_b]

    def batched_one():  # one context (what the autotuner times on its stream)
        render_groups(ctxs[:1], ptrs_b)

    def batched():
        render_groups(ctxs, ptrs_b)

    def plain():
        for k, sc in enumerate(sset):
            comps[k].render(outs_p[k].data_ptr(), sc.width, sc.background, height=sc.height)

    def timed(fn, reps):
        torch.cuda.synchronize()
        barrier()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return over_ranks((time.perf_counter() - t) / reps)

    # the autotuner picks the digit width, rasterizer block and painter block
    # for the batched pipeline; the same setting is applied to every
    # per-scene composition so that the comparison isolates batching
    from cassia_gb300 import autotune
    t_tune = time.time()
    tuning, trials = autotune.tune(ctx, batched_one, snapshot=lambda: [o.clone() for o in outs_b],
                                   same=lambda a, b: all(torch.equal(x, y) for x, y in zip(a, b)), reps=2)
    tune_s = time.time() - t_tune
    for c in ctxs[1:]:
        c.set_tuning(**tuning)
    if args.frame_mode == "graph":  # after tuning: each tuning is a new frame geometry
        for c in ctxs:
            c.set_graph_mode(True)
    for c in comps:
        c.set_tuning(**tuning)
    for _ in range(args.warmup):
        batched()
        plain()
    exact = all(torch.equal(a, b) for a, b in zip(outs_b, outs_p))
    launches0 = kernel_launches()
    with ClockSampler(local) as clk:
        tb = timed(batched, args.steps)
    launches = kernel_launches() - launches0
    # the plain loop both ways: every frame enqueued stage by stage, and
    # every scene replayed from its own frame graph
    tp = timed(plain, max(1, args.steps // 2))
    for c in comps:
        c.set_graph_mode(True)
    for _ in range(2):
        plain()
    tpg = timed(plain, max(1, args.steps // 2))
    exact = exact and all(torch.equal(a, b) for a, b in zip(outs_b, outs_p))
    tp_ref = tpg if args.frame_mode == "graph" else tp
    segs = sum(c.count_segments()[0] for c in comps)
    # e2e: the same batched pass into pinned host buffers (RGBA8 read back each pass)
    host = [torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8).pin_memory().numpy() for sc in sset]

    def batched_host():  # page-locked host buffers, written by the painter directly
        render_groups(ctxs, host, with_heights=False, mapped=True)

    for _ in range(args.warmup):
        batched_host()
    te = timed(batched_host, max(1, args.steps // 2))
    if rank == 0:
        line = {
            "metric": "scenes/s", "value": world * len(sset) / tb, "unit": "scenes/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tb * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+int (fixed point)", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "scenes": len(sset), "layers": int(sum(s.n_layers for s in sset)),
                       "frames_per_pass": len(groups), "segments_per_pass": int(segs),
                       "contexts": len(ctxs),
                       "l2": "inputs larger than L2"},
            "plain_scenes_per_s": world * len(sset) / tp_ref, "plain_ms_per_pass": tp_ref * 1e3,
            "speedup_vs_plain": tp_ref / tb, "bit_exact_batched_vs_plain": bool(exact), "frame_mode": args.frame_mode,
            "plain_staged_ms_per_pass": tp * 1e3, "plain_graph_ms_per_pass": tpg * 1e3,
            "speedup_vs_plain_staged": tp / tb, "speedup_vs_plain_graph": tpg / tb,
            "tuning": tuning, "autotune": {"trials": len(trials), "seconds": tune_s,
                                           "ms_per_pass": {str(i): t["ms"] for i, t in enumerate(trials)}},
            "e2e": {"value": world * len(sset) / te, "unit": "scenes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(sum(s.width * s.height * 4 for s in sset)), "ms_per_step": te * 1e3},
            "gpu_launches": launches, "clocks": clk.summary(), "setup_s": {"scene_gen": gen_s},
        }
        return line
    return None


def run_serve(args, rank, world, local):
    """Serving workload: 64 clients with resident compositions (batched-workload
    distribution), Poisson arrivals at 2,000 requests/s; each frame gives 20%
    of a client's layers a new affine and adds/removes 1%.  Continuous
    batching (4 workers, batches of up to 16, 40 GB HBM budget) of
    incremental frames (each client's sorted segments stay resident; only
    changed layers are rasterized) against the plain loop (one full render
    call per request), on identical request streams.
    A server that keeps up serves the offered rate and no more, so the
    batched server is also run at twice the offered rate ("capacity": the
    frames/s it sustains when saturated), beside the plain loop's, which
    saturates at the offered rate."""
    import torch
    from cassia_gb300 import serving
    from cassia_gb300.composition import kernel_launches
    w = WORKLOADS[args.workload]
    reqs_b = serving.poisson_arrivals(w["rate"], w["n_clients"], w["duration"], seed=w["seed"] + rank)
    reqs_p = serving.poisson_arrivals(w["rate"], w["n_clients"], w["duration"], seed=w["seed"] + rank)
    out = {}
    runs = [("batched", reqs_b), ("plain", reqs_p), ("capacity", None)]
    for mode, reqs in runs:
        if mode == "capacity":
            # the batched server offered twice the configured rate: what it sustains when saturated
            rate = 2.0 * w["rate"]
            reqs = serving.poisson_arrivals(rate, w["n_clients"], w["duration"], seed=w["seed"] + rank + 1)
        # the served form keeps each client's segments resident and
        # re-rasterizes only changed layers; the plain loop re-renders in full
        clients = serving.make_clients(w["n_clients"], seed=w["seed"] + rank, device_out=True,
                                       incremental=mode != "plain")
        srv = serving.Server(clients, mode="plain" if mode == "plain" else "batched", workers=args.serve_workers,
                             max_batch=16, hbm_budget=40e9)
        l0 = kernel_launches()
        with ClockSampler(local) as clk:
            done = srv.run(reqs)
        torch.cuda.synchronize()
        s = serving.latency_summary(done, w["duration"])
        if mode == "capacity":
            s["offered_rate"] = rate
        # whole-job rate: the frames of every replica over the slowest replica's span
        span = over_ranks(s["requests"] / s["frames_per_s"])
        s["frames_per_s_all_ranks"] = over_ranks(s["requests"], "sum") / span
        s["gpu_launches"] = kernel_launches() - l0
        s["clocks"] = clk.summary()
        if mode == "batched":
            # each sampled client's last frame equals the same state rendered alone
            same = True
            for k in range(0, len(clients), max(1, len(clients) // 8)):
                cl = clients[k]
                alone = torch.zeros_like(cl.out)
                cl.comp.render(alone.data_ptr(), cl.scene.width, cl.scene.background, height=cl.scene.height)
                same &= bool(torch.equal(alone, cl.out))
            s["mix_equals_alone_sampled"] = same
        out[mode] = s
        del clients, srv
        torch.cuda.empty_cache()
    if rank == 0:
        b, p = out["batched"], out["plain"]
        line = {
            "metric": "frames/s", "value": b["frames_per_s_all_ranks"], "unit": "frames/s", "n_gpus": world,
            "steps": b["requests"], "warmup": 0, "ms_per_step": 1e3 / b["frames_per_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+int (fixed point)", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "clients": w["n_clients"], "offered_rate": w["rate"],
                       "duration_s": w["duration"], "hbm_budget_gb": 40, "max_batch": 16, "workers": args.serve_workers,
                       "served": "continuous batching, incremental frames", "plain": "one full render per request"},
            "p50_ms": b["p50_ms"], "p99_ms": b["p99_ms"], "batched": b, "plain": p,
            "capacity": {k: out["capacity"][k] for k in ("offered_rate", "frames_per_s", "frames_per_s_all_ranks",
                                                         "p50_ms", "p99_ms", "mean_batch")},
            "speedup_vs_plain": b["frames_per_s_all_ranks"] / p["frames_per_s_all_ranks"],
            "capacity_speedup_vs_plain": (out["capacity"]["frames_per_s_all_ranks"] /
                                          p["frames_per_s_all_ranks"]),
            "gpu_launches": b["gpu_launches"], "clocks": b["clocks"],
        }
        return line
    return None


def scene_config(workload, scene, world):
    """The workload as both arms name it: the scene, not what a run measured."""
    return {"workload": workload, "canvas": [scene.width, scene.height], "layers": scene.n_layers,
            "segment_format": "wide (17-bit layer)" if scene.wide else "reference u16",
            "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    scene = make_scene(args.workload)
    r = cpu_reference(scene, args.steps, args.warmup, budget_s=args.cpu_budget)
    line = {
        "metric": "Msegments/s", "value": r["value"], "unit": "Msegments/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+int (fixed point)",
        "data": "synthetic (seeded)",
        "config": scene_config(args.workload, scene, world),
        "frames_per_s": r["frames_per_s"],
        "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": r["value"], "unit": "Msegments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mixed100k", choices=list(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--update-steps", type=int, default=5,
                    help="frames re-transforming 20%% / 5%% of the layers, full vs incremental (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quiet", action="store_true")
    ap.add_argument("--frame-mode", default="graph", choices=["staged", "graph"],
                    help="graph: frames replayed from a captured CUDA graph (cgb_set_graph_mode)")
    ap.add_argument("--serve-workers", type=int, default=4,
                    help="render workers of the served form (4 measured best: 3 leave the GPU idle during "
                         "host updates, 6 add nothing)")
    ap.add_argument("--blend-mode", type=int, default=None, choices=range(12),
                    help="give every layer this blend mode (the cost of one mode; changes the scene)")
    ap.add_argument("--batch-streams", type=int, default=2,
                    help="batch256: contexts (streams) the groups of scenes are rendered on at once")
    ap.add_argument("--no-forms", dest="forms", action="store_false",
                    help="mixed100k: skip the batched (batch256) and served (serve) sub-objects")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="seconds of host work the reference arm's samples are sized to")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        if args.impl == "ours":
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return rc

    torch.cuda.set_device(local)
    if WORKLOADS[args.workload]["kind"] in ("batch", "serve"):
        fn = run_batch if WORKLOADS[args.workload]["kind"] == "batch" else run_serve
        line = fn(args, rank, world, local)
        if line is not None:
            print(json.dumps(line))
        if dist:
            dist.destroy_process_group()
        return 0
    from cassia_gb300 import Composition, scenes
    from cassia_gb300.composition import kernel_launches

    t0 = time.time()
    scene = make_scene(args.workload)
    if args.blend_mode is not None:
        scene.blend_mode[:] = args.blend_mode
    gen_s = time.time() - t0
    comp = Composition(wide=scene.wide)
    t0 = time.time()
    scenes.load(scene, comp)
    load_s = time.time() - t0
    H, W = scene.height, scene.width
    # The reference rasterizes every line of the frame; render mode skips lines
    # whose segments cannot reach the canvas.  The metric counts the
    # reference's segments, counted once here.
    ref_segments, _ = comp.count_segments()
    if args.frame_mode == "graph":
        comp.set_graph_mode(True)
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.ExternalStream(comp.stream())

    def frame():
        comp.render(out.data_ptr(), W, scene.background, height=H)

    for _ in range(args.warmup):
        frame()
    comp.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    stats = []
    launches0 = kernel_launches()
    with ClockSampler(local) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            frame()
            stats.append(comp.stats())
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = kernel_launches() - launches0
    if dist:
        dist.barrier()
    ms_total = ev0.elapsed_time(ev1)
    ms_step = ms_total / args.steps
    ms_step = over_ranks(ms_step)
    st = stats[-1]
    segs = ref_segments
    value = world * segs / (ms_step / 1e3) / 1e6

    # stage times (device events on the launching stream), averaged over the timed steps
    stage_ms = {k: statistics.mean(s[k + "_ms"] for s in stats) for k in
                ("build", "rasterize", "sort", "carry", "paint", "total")}
    peak, peak_kind = load_peaks()
    sb = stage_bytes(st, scene)
    dom = max(("rasterize", "sort", "paint"), key=lambda k: stage_ms[k])
    achieved = sb[dom] / (stage_ms[dom] / 1e3) / 1e9
    traffic = read_traffic(args.workload, dom)
    frame_bytes = 18 * st["lines"] + 32 * segs + 32 * scene.n_layers + 4 * W * H

    # e2e through the public API with host buffers: every step uploads all
    # layer transforms from pinned host memory (the per-frame input of a
    # retained scene) and reads the RGBA8 frame back into pinned host memory.
    e2e = None
    if args.e2e_steps > 0:
        host_img = torch.zeros((H, W, 4), dtype=torch.uint8).pin_memory().numpy()
        ids = np.arange(scene.n_layers, dtype=np.uint32)
        tr = torch.from_numpy(scene.transforms if scene.transforms is not None
                              else np.tile(np.array([[1, 0, 0, 1, 0, 0]], np.float32), (scene.n_layers, 1)))
        # two placements prepared before the timed steps (the caller's input of
        # a frame), alternated so that every frame moves every layer
        tr = [tr.pin_memory().numpy() for _ in range(2)]
        tr[1][:, 4] += np.float32(0.25)
        # the frame goes to page-locked host memory that the painter writes
        # directly (CGB_MEMORY_HOST_MAPPED): no device staging and copy back
        for k in range(args.warmup):
            comp.set_transforms(ids, tr[k % 2])
            comp.render(host_img, W, scene.background, mapped=True)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.e2e_steps):
            comp.set_transforms(ids, tr[(args.warmup + k) % 2])
            comp.render(host_img, W, scene.background, mapped=True)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        e2e_s = over_ranks(e2e_s)
        h2d = scene.n_layers * (6 * 4)
        e2e = {"value": world * segs / e2e_s / 1e6, "unit": "Msegments/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": W * H * 4, "ms_per_step": e2e_s * 1e3}

    # Frames that give 20% (the serving workload's update) or 5% of the
    # layers a new affine: every frame in full, replayed from the frame graph,
    # against incremental frames (only the changed layers rasterized and
    # sorted, the rest kept resident and merged).  Same seeded updates.
    updates = None
    if args.update_steps > 0:
        ids = np.arange(scene.n_layers, dtype=np.uint32)
        base = (scene.transforms if scene.transforms is not None
                else np.tile(np.array([[1, 0, 0, 1, 0, 0]], np.float32), (scene.n_layers, 1))).astype(np.float32)

        def update(k, frac):
            rng = np.random.default_rng(7000 + k)
            sel = ids[rng.random(len(ids)) < frac]
            t = base[sel].copy()
            th = rng.uniform(-0.05, 0.05, len(sel)).astype(np.float32)
            c, s_ = np.cos(th), np.sin(th)
            a, b, cc, d = t[:, 0].copy(), t[:, 1].copy(), t[:, 2].copy(), t[:, 3].copy()
            t[:, 0], t[:, 1], t[:, 2], t[:, 3] = c * a - s_ * cc, c * b - s_ * d, s_ * a + c * cc, s_ * b + c * d
            t[:, 4] += rng.uniform(-3, 3, len(sel)).astype(np.float32)
            t[:, 5] += rng.uniform(-3, 3, len(sel)).astype(np.float32)
            base[sel] = t
            comp.set_transforms(sel, t)

        updates = {"steps": args.update_steps}
        start = base.copy()
        for frac in (0.2, 0.05):
            res = {}
            for mode in ("full", "incremental"):
                base[:] = start
                comp.set_transforms(ids, base)
                comp.set_incremental(mode == "incremental")
                comp.render(out.data_ptr(), W, scene.background, height=H)  # the first frame of the mode
                for k in (-2, -1):  # untimed update frames: the incremental ones size the sync-free form
                    update(k, frac)
                    comp.render(out.data_ptr(), W, scene.background, height=H)
                torch.cuda.synchronize()
                ms, dev = [], []
                for k in range(1, args.update_steps + 1):
                    update(k, frac)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    comp.render(out.data_ptr(), W, scene.background, height=H)
                    ms.append((time.perf_counter() - t0) * 1e3)
                    st_k = comp.stats()
                    dev.append(st_k["total_ms"])
                res[mode] = {"ms_per_frame": statistics.mean(ms), "device_ms_per_frame": statistics.mean(dev),
                             "segments_rasterized": int(st_k["segments"]),
                             "graph_replayed": int(st_k["graph_replayed"]),
                             "incremental_form": int(st_k["incremental_form"])}
            res["speedup"] = res["full"]["ms_per_frame"] / res["incremental"]["ms_per_frame"]
            updates[f"changed_{int(frac * 100)}pct"] = res
        comp.set_incremental(False)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            r = cpu_reference(scene, steps=1, warmup=0, budget_s=45.0)
            cpu = {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # report, do not hide
            cpu = {"value": None, "error": repr(e)}

    if rank == 0:
        line = {
            "metric": "Msegments/s", "value": value, "unit": "Msegments/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+int (fixed point)", "data": "synthetic (seeded)",
            "config": dict(scene_config(args.workload, scene, world),
                           **({} if args.blend_mode is None else {"blend_mode": args.blend_mode})),
            "frame_counts": {"lines": st["lines"], "segments_per_frame": segs,
                             "segments_rasterized": st["segments"],
                             "painted_segments": st["painted_segments"], "tile_layers": st["tile_layers"],
                             "work_items": st["work_items"], "lines_mb": st["lines"] * 20 // 2**20,
                             "segments_mb": segs * 8 // 2**20},
            "frames_per_s": world * 1e3 / ms_step,
            "frame_mode": args.frame_mode, "graph_replayed": int(st.get("graph_replayed", 0)),
            "sort_passes": int(st["sort_passes"]), "sort_passes_skipped": int(st["sort_passes_skipped"]),
            "stage_ms": stage_ms,
            "roofline": {"bound": "hbm", "kernel": STAGE_KERNELS[dom], "stage": dom, "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": traffic, "algorithmic_bytes": sb[dom],
                         "limiter": STAGE_LIMITERS.get(dom)},
            "frame_roofline": {"algorithmic_bytes": frame_bytes,
                               "achieved": frame_bytes / (ms_step / 1e3) / 1e9,
                               "frac": frame_bytes / (ms_step / 1e3) / 1e9 / peak},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "update_frames": updates,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "setup_s": {"scene_gen": gen_s, "load_insert_paths": load_s},
        }
    comp.close()
    del out
    torch.cuda.empty_cache()
    if args.forms and args.workload == "mixed100k" and args.blend_mode is None:
        # the other single-frame configurations (the 50,000-glyph and the
        # 1,000-circle scenes), then the batched (256 scenes) and served (64
        # clients) forms, each as a sub-object of the headline line
        others = {name: measure_frames(name, steps=20, warmup=3, local=local) for name in ("glyphs", "circles")}
        torch.cuda.empty_cache()
        fa = argparse.Namespace(**vars(args))
        fa.workload, fa.steps, fa.warmup = "batch256", 3, 3
        b = run_batch(fa, rank, world, local)
        torch.cuda.empty_cache()
        fa.workload = "serve"
        v = run_serve(fa, rank, world, local)
        torch.cuda.empty_cache()
        if rank == 0:
            line["workloads"] = others
            line["batched"] = {k: b[k] for k in (
                "metric", "value", "unit", "ms_per_step", "steps", "warmup", "config", "speedup_vs_plain",
                "speedup_vs_plain_graph", "speedup_vs_plain_staged", "plain_graph_ms_per_pass",
                "plain_staged_ms_per_pass", "bit_exact_batched_vs_plain", "tuning", "e2e", "gpu_launches", "clocks")}
            line["served"] = {
                "metric": v["metric"], "value": v["value"], "unit": v["unit"], "config": v["config"],
                "p50_ms": v["p50_ms"], "p99_ms": v["p99_ms"], "speedup_vs_plain": v["speedup_vs_plain"],
                "plain_frames_per_s": v["plain"]["frames_per_s_all_ranks"],
                "capacity": v["capacity"], "capacity_speedup_vs_plain": v["capacity_speedup_vs_plain"],
                "mix_equals_alone_sampled": v["batched"]["mix_equals_alone_sampled"],
                "requests": v["batched"]["requests"], "mean_batch": v["batched"]["mean_batch"],
                "gpu_launches": v["gpu_launches"], "clocks": v["clocks"]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
