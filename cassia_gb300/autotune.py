"""Autotuner for the pipeline's parallel decomposition (cgb_tuning).

The knobs change how the work is split, never the pixels: the radix digit
width (how many sort passes a key takes), the rasterizer's threads per block
and pixel steps per thread, and the painter's tiles (warps) per block.  The
tuner times a caller-supplied workload under candidate settings with CUDA
events on the handle's stream, by coordinate descent from the current
setting, checks that every candidate renders the same output as the starting
one, and keeps the fastest.  Results can be cached in a JSON file keyed by a
workload signature and the GPU name.
"""
import json
import os
from typing import Callable, Dict, List, Optional

KNOBS: Dict[str, List[int]] = {
    "radix_bits": [8, 9],
    "raster_block": [128, 256],
    "steps_per_thread": [4, 8],
    "paint_warps": [2, 4, 8],
}


def _to_tuning(point: dict) -> dict:
    return {"radix_bits": point["radix_bits"], "raster_block": point["raster_block"],
            "steps_per_block": point["raster_block"] * point["steps_per_thread"],
            "paint_warps": point["paint_warps"]}


def _from_tuning(t: dict) -> dict:
    return {"radix_bits": t["radix_bits"], "raster_block": t["raster_block"],
            "steps_per_thread": t["steps_per_block"] // t["raster_block"], "paint_warps": t["paint_warps"]}


def time_ms(ctx, run: Callable[[], None], reps: int = 3) -> float:
    """Mean device time of run() on ctx's stream over reps calls, after one warm-up call."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream())
    run()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        run()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune(ctx, run: Callable[[], None], snapshot: Optional[Callable[[], object]] = None,
         same: Optional[Callable[[object, object], bool]] = None, reps: int = 3, rounds: int = 2):
    """Coordinate descent over KNOBS.  `run` renders the workload through
    ctx's pipeline; `snapshot` returns its output and `same` compares two
    snapshots (every candidate must render what the starting setting does).
    Leaves the best setting on ctx and returns (tuning, trials)."""
    start = _from_tuning(ctx.tuning())
    ctx.set_tuning(**_to_tuning(start))
    ref = None
    if snapshot is not None:
        run()
        ref = snapshot()
    best, best_ms = dict(start), time_ms(ctx, run, reps)
    trials = [{"tuning": _to_tuning(best), "ms": best_ms}]
    seen = {tuple(sorted(best.items()))}
    for _ in range(rounds):
        improved = False
        for knob, values in KNOBS.items():
            for v in values:
                cand = dict(best, **{knob: v})
                key = tuple(sorted(cand.items()))
                if key in seen:
                    continue
                seen.add(key)
                ctx.set_tuning(**_to_tuning(cand))
                ms = time_ms(ctx, run, reps)
                if ref is not None and not same(ref, snapshot()):
                    raise RuntimeError(f"autotune: tuning {_to_tuning(cand)} changed the output")
                trials.append({"tuning": _to_tuning(cand), "ms": ms})
                if ms < best_ms:
                    best, best_ms, improved = cand, ms, True
        if not improved:
            break
    ctx.set_tuning(**_to_tuning(best))
    return _to_tuning(best), trials


def cached_tune(ctx, signature: str, run, path: Optional[str] = None, **kw):
    """tune() once per (signature, GPU); later calls apply the stored result."""
    import torch
    path = path or os.path.join(os.path.expanduser("~"), ".cache", "cassia_gb300", "tuning.json")
    key = f"{signature}|{torch.cuda.get_device_name()}"
    table = {}
    if os.path.exists(path):
        try:
            with open(path) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
    if key in table:
        ctx.set_tuning(**table[key])
        return table[key], []
    best, trials = tune(ctx, run, **kw)
    table[key] = best
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(table, f, indent=1)
    except OSError:
        pass
    return best, trials
