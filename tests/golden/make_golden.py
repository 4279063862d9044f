"""Generates tests/golden/golden.json: the oracle's pixel segments and RGBA8 frames
for the benchmark configurations at their full sizes, as SHA-256 digests.

The reference (Rust surpass/mold) cannot be built here, so the golden values
come from the oracle (oracle/surpass_oracle.cpp, the statement-by-statement
restatement pinned by the reference's own known-answer tests in
tests/test_oracle_kats.py).  The GPU parity tests compare the CUDA path with
these digests directly, and a CPU test checks that the oracle still produces
them (on x86 and on Arm: the oracle is portable C++ compiled with
-ffp-contract=off).

    python tests/golden/make_golden.py          # rewrites golden.json
"""
import hashlib
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# name -> (scenes generator, keyword arguments); the same seeds and sizes as
# bench.py's workloads (config 1 circles, config 2a mixed65k, config 2
# mixed100k in the widened 17-bit layer format, config 3 glyphs) and two
# small cases that the CPU suite checks quickly
CASES = {
    "circles_small": ("circles", dict(seed=11, n_layers=300, size=256)),
    "mixed_small": ("mixed", dict(seed=12, n_layers=400, width=320, height=200)),
    "config1_circles": ("circles", dict(seed=1, n_layers=1000, size=1024)),
    "config2a_mixed65k": ("mixed", dict(seed=2, n_layers=65_535, width=2560, height=1600)),
    "config2_mixed100k": ("mixed", dict(seed=2, n_layers=100_000, width=2560, height=1600)),
    "config3_glyphs": ("glyphs", dict(seed=3, n_layers=50_000, width=3840, height=2160)),
}

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")


def make_scene(name):
    from cassia_gb300 import scenes
    fn, kw = CASES[name]
    return getattr(scenes, fn)(**kw)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_values(name, threads=8):
    import oracle
    from cassia_gb300 import scenes
    sc = make_scene(name)
    o = oracle.Composition(wide=sc.wide)
    scenes.load(sc, o)
    segs, none = o.pixel_segments(threads=threads)
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    o.render(img, sc.width, sc.background, threads=threads)
    return {
        "canvas": [sc.width, sc.height], "layers": sc.n_layers, "wide": bool(sc.wide),
        "segments": int(len(segs)), "none": int(none),
        "segments_sha256": digest(segs.astype("<u8")), "rgba_sha256": digest(img),
    }


def load():
    with open(PATH) as f:
        return json.load(f)


def main():
    out = {"generator": "tests/golden/make_golden.py", "source": "oracle/surpass_oracle.cpp",
           "segments": "canonical order (ascending full u64), little-endian u64", "cases": {}}
    for name in CASES:
        t = time.time()
        out["cases"][name] = {"scene": {"generator": CASES[name][0], **CASES[name][1]}, **oracle_values(name)}
        print(f"{name}: {out['cases'][name]['segments']} segments, {time.time() - t:.1f} s", flush=True)
    with open(PATH, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
