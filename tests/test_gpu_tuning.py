"""Tuning knobs change the parallel decomposition, never the pixels.

Every value of every knob (digit width, rasterizer block and steps per
thread, painter tiles per block) must render the same RGBA8 frame as the
default, and the default must equal the oracle; the autotuner must leave a
valid setting that renders the same frame.
"""
import numpy as np
import pytest

import oracle
from cassia_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.mixed(seed=31, n_layers=2500, width=520, height=300)


def test_every_knob_renders_the_same_frame(gpu_lib):
    import torch
    from cassia_gb300 import Composition
    sc = _scene()
    c = Composition(wide=sc.wide)
    scenes.load(sc, c)
    ref = np.zeros((sc.height, sc.width, 4), np.uint8)
    c.render(ref, sc.width, sc.background)
    o = oracle.Composition(wide=sc.wide)
    scenes.load(sc, o)
    want = np.zeros_like(ref)
    o.render(want, sc.width, sc.background, threads=8)
    assert np.array_equal(ref, want)
    settings = ([dict(radix_bits=b) for b in (4, 6, 7, 8, 9)] +
                [dict(raster_block=b, steps_per_block=b * i) for b in (32, 96, 128, 256) for i in (4, 8)] +
                [dict(paint_warps=w) for w in (2, 4, 8)])
    default = c.tuning()
    for t in settings:
        c.set_tuning(**default)
        c.set_tuning(**t)
        img = np.zeros_like(ref)
        c.render(img, sc.width, sc.background)
        assert np.array_equal(img, ref), f"tuning {t} changed the frame"
    c.set_tuning(**default)


def test_invalid_tuning_is_rejected(gpu_lib):
    from cassia_gb300 import Composition
    from cassia_gb300.abi import CassiaError
    c = Composition()
    for bad in (dict(radix_bits=10), dict(raster_block=48), dict(raster_block=512),
                dict(raster_block=128, steps_per_block=256), dict(paint_warps=3)):
        with pytest.raises(CassiaError):
            c.set_tuning(**bad)


def test_autotune_keeps_the_frame(gpu_lib):
    import torch
    from cassia_gb300 import Composition, autotune
    sc = _scene()
    c = Composition(wide=sc.wide)
    scenes.load(sc, c)
    out = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")

    def run():
        c.render(out.data_ptr(), sc.width, sc.background, height=sc.height)

    best, trials = autotune.tune(c, run, snapshot=lambda: out.clone(), same=torch.equal, reps=1, rounds=1)
    assert len(trials) >= 2
    assert c.tuning() == best
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    c.render(img, sc.width, sc.background)
    o = oracle.Composition(wide=sc.wide)
    scenes.load(sc, o)
    want = np.zeros_like(img)
    o.render(want, sc.width, sc.background, threads=8)
    assert np.array_equal(img, want)
