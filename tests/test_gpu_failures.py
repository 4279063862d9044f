"""Failure detection without a GPU fault.

The device-side waits are bounded: the self-test makes the sort's look-back
wait on a tile that never publishes and expects the expiry to come back as
CGB_ERR_DEVICE_TIMEOUT with the context still usable.  Host-side injection:
an HBM budget too small for the frame, malformed path commands, layer ids
beyond the format, NaN coordinates (which must render as the oracle does).
"""
import ctypes

import numpy as np
import pytest

import oracle
from cassia_gb300 import abi, scenes
from cassia_gb300.types import Path, solid

from . import test_oracle_kats as kats

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_the_device_recovers(gpu_lib):
    from cassia_gb300 import Composition
    assert gpu_lib.cgb_selftest_bounded_wait() == abi.ERR_DEVICE_TIMEOUT, gpu_lib.cgb_last_error()
    # the process's context still renders correctly
    c, o = Composition(), oracle.Composition()
    for comp in (c, o):
        lid = comp.create_layer()
        comp.insert_in_layer(lid, kats.pixel_path(3, 2))
        comp.set_props(lid, solid((1.0, 0.0, 0.0, 1.0)))
    a = np.zeros((8, 8, 4), np.uint8)
    b = np.zeros_like(a)
    c.render(a, 8, (1.0, 1.0, 1.0, 1.0))
    o.render(b, 8, (1.0, 1.0, 1.0, 1.0))
    assert np.array_equal(a, b)


def test_over_budget_is_reported_and_other_handles_work(gpu_lib):
    from cassia_gb300 import Composition
    sc = scenes.mixed(seed=41, n_layers=3000, width=640, height=480)
    small = Composition(hbm_budget=1 << 20)
    with pytest.raises(abi.CassiaError) as ex:
        scenes.load(sc, small)
        img = np.zeros((sc.height, sc.width, 4), np.uint8)
        small.render(img, sc.width, sc.background)
    assert ex.value.status == abi.ERR_OVER_BUDGET
    big = Composition()
    scenes.load(sc, big)
    img = np.zeros((sc.height, sc.width, 4), np.uint8)
    big.render(img, sc.width, sc.background)
    assert img.any()


def test_malformed_inputs_are_rejected(gpu_lib):
    from cassia_gb300 import Composition
    c = Composition()
    lid = c.create_layer()
    kinds = (ctypes.c_uint32 * 1)(17)  # no such path command
    pts = (ctypes.c_float * 4)(0, 0, 1, 1)
    assert gpu_lib.cgb_insert_in_layer(c._h, lid, kinds, 1, pts, 4, None) == abi.ERR_INVALID_ARG
    kinds = (ctypes.c_uint32 * 1)(abi.CMD_LINE)
    assert gpu_lib.cgb_insert_in_layer(c._h, lid, kinds, 1, pts, 3, None) == abi.ERR_INVALID_ARG  # 3 of 4 floats
    segs = (ctypes.c_float * 4)(0, 0, 1, 1)
    assert gpu_lib.cgb_insert_lines(c._h, 1 << 16, segs, 1) == abi.ERR_LAYER_LIMIT  # beyond u16 ids
    with pytest.raises(abi.CassiaError) as ex:
        c.create_layers((1 << 16) + 1)
    assert ex.value.status == abi.ERR_LAYER_LIMIT
    assert gpu_lib.cgb_render(None, None, None, None) == abi.ERR_INVALID_ARG


def test_nan_coordinates_render_as_the_oracle(gpu_lib):
    from cassia_gb300 import Composition
    nan = float("nan")
    g, o = Composition(), oracle.Composition()
    for c in (g, o):
        lid = c.create_layer()
        c.insert_lines(lid, [[1.5, 1.0, 30.0, 20.0], [30.0, 20.0, nan, 4.0], [nan, 4.0, 1.5, 1.0],
                             [5.0, nan, 9.0, 25.0], [9.0, 25.0, 5.0, 3.0]])
        c.set_props(lid, solid((0.2, 0.6, 0.9, 0.8)))
        lid = c.create_layer()
        c.insert_in_layer(lid, Path().line((2.0, 2.0), (28.0, 6.0)).line((28.0, 6.0), (8.0, 28.0)).close())
        c.set_props(lid, solid((0.9, 0.3, 0.1, 0.7)))
    a = np.zeros((32, 40, 4), np.uint8)
    b = np.zeros_like(a)
    g.render(a, 40, (1.0, 1.0, 1.0, 1.0))
    o.render(b, 40, (1.0, 1.0, 1.0, 1.0))
    assert np.array_equal(a, b)
    gs, gn = g.pixel_segments(canonical=True)
    os_, on = o.pixel_segments(threads=2)
    assert gn == on and np.array_equal(gs, os_)
