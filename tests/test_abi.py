"""The C-ABI library builds, loads without a GPU and exports every symbol
declared in include/*.h."""
import ctypes
import os

import pytest

from cassia_gb300 import abi


@pytest.fixture(scope="module")
def built_lib():
    from cassia_gb300 import build
    path = build.build()
    assert os.path.exists(path)
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = abi.header_symbols()
    assert "cgb_render" in names and "cgb_pixel_segments" in names and "cgb_composition_new" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in abi.header_symbols() if not hasattr(built_lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    # every declared entry point has a ctypes signature in cassia_gb300.abi
    lib = abi.load_library()
    for n in abi.header_symbols():
        fn = getattr(lib, n)
        assert fn.restype is not None or n.startswith("cgb_")


def test_version_string(built_lib):
    built_lib.cgb_version.restype = ctypes.c_char_p
    assert b"sm_103a" in built_lib.cgb_version()


def test_no_device_is_reported_not_crashed(built_lib):
    # On a machine without a GPU, creating a composition fails cleanly.
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = abi.load_library()
    h = ctypes.c_void_p()
    st = lib.cgb_composition_new(0, 0, ctypes.byref(h))
    assert st == abi.ERR_NO_DEVICE
