"""ctypes mirror of include/cassia_gb300.h (plain-data types and constants).

Importing this module loads no native code; `load_library()` does, and fails
loudly when the CUDA library has not been built.
"""
import ctypes
import os

# status codes
OK = 0
ERR_INVALID_ARG = 1
ERR_OUT_OF_MEMORY = 2
ERR_OVER_BUDGET = 3
ERR_LAYER_LIMIT = 4
ERR_DEVICE_TIMEOUT = 5
ERR_DEVICE = 6
ERR_NO_DEVICE = 7
ERR_CAPACITY = 8
ERR_NOT_FOUND = 9
ERR_SCALE = 10

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "OVER_BUDGET", 4: "LAYER_LIMIT",
    5: "DEVICE_TIMEOUT", 6: "DEVICE", 7: "NO_DEVICE", 8: "CAPACITY", 9: "NOT_FOUND", 10: "SCALE",
}

FILL_NONZERO, FILL_EVENODD = 0, 1
FUNC_DRAW, FUNC_CLIP = 0, 1
FILL_SOLID, FILL_GRADIENT = 0, 1
GRADIENT_LINEAR, GRADIENT_RADIAL = 0, 1
CMD_LINE, CMD_QUAD, CMD_RAT_QUAD, CMD_CUBIC, CMD_RAT_CUBIC, CMD_CLOSE = range(6)
CMD_FLOATS = {CMD_LINE: 4, CMD_QUAD: 6, CMD_RAT_QUAD: 9, CMD_CUBIC: 8, CMD_RAT_CUBIC: 12, CMD_CLOSE: 0}
COMPOSITION_WIDE_LAYERS = 1
COMPOSITION_PRIORITY_HIGH = 2
COMPOSITION_PRIORITY_LOW = 4
TRANSFORM_UNCHECKED = 1
SORT_CANONICAL, SORT_KEY = 0, 1
MEMORY_HOST, MEMORY_DEVICE, MEMORY_HOST_MAPPED = 0, 1, 2


class CgbProps(ctypes.Structure):
    _fields_ = [
        ("fill_rule", ctypes.c_uint32),
        ("func", ctypes.c_uint32),
        ("clip_layers", ctypes.c_uint32),
        ("is_clipped", ctypes.c_uint32),
        ("blend_mode", ctypes.c_uint32),
        ("fill_kind", ctypes.c_uint32),
        ("color", ctypes.c_float * 4),
        ("gradient_type", ctypes.c_uint32),
        ("n_stops", ctypes.c_uint32),
        ("gradient_start", ctypes.c_float * 2),
        ("gradient_end", ctypes.c_float * 2),
        ("stops", ctypes.POINTER(ctypes.c_float)),
    ]


class CgbLayerUpdate(ctypes.Structure):
    _fields_ = [
        ("comp", ctypes.c_void_p),
        ("n_transforms", ctypes.c_size_t),
        ("transform_ids", ctypes.POINTER(ctypes.c_uint32)),
        ("transforms", ctypes.POINTER(ctypes.c_float)),
        ("transform_flags", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("n_removed", ctypes.c_size_t),
        ("removed_ids", ctypes.POINTER(ctypes.c_uint32)),
        ("n_added", ctypes.c_size_t),
        ("added_from", ctypes.c_void_p),
        ("added_from_ids", ctypes.POINTER(ctypes.c_uint32)),
        ("added_props", ctypes.POINTER(CgbProps)),
        ("added_transforms", ctypes.POINTER(ctypes.c_float)),
        ("added_ids", ctypes.POINTER(ctypes.c_uint32)),
    ]


# cgb_flush_fn: (user, pixels, n_pixels)
FLUSH_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t)


class CgbBuffer(ctypes.Structure):
    _fields_ = [
        ("pixels", ctypes.c_void_p),
        ("width", ctypes.c_uint64),
        ("height", ctypes.c_uint64),
        ("width_stride", ctypes.c_uint64),
        ("layer_cache", ctypes.c_int32),
        ("memory", ctypes.c_uint32),
        ("flusher", FLUSH_FN),
        ("flusher_user", ctypes.c_void_p),
    ]


class CgbCassiaStyling(ctypes.Structure):
    """cassia's CassiaStyling (cassia/src/Cassia.h:25-30)."""
    _fields_ = [
        ("fill", ctypes.c_float * 4),
        ("fill_rule", ctypes.c_uint32),
        ("blend_mode", ctypes.c_uint32),
        ("_padding", ctypes.c_uint32 * 2),
    ]


class CgbRect(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_uint64), ("x1", ctypes.c_uint64), ("y0", ctypes.c_uint64), ("y1", ctypes.c_uint64)]


class CgbStats(ctypes.Structure):
    _fields_ = [
        ("lines", ctypes.c_uint64),
        ("steps", ctypes.c_uint64),
        ("segments", ctypes.c_uint64),
        ("painted_segments", ctypes.c_uint64),
        ("tile_layers", ctypes.c_uint64),
        ("work_items", ctypes.c_uint64),
        ("sort_passes", ctypes.c_uint32),
        ("item_sort_passes", ctypes.c_uint32),
        ("build_ms", ctypes.c_float),
        ("rasterize_ms", ctypes.c_float),
        ("sort_ms", ctypes.c_float),
        ("carry_ms", ctypes.c_float),
        ("paint_ms", ctypes.c_float),
        ("total_ms", ctypes.c_float),
        ("graph_replayed", ctypes.c_uint32),
        ("graphs_cached", ctypes.c_uint32),
        ("incremental_form", ctypes.c_uint32),
        ("sort_passes_skipped", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class CgbTuning(ctypes.Structure):
    _fields_ = [
        ("radix_bits", ctypes.c_uint32),
        ("raster_block", ctypes.c_uint32),
        ("steps_per_block", ctypes.c_uint32),
        ("paint_warps", ctypes.c_uint32),
    ]


PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(PACKAGE_DIR, "_build", "libcassia_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(PACKAGE_DIR), "include", "cassia_gb300.h")


class CassiaError(RuntimeError):
    def __init__(self, status, where, message=""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{where}: {name}" + (f" ({message})" if message else ""))


_LIB = None


def load_library():
    """Loads the in-tree CUDA library.  Raises if it has not been built: the
    package has no CPU fallback."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIBRARY_PATH):
        raise RuntimeError(
            f"cassia_gb300 CUDA library not built: {LIBRARY_PATH} is missing "
            "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = ctypes.CDLL(LIBRARY_PATH)
    _declare(lib)
    _LIB = lib
    return lib


def _declare(lib):
    P = ctypes.POINTER
    u32, u64, i32, sz = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_size_t
    vp, fp = ctypes.c_void_p, P(ctypes.c_float)
    handle = vp
    sigs = {
        "cgb_version": ([], ctypes.c_char_p),
        "cgb_last_error": ([], ctypes.c_char_p),
        "cgb_composition_new": ([u32, u64, P(vp)], i32),
        "cgb_composition_free": ([handle], i32),
        "cgb_create_layer": ([handle, P(u32)], i32),
        "cgb_create_layers": ([handle, sz, P(u32)], i32),
        "cgb_insert_in_layer": ([handle, u32, P(u32), sz, fp, sz, fp], i32),
        "cgb_insert_paths": ([handle, sz, P(u32), P(u64), P(u32), P(u64), fp, fp, P(ctypes.c_uint8)], i32),
        "cgb_insert_lines": ([handle, u32, fp, sz], i32),
        "cgb_insert_layer_copies": ([handle, sz, P(u32), handle, P(u32)], i32),
        "cgb_get_memory": ([handle, P(u64)], i32),
        "cgb_update_layers": ([sz, P(CgbLayerUpdate)], i32),
        "cgb_layer_set_enabled": ([handle, u32, ctypes.c_int], i32),
        "cgb_layer_set_transform": ([handle, u32, fp, u32], i32),
        "cgb_layer_set_order": ([handle, u32, u32], i32),
        "cgb_layer_set_props": ([handle, u32, P(CgbProps)], i32),
        "cgb_layers_set_transforms": ([handle, sz, P(u32), fp, u32], i32),
        "cgb_layers_set_props": ([handle, sz, P(u32), P(CgbProps)], i32),
        "cgb_layers_set_enabled": ([handle, sz, P(u32), P(ctypes.c_uint8)], i32),
        "cgb_remove_disabled": ([handle], i32),
        "cgb_lines_len": ([handle, P(u64), P(u64)], i32),
        "cgb_create_buffer_layer_cache": ([handle, P(i32)], i32),
        "cgb_release_buffer_layer_cache": ([handle, i32], i32),
        "cgb_render": ([handle, P(CgbBuffer), fp, P(CgbRect)], i32),
        "cgb_cassia_render": ([handle, P(u64), sz, P(CgbCassiaStyling), sz, P(CgbBuffer), fp], i32),
        "cgb_render_batch": ([handle, sz, P(vp), P(CgbBuffer), fp, P(CgbRect)], i32),
        "cgb_pixel_segments": ([handle, P(u64), sz, P(u64), P(u64), u32], i32),
        "cgb_get_stats": ([handle, P(CgbStats)], i32),
        "cgb_set_tuning": ([handle, P(CgbTuning)], i32),
        "cgb_set_graph_mode": ([handle, ctypes.c_int, ctypes.c_float], i32),
        "cgb_set_incremental": ([handle, ctypes.c_int], i32),
        "cgb_get_tuning": ([handle, P(CgbTuning)], i32),
        "cgb_synchronize": ([handle], i32),
        "cgb_get_stream": ([handle, P(vp)], i32),
        "cgb_kernel_launches": ([], u64),
        "cgb_composition_clear": ([handle], i32),
        "cgb_sort_keys_noalloc": ([vp, vp, sz, u32, u32, vp], i32),
        "cgb_selftest_bounded_wait": ([], i32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def header_symbols(path=HEADER_PATH):
    """Names of the functions declared CGB_EXPORT in include/*.h."""
    import re
    names = []
    inc = os.path.dirname(path)
    for fname in sorted(os.listdir(inc)):
        if not fname.endswith(".h"):
            continue
        with open(os.path.join(inc, fname)) as f:
            text = f.read()
        names += re.findall(r"CGB_EXPORT\s+[\w\s\*]+?\b(\w+)\s*\(", text)
    return names
