"""mold::Composition over the CUDA library's C ABI (include/cassia_gb300.h).

Composition mirrors mold/src/composition.rs:26-329: create_layer,
insert_in_layer(_transformed), layer setters (mold/src/layer.rs:145-244),
render into a Buffer, pixel_segments, remove_disabled and buffer layer
caches.  Every call goes through the native library; there is no CPU path.
"""
import ctypes
from typing import Optional

import numpy as np

from . import abi
from .types import Path, Props, transform_array


def _check(lib, st, where):
    if st != abi.OK:
        msg = lib.cgb_last_error()
        raise abi.CassiaError(st, where, msg.decode() if msg else "")


def _u32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def _u64p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _buffer(pixels, width, layer_cache=-1, width_stride=None, height=None, mapped=False):
    """mapped: `pixels` (a numpy array) is page-locked host memory the device
    writes directly (CGB_MEMORY_HOST_MAPPED), e.g. a pinned torch tensor's numpy view."""
    stride = width_stride or width
    b = abi.CgbBuffer()
    if isinstance(pixels, np.ndarray):
        assert pixels.dtype == np.uint8 and pixels.flags.c_contiguous
        b.pixels = pixels.ctypes.data
        b.height = pixels.size // (4 * stride)
        b.memory = abi.MEMORY_HOST_MAPPED if mapped else abi.MEMORY_HOST
    else:
        b.pixels = int(pixels)
        b.height = int(height)
        b.memory = abi.MEMORY_DEVICE
    b.width = width
    b.width_stride = stride
    b.layer_cache = -1 if layer_cache is None else layer_cache
    return b


def render_batch(ctx, scenes, pixels, widths, backgrounds, crops=None, heights=None, layer_caches=None,
                 mapped=False):
    """Renders several Compositions in one pipeline (cgb_render_batch) on
    `ctx`'s stream.  pixels[k] is a host numpy RGBA8 array (page-locked and
    written directly with `mapped`) or a device pointer (then heights[k] is
    required)."""
    lib = abi.load_library()
    n = len(scenes)
    bufs = (abi.CgbBuffer * max(n, 1))()
    for k in range(n):
        bufs[k] = _buffer(pixels[k], widths[k], layer_cache=-1 if layer_caches is None else layer_caches[k],
                          height=None if heights is None else heights[k], mapped=mapped)
    handles = (ctypes.c_void_p * max(n, 1))(*[s._h.value for s in scenes])
    bg = (ctypes.c_float * (4 * max(n, 1)))(*[float(v) for b in backgrounds for v in b])
    cr = None
    if crops is not None:
        cr = (abi.CgbRect * max(n, 1))(*[abi.CgbRect(*c) for c in crops])
    _check(lib, lib.cgb_render_batch(ctx._h, n, handles, bufs, bg, cr), "render_batch")
    return pixels


def solid_props(fill_rules, blend_modes, colors):
    """A cgb_props array of Solid Draw props, one per entry."""
    fr = np.asarray(fill_rules, np.uint32)
    n = len(fr)
    arr = (abi.CgbProps * max(n, 1))()
    view = np.frombuffer(arr, dtype=np.uint8).reshape(max(n, 1), ctypes.sizeof(abi.CgbProps))
    u32 = view[:, :40].view(np.uint32)
    u32[:n, 0] = fr
    u32[:n, 1] = abi.FUNC_DRAW
    u32[:n, 4] = np.asarray(blend_modes, np.uint32)
    u32[:n, 5] = abi.FILL_SOLID
    view[:n, 24:40].view(np.float32)[:] = np.asarray(colors, np.float32).reshape(-1, 4)
    return arr


def update_layers(updates):
    """cgb_update_layers: each update is a dict with `comp` and any of
    `transform_ids` + `transforms` (n x 6), `removed_ids`, and `added_from`
    (a Composition) + `added_from_ids` + `added_props` (a cgb_props array, as
    solid_props makes) + `added_transforms` (n x 6).  Returns, per update,
    the new layers' ids (uint32 array).  Transforms are stored unchecked."""
    lib = abi.load_library()
    n = len(updates)
    arr = (abi.CgbLayerUpdate * max(n, 1))()
    keep, outs = [], []
    for k, u in enumerate(updates):
        r = arr[k]
        r.comp = u["comp"]._h.value
        r.transform_flags = abi.TRANSFORM_UNCHECKED
        if u.get("transform_ids") is not None and len(u["transform_ids"]):
            ids = np.ascontiguousarray(u["transform_ids"], np.uint32)
            t = np.ascontiguousarray(u["transforms"], np.float32)
            keep += [ids, t]
            r.n_transforms, r.transform_ids, r.transforms = len(ids), _u32p(ids), _fp(t)
        if u.get("removed_ids") is not None and len(u["removed_ids"]):
            ids = np.ascontiguousarray(u["removed_ids"], np.uint32)
            keep.append(ids)
            r.n_removed, r.removed_ids = len(ids), _u32p(ids)
        out = np.zeros(0, np.uint32)
        if u.get("added_from_ids") is not None and len(u["added_from_ids"]):
            src = np.ascontiguousarray(u["added_from_ids"], np.uint32)
            out = np.zeros(len(src), np.uint32)
            keep += [src, out]
            r.n_added, r.added_from, r.added_from_ids, r.added_ids = len(src), u["added_from"]._h.value, _u32p(src), \
                _u32p(out)
            if u.get("added_props") is not None:
                keep.append(u["added_props"])
                r.added_props = ctypes.cast(u["added_props"], ctypes.POINTER(abi.CgbProps))
            if u.get("added_transforms") is not None:
                t = np.ascontiguousarray(u["added_transforms"], np.float32)
                keep.append(t)
                r.added_transforms = _fp(t)
        outs.append(out)
    _check(lib, lib.cgb_update_layers(n, arr), "update_layers")
    return outs


def kernel_launches() -> int:
    """Kernels launched by the native library in this process."""
    return int(abi.load_library().cgb_kernel_launches())


class Composition:
    """mold::Composition on the GPU.  `wide=True` selects the 17-bit layer
    segment format for more than 65,536 layer orders; `hbm_budget` caps the
    device memory the handle may hold (bytes, 0 = unlimited); `priority`
    ("normal", "high", "low") sets the priority of the handle's stream."""

    def __init__(self, wide: bool = False, hbm_budget: int = 0, priority: str = "normal"):
        self._lib = abi.load_library()
        h = ctypes.c_void_p()
        flags = abi.COMPOSITION_WIDE_LAYERS if wide else 0
        flags |= {"normal": 0, "high": abi.COMPOSITION_PRIORITY_HIGH, "low": abi.COMPOSITION_PRIORITY_LOW}[priority]
        _check(self._lib, self._lib.cgb_composition_new(flags, hbm_budget, ctypes.byref(h)), "Composition::new")
        self._h = h
        self.wide = wide

    def close(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self._lib.cgb_composition_free(h)

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- layers -------------------------------------------------------------
    def create_layer(self) -> Optional[int]:
        out = ctypes.c_uint32()
        st = self._lib.cgb_create_layer(self._h, ctypes.byref(out))
        return None if st else out.value

    def create_layers(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1), np.uint32)
        _check(self._lib, self._lib.cgb_create_layers(self._h, n, _u32p(out)), "create_layers")
        return out[:n]

    def insert_in_layer(self, layer_id: int, path: Path, transform9=None):
        k, p = path.c_arrays()
        st = self._lib.cgb_insert_in_layer(self._h, layer_id, k, len(path.kinds), p, len(path.points),
                                           transform_array(transform9, 9))
        _check(self._lib, st, "insert_in_layer")
        return self

    def insert_paths(self, scene, transforms9=None, has_transform=None):
        """Batched insert_in_layer of every path of a scene (cassia_gb300.scenes.Scene)."""
        s = scene
        t9 = None if transforms9 is None else np.ascontiguousarray(transforms9, np.float32)
        ht = None if has_transform is None else np.ascontiguousarray(has_transform, np.uint8)
        st = self._lib.cgb_insert_paths(
            self._h, s.n_paths, _u32p(s.path_layer), _u64p(s.cmd_offsets), _u32p(s.kinds), _u64p(s.point_offsets),
            _fp(s.points), None if t9 is None else _fp(t9),
            None if ht is None else ht.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        _check(self._lib, st, "insert_paths")

    def insert_lines(self, layer_id: int, segs):
        segs = np.ascontiguousarray(np.asarray(segs, np.float32).reshape(-1, 4))
        _check(self._lib, self._lib.cgb_insert_lines(self._h, layer_id, _fp(segs), len(segs)), "insert_lines")

    def insert_layer_copies(self, layer_ids, src: "Composition", src_layer_ids):
        """insert_in_layer of paths already flattened into `src`: layer
        layer_ids[k] gets a copy of the lines src holds for src_layer_ids[k]
        (device to device, no flattening, no wait)."""
        ids = np.ascontiguousarray(layer_ids, np.uint32)
        sids = np.ascontiguousarray(src_layer_ids, np.uint32)
        if len(ids) != len(sids):
            raise ValueError("layer_ids and src_layer_ids differ in length")
        _check(self._lib, self._lib.cgb_insert_layer_copies(self._h, len(ids), _u32p(ids), src._h, _u32p(sids)),
               "insert_layer_copies")

    def device_bytes(self) -> int:
        """Device memory the handle holds (what its HBM budget is checked against)."""
        out = ctypes.c_uint64()
        _check(self._lib, self._lib.cgb_get_memory(self._h, ctypes.byref(out)), "get_memory")
        return out.value

    def set_enabled(self, layer_id: int, enabled: bool):
        _check(self._lib, self._lib.cgb_layer_set_enabled(self._h, layer_id, int(bool(enabled))), "set_enabled")

    def set_enabled_many(self, ids, enabled):
        ids = np.ascontiguousarray(ids, np.uint32)
        en = np.ascontiguousarray(enabled, np.uint8)
        st = self._lib.cgb_layers_set_enabled(self._h, len(ids), _u32p(ids),
                                              en.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        _check(self._lib, st, "set_enabled_many")

    def set_transform(self, layer_id: int, affine6, unchecked: bool = False):
        st = self._lib.cgb_layer_set_transform(self._h, layer_id, transform_array(affine6, 6),
                                               abi.TRANSFORM_UNCHECKED if unchecked else 0)
        _check(self._lib, st, "set_transform")

    def set_transforms(self, ids, affine6, unchecked: bool = True):
        ids = np.ascontiguousarray(ids, np.uint32)
        t = np.ascontiguousarray(affine6, np.float32)
        st = self._lib.cgb_layers_set_transforms(self._h, len(ids), _u32p(ids), _fp(t),
                                                 abi.TRANSFORM_UNCHECKED if unchecked else 0)
        _check(self._lib, st, "set_transforms")

    def set_order(self, layer_id: int, order: int):
        _check(self._lib, self._lib.cgb_layer_set_order(self._h, layer_id, order), "set_order")

    def set_props(self, layer_id: int, props: Props):
        p, keep = props.to_c()
        _check(self._lib, self._lib.cgb_layer_set_props(self._h, layer_id, ctypes.byref(p)), "set_props")

    def set_layers_solid(self, ids, fill_rules, blend_modes, colors):
        ids = np.ascontiguousarray(ids, np.uint32)
        n = len(ids)
        arr = solid_props(fill_rules, blend_modes, colors)
        st = self._lib.cgb_layers_set_props(self._h, n, _u32p(ids), arr)
        _check(self._lib, st, "set_layers_solid")

    def remove_disabled(self):
        _check(self._lib, self._lib.cgb_remove_disabled(self._h), "remove_disabled")

    def lens(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib, self._lib.cgb_lines_len(self._h, ctypes.byref(a), ctypes.byref(b)), "lines_len")
        return a.value, b.value

    def create_buffer_layer_cache(self) -> Optional[int]:
        out = ctypes.c_int32()
        st = self._lib.cgb_create_buffer_layer_cache(self._h, ctypes.byref(out))
        return None if st else out.value

    def release_buffer_layer_cache(self, cache_id: int):
        _check(self._lib, self._lib.cgb_release_buffer_layer_cache(self._h, cache_id), "release_cache")

    # ---- frames -----------------------------------------------------------------
    def render(self, pixels, width, background, crop=None, layer_cache=-1, width_stride=None, height=None,
               flusher=None, mapped=False):
        """Composition::render.  `pixels` is a host uint8 numpy array of shape
        (height, width_stride, 4) (page-locked and written directly by the
        device with `mapped`), or a device pointer (int) with `height` given.
        `flusher(view)` (host buffers) is called with an (n, 4) uint8 view of
        each row slice of every tile written, as mold's Buffer::flusher."""
        b = _buffer(pixels, width, layer_cache, width_stride, height, mapped)
        cb = None
        if flusher is not None:
            def _flush(user, ptr, n):
                flusher(np.ctypeslib.as_array(ptr, shape=(n * 4,)).reshape(n, 4))
            cb = abi.FLUSH_FN(_flush)
            b.flusher = cb
        bg = (ctypes.c_float * 4)(*background)
        cr = None
        if crop is not None:
            cr = abi.CgbRect(*crop)
        st = self._lib.cgb_render(self._h, ctypes.byref(b), bg, None if cr is None else ctypes.byref(cr))
        _check(self._lib, st, "render")
        return pixels

    def cassia_render(self, segments, stylings, pixels, width, background, height=None):
        """cassia_render, headless: paints externally produced pixel segments
        (reference CompactSegments, any order, NONE allowed) with
        stylings[order] = (rgba, fill_rule, blend_mode) into `pixels`."""
        segs = np.ascontiguousarray(segments, np.uint64)
        arr = (abi.CgbCassiaStyling * max(len(stylings), 1))()
        for k, (fill, fr, bm) in enumerate(stylings):
            arr[k].fill[:] = [float(v) for v in fill]
            arr[k].fill_rule = int(fr)
            arr[k].blend_mode = int(bm)
        b = _buffer(pixels, width, -1, None, height)
        bg = (ctypes.c_float * 4)(*background)
        st = self._lib.cgb_cassia_render(self._h, _u64p(segs), len(segs), arr, len(stylings), ctypes.byref(b), bg)
        _check(self._lib, st, "cassia_render")
        return pixels

    def count_segments(self):
        """Real pixel segments the reference's rasterizer emits for the current
        scene (Composition::pixel_segments without the copy), and its NONE count."""
        n, none = ctypes.c_uint64(), ctypes.c_uint64()
        st = self._lib.cgb_pixel_segments(self._h, None, 0, ctypes.byref(n), ctypes.byref(none), abi.SORT_KEY)
        if st not in (abi.OK, abi.ERR_CAPACITY):
            _check(self._lib, st, "pixel_segments")
        return n.value, none.value

    def pixel_segments(self, canonical: bool = True):
        """Composition::pixel_segments: (sorted real segments, NONE count)."""
        n, none = ctypes.c_uint64(), ctypes.c_uint64()
        order = abi.SORT_CANONICAL if canonical else abi.SORT_KEY
        st = self._lib.cgb_pixel_segments(self._h, None, 0, ctypes.byref(n), ctypes.byref(none), order)
        if st not in (abi.OK, abi.ERR_CAPACITY):
            _check(self._lib, st, "pixel_segments")
        out = np.zeros(max(1, n.value), np.uint64)
        st = self._lib.cgb_pixel_segments(self._h, _u64p(out), n.value, ctypes.byref(n), ctypes.byref(none), order)
        _check(self._lib, st, "pixel_segments")
        return out[:n.value], none.value

    def stats(self) -> dict:
        s = abi.CgbStats()
        _check(self._lib, self._lib.cgb_get_stats(self._h, ctypes.byref(s)), "get_stats")
        return s.as_dict()

    def tuning(self) -> dict:
        t = abi.CgbTuning()
        _check(self._lib, self._lib.cgb_get_tuning(self._h, ctypes.byref(t)), "get_tuning")
        return {k: getattr(t, k) for k, _ in t._fields_}

    def set_tuning(self, **kw):
        t = abi.CgbTuning(**kw)
        _check(self._lib, self._lib.cgb_set_tuning(self._h, ctypes.byref(t)), "set_tuning")

    def set_graph_mode(self, enabled: bool = True, headroom: float = 0.125):
        """Replays frames whose geometry repeats from a captured CUDA graph
        (cgb_set_graph_mode); buffers get `headroom` above the counts of the
        frame a graph was captured after.  Pixels are identical either way."""
        _check(self._lib, self._lib.cgb_set_graph_mode(self._h, 1 if enabled else 0, float(headroom)),
               "set_graph_mode")

    def set_incremental(self, enabled: bool = True):
        """Keep the last frame's sorted segments on the device and rasterize
        only the layers whose geometry changed (cgb_set_incremental)."""
        _check(self._lib, self._lib.cgb_set_incremental(self._h, 1 if enabled else 0), "set_incremental")

    def stream(self) -> int:
        """The cudaStream_t (as an int) the handle launches on."""
        out = ctypes.c_void_p()
        _check(self._lib, self._lib.cgb_get_stream(self._h, ctypes.byref(out)), "get_stream")
        return out.value or 0

    def clear(self):
        _check(self._lib, self._lib.cgb_composition_clear(self._h), "clear")

    def synchronize(self):
        _check(self._lib, self._lib.cgb_synchronize(self._h), "synchronize")
