"""Python binding of the CPU oracle (surpass_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg, as the checker or the timed CPU baseline.  The
cassia_gb300 package never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

from cassia_gb300 import abi
from cassia_gb300.types import Path, Props, transform_array

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "surpass_oracle.cpp")
LIB = os.path.join(HERE, "_build", "libsurpass_oracle.so")

# Strict IEEE f32: no contraction, no fast-math (Rust never contracts a*b+c).
CXXFLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    deps = [SRC, os.path.join(HERE, "surpass_oracle.h"),
            os.path.join(os.path.dirname(HERE), "include", "cassia_gb300.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", *CXXFLAGS, "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        u32, u64, i32, sz, i64 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_size_t, ctypes.c_int64
        fp, vp = P(ctypes.c_float), ctypes.c_void_p
        sigs = {
            "orc_flatten": ([P(u32), sz, fp, fp, fp, sz], sz),
            "orc_build_lines": ([sz, fp, fp, fp, fp, P(u32), fp, P(u32), P(ctypes.c_int32), fp, fp, P(u32), fp, fp,
                                 fp, fp, P(ctypes.c_uint8)], None),
            "orc_rasterize_lines": ([sz, fp, fp, fp, fp, P(u32), P(u64), sz], sz),
            "orc_blend_scalar": ([u32, fp, fp, fp], None),
            "orc_blend_vector": ([u32, fp, fp, fp], None),
            "orc_gradient_color_at": ([P(abi.CgbProps), ctypes.c_float, ctypes.c_float, fp], None),
            "orc_to_bytes": ([fp, P(ctypes.c_uint8)], None),
            "orc_comp_new": ([u32], vp),
            "orc_comp_free": ([vp], None),
            "orc_comp_create_layer": ([vp, P(u32)], ctypes.c_int),
            "orc_comp_insert_path": ([vp, u32, P(u32), sz, fp, fp], ctypes.c_int),
            "orc_comp_insert_lines": ([vp, u32, fp, sz], ctypes.c_int),
            "orc_comp_insert_paths": ([vp, sz, P(u32), P(u64), P(u32), P(u64), fp, fp, P(ctypes.c_uint8)],
                                      ctypes.c_int),
            "orc_layers_set_solid": ([vp, sz, P(u32), P(u32), P(u32), fp], ctypes.c_int),
            "orc_layers_set_transforms": ([vp, sz, P(u32), fp, u32], ctypes.c_int),
            "orc_layer_set_enabled": ([vp, u32, ctypes.c_int], ctypes.c_int),
            "orc_layer_set_transform": ([vp, u32, fp, u32], ctypes.c_int),
            "orc_layer_set_order": ([vp, u32, u32], ctypes.c_int),
            "orc_layer_set_props": ([vp, u32, P(abi.CgbProps)], ctypes.c_int),
            "orc_comp_remove_disabled": ([vp], ctypes.c_int),
            "orc_comp_lens": ([vp, P(u64), P(u64)], None),
            "orc_comp_create_cache": ([vp, P(i32)], ctypes.c_int),
            "orc_comp_release_cache": ([vp, i32], ctypes.c_int),
            "orc_comp_render": ([vp, P(ctypes.c_uint8), sz, sz, sz, fp, P(i64), i32, ctypes.c_int], ctypes.c_int),
            "orc_comp_pixel_segments": ([vp, P(u64), sz, P(u64), P(u64), ctypes.c_int], ctypes.c_int),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _check(st, where):
    if st != 0:
        raise abi.CassiaError(st, where)


def flatten(path: Path, transform9=None):
    """PathSegments (mold/src/path/segments.rs) -> float32 array (n, 4)."""
    L = lib()
    k, p = path.c_arrays()
    t = transform_array(transform9, 9)
    n = L.orc_flatten(k, len(path.kinds), p, t, None, 0)
    out = np.zeros((max(n, 1), 4), np.float32)
    L.orc_flatten(k, len(path.kinds), p, t, _fptr(out), n)
    return out[:n]


def build_lines(segs, layer_ids=None, default_transform=None):
    """LinesBuilder::build with layers(_) == None; returns a dict of arrays."""
    L = lib()
    segs = np.ascontiguousarray(np.asarray(segs, np.float32).reshape(-1, 4))
    n = len(segs)
    cols = [np.ascontiguousarray(segs[:, i]) for i in range(4)]
    lids = np.zeros(n, np.uint32) if layer_ids is None else np.ascontiguousarray(layer_ids, np.uint32)
    out = {
        "orders": np.zeros(n, np.uint32), "starts": np.zeros(n, np.int32), "starts_f32": np.zeros(n, np.float32),
        "ends_f32": np.zeros(n, np.float32), "lengths": np.zeros(n, np.uint32), "slopes": np.zeros(n, np.float32),
        "slopes_recip": np.zeros(n, np.float32), "py_slope_pxs": np.zeros(n, np.float32),
        "px_slope_recip_pys": np.zeros(n, np.float32), "octants": np.zeros(n, np.uint8),
    }
    t = transform_array(default_transform, 6)
    P = ctypes.POINTER
    L.orc_build_lines(n, *[_fptr(c) for c in cols], lids.ctypes.data_as(P(ctypes.c_uint32)), t,
                      out["orders"].ctypes.data_as(P(ctypes.c_uint32)), out["starts"].ctypes.data_as(P(ctypes.c_int32)),
                      _fptr(out["starts_f32"]), _fptr(out["ends_f32"]),
                      out["lengths"].ctypes.data_as(P(ctypes.c_uint32)), _fptr(out["slopes"]),
                      _fptr(out["slopes_recip"]), _fptr(out["py_slope_pxs"]), _fptr(out["px_slope_recip_pys"]),
                      out["octants"].ctypes.data_as(P(ctypes.c_uint8)))
    return out


def rasterize_lines(segs, layer_ids=None):
    """Rasterizer::rasterize over LinesBuilder::build(|_| None): the
    reference's 2*S u64 array with NONE slots."""
    L = lib()
    segs = np.ascontiguousarray(np.asarray(segs, np.float32).reshape(-1, 4))
    n = len(segs)
    cols = [np.ascontiguousarray(segs[:, i]) for i in range(4)]
    lids = np.zeros(n, np.uint32) if layer_ids is None else np.ascontiguousarray(layer_ids, np.uint32)
    P = ctypes.POINTER
    lp = lids.ctypes.data_as(P(ctypes.c_uint32))
    m = L.orc_rasterize_lines(n, *[_fptr(c) for c in cols], lp, None, 0)
    out = np.zeros(max(m, 1), np.uint64)
    L.orc_rasterize_lines(n, *[_fptr(c) for c in cols], lp, out.ctypes.data_as(P(ctypes.c_uint64)), m)
    return out[:m]


def blend_scalar(mode, dst, src):
    L = lib()
    d = (ctypes.c_float * 4)(*dst)
    s = (ctypes.c_float * 4)(*src)
    o = (ctypes.c_float * 4)()
    L.orc_blend_scalar(int(mode), d, s, o)
    return list(o)


def blend_vector(mode, dst, src):
    L = lib()
    d = (ctypes.c_float * 3)(*dst)
    s = (ctypes.c_float * 3)(*src)
    o = (ctypes.c_float * 3)()
    L.orc_blend_vector(int(mode), d, s, o)
    return list(o)


def gradient_color_at(props: Props, x, y):
    L = lib()
    p, keep = props.to_c()
    o = (ctypes.c_float * 32)()
    L.orc_gradient_color_at(ctypes.byref(p), float(x), float(y), o)
    a = np.frombuffer(o, np.float32).reshape(4, 8)
    return [tuple(float(a[ch, k]) for ch in range(4)) for k in range(8)]


def to_bytes(color):
    L = lib()
    c = (ctypes.c_float * 4)(*color)
    o = (ctypes.c_uint8 * 4)()
    L.orc_to_bytes(c, o)
    return bytes(o)


class Composition:
    """mold::Composition restated on the CPU (mold/src/composition.rs)."""

    def __init__(self, wide=False):
        self._L = lib()
        self._h = self._L.orc_comp_new(abi.COMPOSITION_WIDE_LAYERS if wide else 0)

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self._L.orc_comp_free(h)

    def create_layer(self):
        out = ctypes.c_uint32()
        st = self._L.orc_comp_create_layer(self._h, ctypes.byref(out))
        return None if st else out.value

    def create_layers(self, n):
        return np.array([self.create_layer() for _ in range(n)], np.uint32)

    def insert_in_layer(self, layer_id, path: Path, transform9=None):
        k, p = path.c_arrays()
        _check(self._L.orc_comp_insert_path(self._h, layer_id, k, len(path.kinds), p,
                                            transform_array(transform9, 9)), "insert_in_layer")
        return self

    def insert_lines(self, layer_id, segs):
        segs = np.ascontiguousarray(np.asarray(segs, np.float32).reshape(-1, 4))
        _check(self._L.orc_comp_insert_lines(self._h, layer_id, _fptr(segs), len(segs)), "insert_lines")

    def insert_paths(self, scene):
        P = ctypes.POINTER
        s = scene
        st = self._L.orc_comp_insert_paths(
            self._h, s.n_paths, s.path_layer.ctypes.data_as(P(ctypes.c_uint32)),
            s.cmd_offsets.ctypes.data_as(P(ctypes.c_uint64)), s.kinds.ctypes.data_as(P(ctypes.c_uint32)),
            s.point_offsets.ctypes.data_as(P(ctypes.c_uint64)), _fptr(s.points), None, None)
        _check(st, "insert_paths")

    def set_layers_solid(self, ids, fill_rules, blend_modes, colors):
        P = ctypes.POINTER
        ids = np.ascontiguousarray(ids, np.uint32)
        fr = np.ascontiguousarray(fill_rules, np.uint32)
        bm = np.ascontiguousarray(blend_modes, np.uint32)
        col = np.ascontiguousarray(colors, np.float32)
        st = self._L.orc_layers_set_solid(self._h, len(ids), ids.ctypes.data_as(P(ctypes.c_uint32)),
                                          fr.ctypes.data_as(P(ctypes.c_uint32)),
                                          bm.ctypes.data_as(P(ctypes.c_uint32)), _fptr(col))
        _check(st, "set_layers_solid")

    def set_transforms(self, ids, affine6, unchecked=True):
        P = ctypes.POINTER
        ids = np.ascontiguousarray(ids, np.uint32)
        t = np.ascontiguousarray(affine6, np.float32)
        st = self._L.orc_layers_set_transforms(self._h, len(ids), ids.ctypes.data_as(P(ctypes.c_uint32)), _fptr(t),
                                               abi.TRANSFORM_UNCHECKED if unchecked else 0)
        _check(st, "set_transforms")

    def set_enabled_many(self, ids, enabled):
        for lid, e in zip(ids, enabled):
            self.set_enabled(int(lid), bool(e))

    def set_enabled(self, layer_id, enabled):
        _check(self._L.orc_layer_set_enabled(self._h, layer_id, int(bool(enabled))), "set_enabled")

    def set_transform(self, layer_id, affine6, unchecked=False):
        st = self._L.orc_layer_set_transform(self._h, layer_id, transform_array(affine6, 6),
                                             abi.TRANSFORM_UNCHECKED if unchecked else 0)
        _check(st, "set_transform")

    def set_order(self, layer_id, order):
        _check(self._L.orc_layer_set_order(self._h, layer_id, order), "set_order")

    def set_props(self, layer_id, props: Props):
        p, keep = props.to_c()
        _check(self._L.orc_layer_set_props(self._h, layer_id, ctypes.byref(p)), "set_props")

    def remove_disabled(self):
        self._L.orc_comp_remove_disabled(self._h)

    def lens(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._L.orc_comp_lens(self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def create_buffer_layer_cache(self):
        out = ctypes.c_int32()
        st = self._L.orc_comp_create_cache(self._h, ctypes.byref(out))
        return None if st else out.value

    def release_buffer_layer_cache(self, cache_id):
        self._L.orc_comp_release_cache(self._h, cache_id)

    def render(self, pixels: np.ndarray, width, background, crop=None, layer_cache=-1, width_stride=None,
               threads=1):
        """pixels: uint8 array of shape (height, width_stride, 4), updated in place."""
        assert pixels.dtype == np.uint8 and pixels.flags.c_contiguous
        stride = width_stride or width
        height = pixels.size // (4 * stride)
        bg = (ctypes.c_float * 4)(*background)
        cr = None if crop is None else (ctypes.c_int64 * 4)(*crop)
        st = self._L.orc_comp_render(self._h, pixels.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), width, height,
                                     stride, bg, cr, -1 if layer_cache is None else layer_cache, threads)
        _check(st, "render")
        return pixels

    def pixel_segments(self, threads=1):
        n, none = ctypes.c_uint64(), ctypes.c_uint64()
        st = self._L.orc_comp_pixel_segments(self._h, None, 0, ctypes.byref(n), ctypes.byref(none), threads)
        out = np.zeros(max(1, n.value), np.uint64)
        st = self._L.orc_comp_pixel_segments(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n.value,
                                             ctypes.byref(n), ctypes.byref(none), threads)
        _check(st, "pixel_segments")
        return out[:n.value], none.value

    def stats(self):
        class S(ctypes.Structure):
            _fields_ = [("build_ms", ctypes.c_double), ("rasterize_ms", ctypes.c_double),
                        ("sort_ms", ctypes.c_double), ("paint_ms", ctypes.c_double), ("lines", ctypes.c_uint64),
                        ("steps", ctypes.c_uint64), ("segments", ctypes.c_uint64)]
        s = S()
        fn = self._L.orc_comp_stats
        fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(S)]
        fn(self._h, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in S._fields_}
