//! Raw bindings to `libcassia_gb300.so`, one item per declaration of
//! `include/cassia_gb300.h` (same names, same field order, same argument
//! order).  mold's `Composition` forwards to these calls:
//!
//! | mold (file:line)                                            | call                                   |
//! |-------------------------------------------------------------|----------------------------------------|
//! | `Composition::new` (mold/src/composition.rs:36-48)          | `cgb_composition_new`                  |
//! | `create_layer` (composition.rs:54-56)                       | `cgb_create_layer`                     |
//! | `insert_in_layer[_transformed]` (composition.rs:58-94)      | `cgb_insert_in_layer`                  |
//! | `Layer::set_*`, `enable`, `disable` (mold/src/layer.rs:158-231) | `cgb_layer_set_*`                  |
//! | `remove_disabled` (composition.rs:124-142)                  | `cgb_remove_disabled`                  |
//! | `create_buffer_layer_cache` (composition.rs:144-151)        | `cgb_create_buffer_layer_cache`        |
//! | `BufferLayerCache::drop` (mold/src/buffer.rs:62-71)         | `cgb_release_buffer_layer_cache`       |
//! | `render` (composition.rs:212-329)                           | `cgb_render`                           |
//! | `pixel_segments` (composition.rs:153-188)                   | `cgb_pixel_segments(.., CGB_SORT_KEY)` |
//!
//! The cassia-format consumer (`cassia_init/render/shutdown`,
//! cassia/src/Cassia.h:32-41) is `cgb_cassia_render`; `dl::CassiaGb300`
//! (feature `dlopen`) loads it the way the reference demo loads libcassia.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

#[cfg(feature = "dlopen")]
pub mod dl;

// ---- status codes ------------------------------------------------------------
pub type cgb_status = i32;
pub const CGB_OK: cgb_status = 0;
pub const CGB_ERR_INVALID_ARG: cgb_status = 1;
pub const CGB_ERR_OUT_OF_MEMORY: cgb_status = 2;
pub const CGB_ERR_OVER_BUDGET: cgb_status = 3;
pub const CGB_ERR_LAYER_LIMIT: cgb_status = 4;
pub const CGB_ERR_DEVICE_TIMEOUT: cgb_status = 5;
pub const CGB_ERR_DEVICE: cgb_status = 6;
pub const CGB_ERR_NO_DEVICE: cgb_status = 7;
pub const CGB_ERR_CAPACITY: cgb_status = 8;
pub const CGB_ERR_NOT_FOUND: cgb_status = 9;
pub const CGB_ERR_SCALE: cgb_status = 10;

// ---- enums (the reference's enum order) ---------------------------------------
pub const CGB_FILL_NONZERO: u32 = 0;
pub const CGB_FILL_EVENODD: u32 = 1;
pub const CGB_BLEND_OVER: u32 = 0;
pub const CGB_BLEND_MULTIPLY: u32 = 1;
pub const CGB_BLEND_SCREEN: u32 = 2;
pub const CGB_BLEND_OVERLAY: u32 = 3;
pub const CGB_BLEND_DARKEN: u32 = 4;
pub const CGB_BLEND_LIGHTEN: u32 = 5;
pub const CGB_BLEND_COLOR_DODGE: u32 = 6;
pub const CGB_BLEND_COLOR_BURN: u32 = 7;
pub const CGB_BLEND_HARD_LIGHT: u32 = 8;
pub const CGB_BLEND_SOFT_LIGHT: u32 = 9;
pub const CGB_BLEND_DIFFERENCE: u32 = 10;
pub const CGB_BLEND_EXCLUSION: u32 = 11;
pub const CGB_FUNC_DRAW: u32 = 0;
pub const CGB_FUNC_CLIP: u32 = 1;
pub const CGB_FILL_SOLID: u32 = 0;
pub const CGB_FILL_GRADIENT: u32 = 1;
pub const CGB_GRADIENT_LINEAR: u32 = 0;
pub const CGB_GRADIENT_RADIAL: u32 = 1;

// mold PathCommand (mold/src/path/mod.rs:13-21); floats per command as in the header.
pub const CGB_CMD_LINE: u32 = 0;
pub const CGB_CMD_QUAD: u32 = 1;
pub const CGB_CMD_RAT_QUAD: u32 = 2;
pub const CGB_CMD_CUBIC: u32 = 3;
pub const CGB_CMD_RAT_CUBIC: u32 = 4;
pub const CGB_CMD_CLOSE: u32 = 5;

pub const CGB_COMPOSITION_WIDE_LAYERS: u32 = 1;
pub const CGB_COMPOSITION_PRIORITY_HIGH: u32 = 2;
pub const CGB_COMPOSITION_PRIORITY_LOW: u32 = 4;
pub const CGB_TRANSFORM_UNCHECKED: u32 = 1;
pub const CGB_SORT_CANONICAL: u32 = 0;
pub const CGB_SORT_KEY: u32 = 1;
pub const CGB_MEMORY_HOST: u32 = 0;
pub const CGB_MEMORY_DEVICE: u32 = 1;
pub const CGB_MEMORY_HOST_MAPPED: u32 = 2;

// ---- plain-data types ------------------------------------------------------------

/// surpass `Props` + `Style` (surpass/src/painter/mod.rs:125-141, style.rs:427-432).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cgb_props {
    pub fill_rule: u32,
    pub func: u32,
    pub clip_layers: u32,
    pub is_clipped: u32,
    pub blend_mode: u32,
    pub fill_kind: u32,
    pub color: [f32; 4],
    pub gradient_type: u32,
    pub n_stops: u32,
    pub gradient_start: [f32; 2],
    pub gradient_end: [f32; 2],
    pub stops: *const f32,
}

/// surpass `Flusher::flush` (surpass/src/painter/buffer_layout.rs:52-54); `None` is NULL.
pub type cgb_flush_fn = Option<unsafe extern "C" fn(user: *mut c_void, pixels: *mut u8, n_pixels: usize)>;

/// mold `Buffer` (mold/src/buffer.rs:19-25).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cgb_buffer {
    pub pixels: *mut u8,
    pub width: u64,
    pub height: u64,
    pub width_stride: u64,
    pub layer_cache: i32,
    pub memory: u32,
    pub flusher: cgb_flush_fn,
    pub flusher_user: *mut c_void,
}

/// surpass painter `Rect` (surpass/src/painter/buffer_layout.rs:37-50).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cgb_rect {
    pub x0: u64,
    pub x1: u64,
    pub y0: u64,
    pub y1: u64,
}

/// Sizes and device stage times of the last render / pixel_segments.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cgb_stats {
    pub lines: u64,
    pub steps: u64,
    pub segments: u64,
    pub painted_segments: u64,
    pub tile_layers: u64,
    pub work_items: u64,
    pub sort_passes: u32,
    pub item_sort_passes: u32,
    pub build_ms: f32,
    pub rasterize_ms: f32,
    pub sort_ms: f32,
    pub carry_ms: f32,
    pub paint_ms: f32,
    pub total_ms: f32,
    pub graph_replayed: u32,
    pub graphs_cached: u32,
    pub incremental_form: u32,
    pub sort_passes_skipped: u32,
}

/// Autotuned knobs (0 keeps the current value).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cgb_tuning {
    pub radix_bits: u32,
    pub raster_block: u32,
    pub steps_per_block: u32,
    pub paint_warps: u32,
}

/// cassia's `CassiaStyling` (cassia/src/Cassia.h:25-30); the demo's `Styling`.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cgb_cassia_styling {
    pub fill: [f32; 4],
    pub fill_rule: u32,
    pub blend_mode: u32,
    pub _padding: [u32; 2],
}

/// One composition's changes between two frames (cgb_update_layers).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cgb_layer_update {
    pub comp: *mut cgb_composition,
    pub n_transforms: usize,
    pub transform_ids: *const u32,
    pub transforms: *const f32,
    pub transform_flags: u32,
    pub reserved: u32,
    pub n_removed: usize,
    pub removed_ids: *const u32,
    pub n_added: usize,
    pub added_from: *mut cgb_composition,
    pub added_from_ids: *const u32,
    pub added_props: *const cgb_props,
    pub added_transforms: *const f32,
    pub added_ids: *mut u32,
}

/// Opaque composition handle.
#[repr(C)]
pub struct cgb_composition {
    _private: [u8; 0],
}

// ---- functions --------------------------------------------------------------------
extern "C" {
    pub fn cgb_version() -> *const c_char;
    pub fn cgb_last_error() -> *const c_char;

    pub fn cgb_composition_new(flags: u32, hbm_budget_bytes: u64, out: *mut *mut cgb_composition) -> cgb_status;
    pub fn cgb_composition_free(c: *mut cgb_composition) -> cgb_status;

    pub fn cgb_create_layer(c: *mut cgb_composition, out_layer_id: *mut u32) -> cgb_status;
    pub fn cgb_create_layers(c: *mut cgb_composition, n: usize, out_layer_ids: *mut u32) -> cgb_status;

    pub fn cgb_insert_in_layer(
        c: *mut cgb_composition,
        layer_id: u32,
        kinds: *const u32,
        n_cmds: usize,
        points: *const f32,
        n_point_floats: usize,
        transform9: *const f32,
    ) -> cgb_status;
    pub fn cgb_insert_paths(
        c: *mut cgb_composition,
        n_paths: usize,
        layer_ids: *const u32,
        cmd_offsets: *const u64,
        kinds: *const u32,
        point_offsets: *const u64,
        points: *const f32,
        transforms9: *const f32,
        has_transform: *const u8,
    ) -> cgb_status;
    pub fn cgb_insert_lines(c: *mut cgb_composition, layer_id: u32, segments: *const f32, n_lines: usize) -> cgb_status;

    pub fn cgb_insert_layer_copies(
        c: *mut cgb_composition,
        n: usize,
        layer_ids: *const u32,
        src: *mut cgb_composition,
        src_layer_ids: *const u32,
    ) -> cgb_status;

    pub fn cgb_layer_set_enabled(c: *mut cgb_composition, layer_id: u32, enabled: c_int) -> cgb_status;
    pub fn cgb_layer_set_transform(c: *mut cgb_composition, layer_id: u32, affine6: *const f32, flags: u32) -> cgb_status;
    pub fn cgb_layer_set_order(c: *mut cgb_composition, layer_id: u32, order: u32) -> cgb_status;
    pub fn cgb_layer_set_props(c: *mut cgb_composition, layer_id: u32, props: *const cgb_props) -> cgb_status;
    pub fn cgb_layers_set_enabled(c: *mut cgb_composition, n: usize, layer_ids: *const u32, enabled: *const u8) -> cgb_status;
    pub fn cgb_layers_set_props(c: *mut cgb_composition, n: usize, layer_ids: *const u32, props: *const cgb_props) -> cgb_status;
    pub fn cgb_layers_set_transforms(
        c: *mut cgb_composition,
        n: usize,
        layer_ids: *const u32,
        affine6: *const f32,
        flags: u32,
    ) -> cgb_status;

    pub fn cgb_update_layers(n: usize, updates: *const cgb_layer_update) -> cgb_status;
    pub fn cgb_remove_disabled(c: *mut cgb_composition) -> cgb_status;
    pub fn cgb_lines_len(c: *mut cgb_composition, builder_len: *mut u64, actual_len: *mut u64) -> cgb_status;

    pub fn cgb_create_buffer_layer_cache(c: *mut cgb_composition, out_cache_id: *mut i32) -> cgb_status;
    pub fn cgb_release_buffer_layer_cache(c: *mut cgb_composition, cache_id: i32) -> cgb_status;

    pub fn cgb_render(
        c: *mut cgb_composition,
        buffer: *const cgb_buffer,
        background: *const f32,
        crop: *const cgb_rect,
    ) -> cgb_status;
    pub fn cgb_render_batch(
        ctx: *mut cgb_composition,
        n: usize,
        scenes: *const *mut cgb_composition,
        buffers: *const cgb_buffer,
        backgrounds: *const f32,
        crops: *const cgb_rect,
    ) -> cgb_status;
    pub fn cgb_pixel_segments(
        c: *mut cgb_composition,
        out: *mut u64,
        cap: usize,
        out_len: *mut u64,
        out_none: *mut u64,
        order: u32,
    ) -> cgb_status;

    pub fn cgb_get_stats(c: *mut cgb_composition, out: *mut cgb_stats) -> cgb_status;
    pub fn cgb_set_graph_mode(c: *mut cgb_composition, enabled: c_int, headroom: f32) -> cgb_status;
    pub fn cgb_set_incremental(c: *mut cgb_composition, enabled: c_int) -> cgb_status;
    pub fn cgb_set_tuning(c: *mut cgb_composition, tuning: *const cgb_tuning) -> cgb_status;
    pub fn cgb_get_tuning(c: *mut cgb_composition, out: *mut cgb_tuning) -> cgb_status;
    pub fn cgb_synchronize(c: *mut cgb_composition) -> cgb_status;
    pub fn cgb_get_stream(c: *mut cgb_composition, out_stream: *mut *mut c_void) -> cgb_status;
    pub fn cgb_get_memory(c: *mut cgb_composition, device_bytes: *mut u64) -> cgb_status;
    pub fn cgb_kernel_launches() -> u64;

    pub fn cgb_sort_keys_noalloc(
        keys: *mut u64,
        out: *mut u64,
        n: usize,
        bit_lo: u32,
        bit_hi: u32,
        stream: *mut c_void,
    ) -> cgb_status;

    pub fn cgb_cassia_render(
        c: *mut cgb_composition,
        segments: *const u64,
        n: usize,
        stylings: *const cgb_cassia_styling,
        m: usize,
        buffer: *const cgb_buffer,
        background: *const f32,
    ) -> cgb_status;

    pub fn cgb_selftest_bounded_wait() -> cgb_status;
    pub fn cgb_composition_clear(c: *mut cgb_composition) -> cgb_status;
}
