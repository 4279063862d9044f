/*
 * cassia_gb300 — GB300-native (sm_103a) surpass/mold rasterize -> sort -> paint.
 *
 * C ABI.  Plain pointers and sizes only.  Every call returns a cgb_status.
 * A composition handle is single-threaded; distinct handles may be used from
 * distinct threads.  Caller-owned arrays are copied during the call.
 *
 * The entry points mirror the reference's two seams:
 *   - mold's Composition / Layer / Path / Props API
 *     (mold/src/composition.rs:26-329, mold/src/layer.rs:145-244,
 *      mold/src/path/mod.rs:25-179, surpass/src/painter/style.rs:189-432),
 *     which drives surpass's LinesBuilder::build -> Rasterizer::rasterize ->
 *     Rasterizer::sort -> BufferLayout::print;
 *   - cassia's headless consumer of sorted pixel segments
 *     (cassia/src/Cassia.h:25-41).
 * Each declaration cites the reference interface it replaces.
 */
#ifndef CASSIA_GB300_H
#define CASSIA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define CGB_EXPORT __declspec(dllexport)
#else
#define CGB_EXPORT __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------------- */
typedef int32_t cgb_status;
#define CGB_OK 0
#define CGB_ERR_INVALID_ARG 1    /* bad pointer, size, id or enum value */
#define CGB_ERR_OUT_OF_MEMORY 2  /* cudaMalloc / host allocation failed */
#define CGB_ERR_OVER_BUDGET 3    /* the handle's HBM budget would be exceeded */
#define CGB_ERR_LAYER_LIMIT 4    /* more layers / tiles than the segment format holds */
#define CGB_ERR_DEVICE_TIMEOUT 5 /* a bounded device-side wait expired (no hang) */
#define CGB_ERR_DEVICE 6         /* a CUDA runtime error */
#define CGB_ERR_NO_DEVICE 7      /* no CUDA device visible */
#define CGB_ERR_CAPACITY 8       /* caller's output array is too small (size reported) */
#define CGB_ERR_NOT_FOUND 9      /* unknown layer id / cache id */
#define CGB_ERR_SCALE 10         /* mold Layer::set_transform scale check (mold/src/layer.rs:186-190) */

/* ---- enums (values are the reference's enum order) -------------------------- */
/* surpass FillRule (surpass/src/painter/style.rs:10-13) */
#define CGB_FILL_NONZERO 0u
#define CGB_FILL_EVENODD 1u
/* surpass BlendMode (surpass/src/painter/style.rs:190-203) */
#define CGB_BLEND_OVER 0u
#define CGB_BLEND_MULTIPLY 1u
#define CGB_BLEND_SCREEN 2u
#define CGB_BLEND_OVERLAY 3u
#define CGB_BLEND_DARKEN 4u
#define CGB_BLEND_LIGHTEN 5u
#define CGB_BLEND_COLOR_DODGE 6u
#define CGB_BLEND_COLOR_BURN 7u
#define CGB_BLEND_HARD_LIGHT 8u
#define CGB_BLEND_SOFT_LIGHT 9u
#define CGB_BLEND_DIFFERENCE 10u
#define CGB_BLEND_EXCLUSION 11u
/* surpass painter Func (surpass/src/painter/mod.rs:125-129) */
#define CGB_FUNC_DRAW 0u
#define CGB_FUNC_CLIP 1u
/* surpass Fill (surpass/src/painter/style.rs:177-181) */
#define CGB_FILL_SOLID 0u
#define CGB_FILL_GRADIENT 1u
/* surpass GradientType (surpass/src/painter/style.rs:21-25) */
#define CGB_GRADIENT_LINEAR 0u
#define CGB_GRADIENT_RADIAL 1u

/* mold PathCommand (mold/src/path/mod.rs:13-21).  Floats per command, in the
 * argument order of mold's Path methods (mold/src/path/mod.rs:53-170):
 *   LINE      4: x0 y0 x1 y1
 *   QUAD      6: x0 y0 x1 y1 x2 y2
 *   RAT_QUAD  9: x0 y0 w0 x1 y1 w1 x2 y2 w2     (points are NOT pre-weighted)
 *   CUBIC     8: x0 y0 .. x3 y3
 *   RAT_CUBIC 12: x0 y0 w0 .. x3 y3 w3
 *   CLOSE     0 */
#define CGB_CMD_LINE 0u
#define CGB_CMD_QUAD 1u
#define CGB_CMD_RAT_QUAD 2u
#define CGB_CMD_CUBIC 3u
#define CGB_CMD_RAT_CUBIC 4u
#define CGB_CMD_CLOSE 5u

/* composition flags */
/* Widened segment format: layer field 17 bits (131,072 orders) in place of the
 * reference's is_none bit; every other field keeps its width and order.  Used
 * for scenes with more than 65,536 layer orders (the reference's u16 limit,
 * mold/src/layer.rs:13, surpass/src/rasterizer/raster_segment.rs:148). */
#define CGB_COMPOSITION_WIDE_LAYERS 1u
/* Stream priority of the handle's stream: work of a high-priority handle
 * (e.g. a client's scene updates) is scheduled before waiting blocks of
 * low-priority handles (e.g. a server's batch renders) on a busy GPU. */
#define CGB_COMPOSITION_PRIORITY_HIGH 2u
#define CGB_COMPOSITION_PRIORITY_LOW 4u

/* layer transform flags */
/* Skip mold's per-axis scale <= ~1 check (mold/src/layer.rs:186-190) and store
 * the affine directly in surpass::Layer::affine_transform
 * (surpass/src/layer.rs:8), which has no such limit. */
#define CGB_TRANSFORM_UNCHECKED 1u

/* pixel_segments ordering */
#define CGB_SORT_CANONICAL 0u /* ascending by the full u64 (a refinement of the reference order) */
#define CGB_SORT_KEY 1u       /* ascending by u64 >> 22, ties in rasterizer order (stable) */

/* ---- plain-data types ---------------------------------------------------------- */

/* surpass painter Props { fill_rule, func: Draw(Style) | Clip(usize) }
 * (surpass/src/painter/mod.rs:125-141) with Style { fill_rule, is_clipped,
 * fill: Solid([f32;4]) | Gradient, blend_mode } (style.rs:427-432).
 * Gradient stops are (r, g, b, a, stop) tuples; a stop < 0 (or -0.0) means
 * "no stop" and is spread evenly as GradientBuilder::build does
 * (style.rs:66-84). */
typedef struct cgb_props {
    uint32_t fill_rule;     /* CGB_FILL_NONZERO | CGB_FILL_EVENODD */
    uint32_t func;          /* CGB_FUNC_DRAW | CGB_FUNC_CLIP */
    uint32_t clip_layers;   /* Func::Clip(n) */
    uint32_t is_clipped;    /* Style::is_clipped */
    uint32_t blend_mode;    /* CGB_BLEND_* */
    uint32_t fill_kind;     /* CGB_FILL_SOLID | CGB_FILL_GRADIENT */
    float color[4];         /* Fill::Solid, linear RGBA */
    uint32_t gradient_type; /* CGB_GRADIENT_* */
    uint32_t n_stops;
    float gradient_start[2];
    float gradient_end[2];
    const float* stops; /* n_stops * 5 floats; copied by the call */
} cgb_props;

/* Output buffer (mold Buffer, mold/src/buffer.rs:19-25): `height` rows of
 * `width_stride` RGBA8 pixels of which the first `width` are painted. */
#define CGB_MEMORY_HOST 0u
#define CGB_MEMORY_DEVICE 1u
/* Page-locked host memory the device can address (cudaHostAlloc,
 * cudaHostRegister): the painter writes the pixels into it directly over the
 * host link, without a device staging buffer and a copy back.  The whole
 * buffer must lie in one page-locked allocation (its first and last byte are
 * checked: CGB_ERR_INVALID_ARG otherwise).  Flushers work as for host
 * buffers. */
#define CGB_MEMORY_HOST_MAPPED 2u
/* surpass Flusher::flush (surpass/src/painter/buffer_layout.rs:52-54): called
 * with each row slice (at most 8 pixels) of every tile the render wrote. */
typedef void (*cgb_flush_fn)(void* user, uint8_t* pixels, size_t n_pixels);

typedef struct cgb_buffer {
    uint8_t* pixels;
    uint64_t width;
    uint64_t height;
    uint64_t width_stride; /* 0 means width */
    int32_t layer_cache;   /* BufferLayerCache id, or -1 */
    uint32_t memory;       /* CGB_MEMORY_HOST | CGB_MEMORY_DEVICE | CGB_MEMORY_HOST_MAPPED */
    /* mold Buffer::flusher (mold/src/buffer.rs:19-25), host buffers only:
     * after the frame, called on the host for the row slices of every tile
     * written (not for tiles left unchanged by a layer cache or outside the
     * crop), tile by tile in row-major order.  NULL for none. */
    cgb_flush_fn flusher;
    void* flusher_user;
} cgb_buffer;

/* surpass painter Rect (surpass/src/painter/buffer_layout.rs:37-50), in
 * pixels; rounded out to whole tiles as Rect::new does. */
typedef struct cgb_rect {
    uint64_t x0, x1, y0, y1;
} cgb_rect;

/* Per-frame sizes and device stage times of the last render / pixel_segments. */
typedef struct cgb_stats {
    uint64_t lines;            /* lines in the builder (L) */
    uint64_t steps;            /* pixel steps, S = sum of line lengths */
    uint64_t segments;         /* real pixel segments, P (the reference emits 2*S slots) */
    uint64_t painted_segments; /* segments inside the canvas rows/tiles (painter input) */
    uint64_t tile_layers;      /* (tile, layer) groups that hold segments */
    uint64_t work_items;       /* (tile, layer) pairs painted, incl. cover-carry-only pairs */
    uint32_t sort_passes;      /* radix passes of the segment sort */
    uint32_t item_sort_passes; /* radix passes of the work-item sort */
    float build_ms, rasterize_ms, sort_ms, carry_ms, paint_ms, total_ms;
    uint32_t graph_replayed;   /* 1: the frame was replayed from a frame graph (cgb_set_graph_mode) */
    uint32_t graphs_cached;    /* frame graphs held by the handle */
    uint32_t incremental_form; /* 0 full frame; incremental frame (cgb_set_incremental): 1 staged,
                                  2 sync-free (no host synchronization between stages) */
    uint32_t sort_passes_skipped; /* of sort_passes, those of the order digits that the frame skipped:
                                     every scene's lines were in non-decreasing layer order, so
                                     those stable passes would have moved no segment */
} cgb_stats;

/* Autotuned knobs (0 keeps the current value).  Every setting renders the
 * same pixels; only the parallel decomposition changes. */
typedef struct cgb_tuning {
    uint32_t radix_bits;     /* widest digit of the radix sorts: 4..9 (passes split the key evenly) */
    uint32_t raster_block;   /* threads per rasterizer block: a multiple of 32 in 32..256 */
    uint32_t steps_per_block;/* pixel steps per rasterizer block: 4 or 8 x raster_block */
    uint32_t paint_warps;    /* warps (8x8 tiles) per painter block: 2, 4 or 8 */
} cgb_tuning;

typedef struct cgb_composition cgb_composition;

/* ---- library --------------------------------------------------------------------- */

/* Version string and the last error message of this thread. */
CGB_EXPORT const char* cgb_version(void);
CGB_EXPORT const char* cgb_last_error(void);

/* ---- mold::Composition ------------------------------------------------------------ */

/* Composition::new (mold/src/composition.rs:36-48).  `hbm_budget_bytes` caps the
 * device memory the handle may hold (0 = unlimited).  Binds the current device. */
CGB_EXPORT cgb_status cgb_composition_new(uint32_t flags, uint64_t hbm_budget_bytes,
                                          cgb_composition** out);
CGB_EXPORT cgb_status cgb_composition_free(cgb_composition* c);

/* Composition::create_layer (mold/src/composition.rs:54-56), IdSet::acquire
 * (mold/src/layer.rs:61-72).  Ids are handed out lowest-free-first. */
CGB_EXPORT cgb_status cgb_create_layer(cgb_composition* c, uint32_t* out_layer_id);
/* n create_layer calls; out_layer_ids receives n ids (stops at the first failure). */
CGB_EXPORT cgb_status cgb_create_layers(cgb_composition* c, size_t n, uint32_t* out_layer_ids);

/* Composition::insert_in_layer / insert_in_layer_transformed
 * (mold/src/composition.rs:58-94): flattens the path on the GPU
 * (PathSegments, mold/src/path/segments.rs) and pushes the lines.
 * `transform9` may be NULL. */
CGB_EXPORT cgb_status cgb_insert_in_layer(cgb_composition* c, uint32_t layer_id,
                                          const uint32_t* kinds, size_t n_cmds,
                                          const float* points, size_t n_point_floats,
                                          const float* transform9);

/* Batched insert_in_layer over many paths: path k owns commands
 * [cmd_offsets[k], cmd_offsets[k+1]) and floats [point_offsets[k],
 * point_offsets[k+1]); `transforms9` is NULL or 9 floats per path, used where
 * has_transform[k] != 0. */
CGB_EXPORT cgb_status cgb_insert_paths(cgb_composition* c, size_t n_paths,
                                       const uint32_t* layer_ids, const uint64_t* cmd_offsets,
                                       const uint32_t* kinds, const uint64_t* point_offsets,
                                       const float* points, const float* transforms9,
                                       const uint8_t* has_transform);

/* LinesBuilder::push (surpass/src/segment.rs:47-53) of already-flattened lines
 * (x0 y0 x1 y1 per line) into a layer, with insert_segments' bookkeeping. */
CGB_EXPORT cgb_status cgb_insert_lines(cgb_composition* c, uint32_t layer_id,
                                       const float* segments, size_t n_lines);

/* Composition::insert_in_layer (mold/src/composition.rs:58-94) of a path
 * that is already flattened: appends to layer layer_ids[k] a copy of the lines
 * that `src` holds for its layer src_layer_ids[k] (src may be `c`), device to
 * device, without flattening again and without waiting for the device.  A
 * source layer's lines must be one run: lines inserted by one call (or by
 * consecutive calls with nothing inserted in between), not moved since by
 * cgb_remove_disabled's garbage collection (CGB_ERR_INVALID_ARG otherwise).
 * Both handles are on one device; `src` must not be used by another thread
 * during the call. */
CGB_EXPORT cgb_status cgb_insert_layer_copies(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                              cgb_composition* src, const uint32_t* src_layer_ids);

/* Layer setters (mold/src/layer.rs:158-231).  set_transform(NULL) = identity. */
CGB_EXPORT cgb_status cgb_layer_set_enabled(cgb_composition* c, uint32_t layer_id, int enabled);
CGB_EXPORT cgb_status cgb_layer_set_transform(cgb_composition* c, uint32_t layer_id,
                                              const float* affine6, uint32_t flags);
CGB_EXPORT cgb_status cgb_layer_set_order(cgb_composition* c, uint32_t layer_id, uint32_t order);
CGB_EXPORT cgb_status cgb_layer_set_props(cgb_composition* c, uint32_t layer_id,
                                          const cgb_props* props);
/* Batched Layer::set_is_enabled: enabled[k] (0/1) applies to layer_ids[k]. */
CGB_EXPORT cgb_status cgb_layers_set_enabled(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                             const uint8_t* enabled);
/* Batched set_props: props[k] applies to layer_ids[k]. */
CGB_EXPORT cgb_status cgb_layers_set_props(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                           const cgb_props* props);
/* Batched set_transform for n layers (6 floats each); flags as above.  The
 * result equals n set_transform calls in order (up to the first error).  A
 * long list (16,384 ids or more) of existing layers with increasing ids is
 * checked and applied by a process-wide pool of host threads. */
CGB_EXPORT cgb_status cgb_layers_set_transforms(cgb_composition* c, size_t n,
                                                const uint32_t* layer_ids, const float* affine6,
                                                uint32_t flags);

/* One composition's changes between two frames, as a client sends them: new
 * transforms for some layers (Layer::set_transform, mold/src/layer.rs:180-197),
 * layers removed (Layer::disable, then Composition::remove_disabled,
 * mold/src/composition.rs:124-142), and layers added (Composition::create_layer
 * and insert_in_layer, composition.rs:54-94) whose paths are already
 * flattened in layers of `added_from` (as cgb_insert_layer_copies), with their
 * props and transforms (either may be NULL).  `transform_flags` apply to both
 * transform lists.  The new layers' ids are written to `added_ids`. */
typedef struct cgb_layer_update {
    cgb_composition* comp;
    size_t n_transforms;
    const uint32_t* transform_ids;
    const float* transforms; /* 6 floats per id */
    uint32_t transform_flags;
    uint32_t reserved;
    size_t n_removed;
    const uint32_t* removed_ids;
    size_t n_added;
    cgb_composition* added_from;
    const uint32_t* added_from_ids;
    const cgb_props* added_props;
    const float* added_transforms; /* 6 floats per added layer */
    uint32_t* added_ids;           /* out: n_added ids */
} cgb_layer_update;

/* Applies n updates in order, each exactly as the separate calls would
 * (cgb_layers_set_transforms, cgb_layers_set_enabled + cgb_remove_disabled,
 * cgb_create_layers + cgb_insert_layer_copies + cgb_layers_set_props +
 * cgb_layers_set_transforms), in one call: a server applies the updates of a
 * whole batch of clients at once.  Stops at the first failing update (the
 * message names it). */
CGB_EXPORT cgb_status cgb_update_layers(size_t n, const cgb_layer_update* updates);

/* Composition::remove_disabled (mold/src/composition.rs:124-142). */
CGB_EXPORT cgb_status cgb_remove_disabled(cgb_composition* c);
/* LinesBuilder::len and Composition::actual_len (composition.rs:116-121). */
CGB_EXPORT cgb_status cgb_lines_len(cgb_composition* c, uint64_t* builder_len,
                                    uint64_t* actual_len);

/* Composition::create_buffer_layer_cache (composition.rs:144-151) and the
 * BufferLayerCache drop (mold/src/buffer.rs:62-71). */
CGB_EXPORT cgb_status cgb_create_buffer_layer_cache(cgb_composition* c, int32_t* out_cache_id);
CGB_EXPORT cgb_status cgb_release_buffer_layer_cache(cgb_composition* c, int32_t cache_id);

/* Composition::render (mold/src/composition.rs:212-329): build lines,
 * rasterize, sort and paint on the GPU into `buffer` (host or device memory).
 * `background` is linear RGBA; `crop` may be NULL. */
CGB_EXPORT cgb_status cgb_render(cgb_composition* c, const cgb_buffer* buffer,
                                 const float background[4], const cgb_rect* crop);

/* Composition::render for n compositions at once: every scene is built,
 * rasterized, sorted and painted in one pipeline (one set of launches) on
 * `ctx`'s stream and scratch buffers; `ctx` may be one of the scenes or an
 * empty composition.  scenes[k] renders into buffers[k] with background
 * backgrounds[4k..4k+3] and crop crops[k] (crops may be NULL).  The
 * reference renders one Composition per call (mold/src/composition.rs:212-329);
 * each scene's pixels equal its own cgb_render. */
CGB_EXPORT cgb_status cgb_render_batch(cgb_composition* ctx, size_t n, cgb_composition* const* scenes,
                                       const cgb_buffer* buffers, const float* backgrounds,
                                       const cgb_rect* crops);

/* Composition::pixel_segments (mold/src/composition.rs:153-188): the real
 * pixel segments after build + rasterize + sort, copied to the host array
 * `out` (capacity `cap` u64).  `*out_len` receives P even when cap < P (then
 * CGB_ERR_CAPACITY).  `*out_none` receives the NONE slots (2*S - P) that the
 * reference's array ends with.  `order` is CGB_SORT_CANONICAL or CGB_SORT_KEY. */
CGB_EXPORT cgb_status cgb_pixel_segments(cgb_composition* c, uint64_t* out, size_t cap,
                                         uint64_t* out_len, uint64_t* out_none, uint32_t order);

/* Sizes and stage times of the last render / pixel_segments. */
CGB_EXPORT cgb_status cgb_get_stats(cgb_composition* c, cgb_stats* out);
/* Frame graphs (replaces the per-stage launches of mold's Composition::render,
 * mold/src/composition.rs:212-329, by one CUDA graph launch).  With enabled
 * != 0, a frame whose geometry repeats -- the same compositions, line counts,
 * canvases, clear-colour-independent layout and tuning -- is replayed from a
 * CUDA graph captured after the first frame of that geometry.  The graph
 * keeps every count of the frame on the device (no host synchronization
 * between stages); its buffers are sized `headroom` (a fraction, e.g. 0.125)
 * above the counts of the frame it was captured after.  A replayed frame
 * whose counts pass them paints nothing and is rendered again stage by stage,
 * then captured anew.  Pixels are identical in both forms.  Up to 32
 * geometries are kept per handle (cgb_render_batch groups included). */
CGB_EXPORT cgb_status cgb_set_graph_mode(cgb_composition* c, int enabled, float headroom);
/* Incremental frames (replaces the full re-rasterization of every frame in
 * mold's Composition::render, mold/src/composition.rs:212-329).  With
 * enabled != 0 the handle keeps the sorted segments of its last frame on the
 * device; the next frame on the same canvas rasterizes and sorts only the
 * lines of layers whose geometry changed since (transform, enabled, order,
 * inserted lines, removal), drops those layers' old segments and merges the
 * rest back in.  Pixels are identical to a full frame.  Works for cgb_render
 * and for the compositions of cgb_render_batch; such frames are staged (no
 * frame graph); once earlier incremental frames of a handle rendered on its own
 * have sized its buffers, they run without host synchronization between
 * stages (a frame whose counts outgrow them is rendered again stage by
 * stage).  Costs 8 bytes of device memory per segment of the frame. */
CGB_EXPORT cgb_status cgb_set_incremental(cgb_composition* c, int enabled);
CGB_EXPORT cgb_status cgb_set_tuning(cgb_composition* c, const cgb_tuning* tuning);
CGB_EXPORT cgb_status cgb_get_tuning(cgb_composition* c, cgb_tuning* out);

/* Synchronize the handle's stream (device buffers written by render are ready). */
CGB_EXPORT cgb_status cgb_synchronize(cgb_composition* c);

/* The cudaStream_t the handle launches on (for callers that order their own
 * work or timing events after a render). */
CGB_EXPORT cgb_status cgb_get_stream(cgb_composition* c, void** out_stream);

/* Device memory the handle holds (its lines, layer tables, frame buffers,
 * resident segments): what its HBM budget is checked against. */
CGB_EXPORT cgb_status cgb_get_memory(cgb_composition* c, uint64_t* device_bytes);

/* Kernels this library has launched in the process (all handles). */
CGB_EXPORT uint64_t cgb_kernel_launches(void);

/* Sorts n u64 keys in device memory by bits [bit_lo, bit_hi) with the same
 * onesweep radix sort the pipeline uses, without allocating any memory.  This
 * entry point has no counterpart in the reference.  It is for callers that
 * cannot allocate device memory while they run (memory reserved up front by a
 * render loop, or owned by another allocator, where cudaMalloc fails or, like
 * cudaFree, synchronizes the device).  `keys` (input, n u64) is overwritten:
 * the sort ping-pongs between it and `out` (n u64), which receives the sorted
 * keys; both are on the current device and must not overlap (overlapping
 * ranges return CGB_ERR_INVALID_ARG).  At most 16,777,216 keys (larger n
 * returns CGB_ERR_CAPACITY before any work).  The scratch is one static device
 * array of about 5 MB held by every GPU that loads the library; the first call
 * on a device looks up its address, so make that first call before any stream
 * capture.  Calls share the array: calls whose work overlaps on the GPU race,
 * so serialize them.  Runs on `stream` (a cudaStream_t, NULL for the default
 * stream) and returns once the sort is complete: it reads an error flag back
 * and waits for the stream, so a call on a stream that is capturing returns
 * CGB_ERR_INVALID_ARG before any work. */
CGB_EXPORT cgb_status cgb_sort_keys_noalloc(uint64_t* keys, uint64_t* out, size_t n, uint32_t bit_lo,
                                            uint32_t bit_hi, void* stream);

/* cassia's styling record (cassia/src/Cassia.h:25-30): a Solid fill, the
 * fill rule and the blend mode of one layer order. */
typedef struct cgb_cassia_styling {
    float fill[4];
    uint32_t fill_rule;
    uint32_t blend_mode;
    uint32_t _padding[2];
} cgb_cassia_styling;

/* cassia_render (cassia/src/Cassia.h:34-39), headless: paints pixel segments
 * produced elsewhere (reference CompactSegments as pixel_segments returns
 * them, in any order, NONE slots allowed; the widened format when the handle
 * was created with CGB_COMPOSITION_WIDE_LAYERS) with stylings[order] as
 * Props { fill_rule, Draw(Style { Solid(fill), blend_mode }) } into `buffer`
 * over `background`.  Segments of orders >= m are dropped.  The handle's own
 * layers are not used.  Both arrays are read during the call. */
CGB_EXPORT cgb_status cgb_cassia_render(cgb_composition* c, const uint64_t* segments, size_t n,
                                        const cgb_cassia_styling* stylings, size_t m, const cgb_buffer* buffer,
                                        const float background[4]);

/* Diagnostic: exercises the bounded device-side wait of the sort's decoupled
 * look-back.  One sort CTA waits on a predecessor tile that never publishes;
 * after its iteration limit (well under a second) it records the expiry in an
 * error flag and returns, without trapping.  Returns CGB_ERR_DEVICE_TIMEOUT
 * when the wait expired as designed and the device then still sorts
 * correctly, CGB_ERR_DEVICE otherwise.  No counterpart in the reference
 * (whose waits are host-side). */
CGB_EXPORT cgb_status cgb_selftest_bounded_wait(void);

/* Drops every layer and line, as Lines::cleared does for the builder
 * (surpass/src/segment.rs:282-301); device buffers are kept for reuse. */
CGB_EXPORT cgb_status cgb_composition_clear(cgb_composition* c);

#ifdef __cplusplus
}
#endif
#endif /* CASSIA_GB300_H */
