// Internal declarations shared by the CUDA translation units of cassia_gb300.
//
// All device arithmetic reproduces the reference (Rust, surpass/mold) bit for
// bit: the library is compiled with -fmad=false so that no a*b+c is
// contracted, and every `mul_add` of the reference is an explicit __fmaf_rn.
// Float->int conversions use the saturating round-toward-zero cvt (NaN -> 0),
// which is Rust's `as`; roundf is round-half-away-from-zero, as f32::round.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/cassia_gb300.h"

namespace cgb {

// surpass/src/lib.rs:18-33
constexpr int PIXEL_WIDTH = 16;
constexpr int PIXEL_SHIFT = 4;
constexpr int PIXEL_MASK = 15;
constexpr int TILE_SHIFT = 3;
constexpr int TILE_MASK = 7;

// ---------------------------------------------------------------------------
// device records
// ---------------------------------------------------------------------------

// surpass::Layer (surpass/src/layer.rs:5-20) indexed by layer id.
struct alignas(16) LayerRec {  // two 16-byte loads
    uint32_t flags;  // LAYER_PRESENT | LAYER_ENABLED | LAYER_HAS_TRANSFORM
    uint32_t order;  // Layer::order (defaults to the id when LAYER_HAS_ORDER is clear)
    float t[6];      // affine_transform
};
constexpr uint32_t LAYER_PRESENT = 1u;
constexpr uint32_t LAYER_ENABLED = 2u;
constexpr uint32_t LAYER_HAS_TRANSFORM = 4u;
constexpr uint32_t LAYER_HAS_ORDER = 8u;

// Output of LinesBuilder::build for one line (surpass/src/segment.rs:208-219),
// packed into 32 bytes (two 16-byte stores and loads).  `length` lives in a
// separate array (it is scanned).
struct alignas(16) LineRec {
    int32_t start;
    float start_f32, end_f32;
    float slope, slope_recip, py_slope_px, px_slope_recip_py;
    uint32_t order_octant;  // order << 3 | octant
};
static_assert(sizeof(LineRec) == 32 && sizeof(LayerRec) == 32, "32-byte line and layer records");

// Painter-side props of one order (LayerProps::get, painter/mod.rs:143-146).
struct PaintProps {
    uint32_t fill_rule;
    uint32_t blend_mode;
    uint32_t flags;  // PROPS_*
    uint32_t aux;    // gradient fills: index of the GradRec; clip layers: the layers they clip
    float color[4];
};
// A gradient fill (style.rs:29-175): type, its stops [first, first + n) in
// the GradStop table (positions already resolved as GradientBuilder::build
// does), start and end points.
struct GradRec {
    uint32_t type, n_stops, first, pad;
    float start[2], end[2];
};
struct GradStop {
    float color[4];
    float stop;
    float pad[3];
};
constexpr uint32_t PROPS_SOLID = 1u;        // Fill::Solid
constexpr uint32_t PROPS_OPAQUE_OVER = 2u;  // Fill::Solid, BlendMode::Over, alpha == 1.0
constexpr uint32_t PROPS_DRAW = 4u;         // Func::Draw
constexpr uint32_t PROPS_PRESENT = 8u;      // an enabled layer holds this order
constexpr uint32_t PROPS_CLIP = 16u;        // Func::Clip
constexpr uint32_t PROPS_CLIPPED = 32u;     // Style::is_clipped (a Draw layer)
// SceneDesc::features
constexpr uint32_t FEAT_GRADIENTS = 1u;     // some layer has a gradient fill
constexpr uint32_t FEAT_CLIPS = 2u;         // some layer clips or is clipped

// One canvas of a frame: a composition's lines, layer table and props, its
// output buffer, and where its tile rows / tiles sit in the frame's global
// row and tile numbering.  A frame renders one or many scenes in one pipeline.
struct SceneDesc {
    const float* p0x;
    const float* p0y;
    const float* p1x;
    const float* p1y;
    const uint32_t* lids;
    const LayerRec* layers;
    const PaintProps* props;    // by order
    const GradRec* grads;       // gradient fills of props (PaintProps::grad)
    const GradStop* stops;
    const uint8_t* unchanged;   // by order, or null (no layer cache)
    int32_t* prev_layers;       // by tile, or null
    uint8_t* out;               // device RGBA8
    const float* default_t;     // LinesBuilder default transform, or null
    uint64_t line_base;         // first global line index
    uint32_t n_lines, n_layer_recs, n_orders, wide;
    uint32_t width, height, stride, rows, row_len;
    uint32_t row_base, tile_base;
    uint32_t crop_h0, crop_h1, crop_v0, crop_v1;  // in tiles
    uint32_t features;                            // FEAT_*
    float clear[4];
    uint8_t* written;                             // by tile: the painter wrote it (flushers), or null
    const uint8_t* rast_dirty;  // incremental frames: by order, 1 = rasterize its lines; null = all lines
};

// Frame-wide geometry of the render-mode segment key, bit fields from high
// to low:
//   key = global tile row | tile column + 1 | order
// (col_bits and order_bits wide), with n_orders and row_len the maxima over
// the frame's scenes.  Sorted, the segments are tile-major: each tile's
// tile-layer groups are contiguous and in paint order, as the reference's
// `u64 >> 22` sort key orders them (tile_j, tile_i, layer).
struct BatchGeom {
    const SceneDesc* scenes;     // device array
    const uint32_t* row_scene;   // device: scene of each global tile row
    uint32_t n_scenes;
    uint32_t total_rows, total_tiles;
    uint32_t n_orders, row_len;
    uint32_t order_bits, col_bits;
    uint32_t key_bits;
    uint64_t total_lines;
};

__host__ __device__ __forceinline__ uint64_t make_render_key(const BatchGeom& bg, uint32_t grow, uint32_t order,
                                                             uint32_t col1) {
    return ((((uint64_t)grow << bg.col_bits) | col1) << bg.order_bits) | order;
}
// The fields of a key (bits 22..63 of a segment) in a layout of order_bits /
// col_bits: its row, tile column + 1 and order, and its (row, order) run
// (row << order_bits | order), along which cover carries flow.
__host__ __device__ __forceinline__ uint32_t key_order(uint64_t key, uint32_t order_bits) {
    return (uint32_t)(key & ((1ull << order_bits) - 1));
}
__host__ __device__ __forceinline__ uint32_t key_col1(uint64_t key, uint32_t order_bits, uint32_t col_bits) {
    return (uint32_t)((key >> order_bits) & ((1ull << col_bits) - 1));
}
__host__ __device__ __forceinline__ uint32_t key_row(uint64_t key, uint32_t order_bits, uint32_t col_bits) {
    return (uint32_t)(key >> (order_bits + col_bits));
}
__host__ __device__ __forceinline__ uint64_t key_run(uint64_t key, uint32_t order_bits, uint32_t col_bits) {
    return ((uint64_t)key_row(key, order_bits, col_bits) << order_bits) | key_order(key, order_bits);
}

// LineRec.order_octant packing: scene << 20 | order << 3 | octant
constexpr int LINE_SCENE_SHIFT = 20;

// ---------------------------------------------------------------------------
// Rust-semantics numerics
// ---------------------------------------------------------------------------

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__device__ __forceinline__ int32_t wabs(int32_t a) { return a < 0 ? wsub(0, a) : a; }

// `v as i32`: truncation, saturation, NaN -> 0 (cvt.rzi.s32.f32).
__device__ __forceinline__ int32_t f2i32(float v) { return __float2int_rz(v); }
// `v as u8`
__device__ __forceinline__ uint32_t f2u8(float v) { return min(__float2uint_rz(v), 255u); }
// `v as usize` for the small positive values of curve subdivision counts.
__device__ __forceinline__ uint64_t f2usize(float v) { return __float2ull_rz(v); }

// segment.rs:13-16
__device__ __forceinline__ int32_t to_sub_pixel(float v) {
    return f2i32(__fmaf_rn(v, (float)PIXEL_WIDTH, copysignf(0.5f, v)));
}

// Low 22 bits of a CompactSegment (raster_segment.rs:142-154): tile_y | tile_x | area | cover.
__device__ __forceinline__ uint32_t low_tile_y(uint32_t low) { return (low >> 19) & 7; }
__device__ __forceinline__ uint32_t low_tile_x(uint32_t low) { return (low >> 16) & 7; }
// pixel index y * 8 + x within the tile (the two 3-bit fields side by side)
__device__ __forceinline__ uint32_t low_cell(uint32_t low) { return (low >> 16) & 63; }
__device__ __forceinline__ int32_t low_area(uint32_t low) { return (int32_t)(low << 16) >> 22; }  // bits 6..15
__device__ __forceinline__ int32_t low_cover(uint32_t low) { return (int32_t)(low << 26) >> 26; }  // bits 0..5

// 8 x i8 cover lanes packed in a u64 (lane y = byte y); lane-wise wrapping add.
__device__ __forceinline__ uint64_t cover_add(uint64_t a, uint64_t b) {
    const uint64_t H = 0x8080808080808080ull;
    return ((a & ~H) + (b & ~H)) ^ ((a ^ b) & H);
}
__device__ __forceinline__ int32_t cover_lane(uint64_t c, int y) { return (int32_t)(int8_t)(uint8_t)(c >> (8 * y)); }
// Cover::is_empty / is_full (painter/mod.rs:164-189, D2), all 8 lanes at
// once.  A lane's wrapping |v| has its low 5 bits zero iff v is a multiple
// of 32 and equal to 16 iff v is 16 modulo 32, since -v = v modulo 32 for
// those values; NonZero's |v| == 16 holds iff the byte is 0x10 or 0xF0 (after
// XOR 0x10: 0x00 or 0xE0, whose low 5 bits are zero and bits 5..7 equal).
__device__ __forceinline__ bool cover_is_empty(uint64_t c, uint32_t fill_rule) {
    if (fill_rule == CGB_FILL_NONZERO) return c == 0;
    return (c & 0x1F1F1F1F1F1F1F1Full) == 0;
}
__device__ __forceinline__ bool cover_is_full(uint64_t c, uint32_t fill_rule) {
    if (fill_rule == CGB_FILL_NONZERO) {
        const uint64_t t = c ^ 0x1010101010101010ull;
        return (t & 0x1F1F1F1F1F1F1F1Full) == 0 && ((t ^ (t >> 1)) & 0x6060606060606060ull) == 0;
    }
    return (c & 0x1F1F1F1F1F1F1F1Full) == 0x1010101010101010ull;
}

// ---------------------------------------------------------------------------
// host-side launchers (defined in the .cu files)
// ---------------------------------------------------------------------------

// A grow-only device buffer accounted against the handle's HBM budget.
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <class T>
    T* as() const { return (T*)p; }
};

// Counts of a frame kept on the device (graph frames).  The scans write S
// (pixel steps), P (painted segments), G (tile-layer groups) and W (work
// items) here instead of returning them to the host, and every kernel that
// consumes one reads it, clamped to the capacity its buffers were sized for;
// a count above its capacity sets its bit in `overflow` (the painter then
// paints nothing and the host renders the frame again with larger buffers).
// Sync-free incremental frames also count the kept resident segments
// (FC_KEPT) and the new ones (FC_NEW); FC_SEGS is then their merge.
enum { FC_STEPS = 0, FC_SEGS = 1, FC_TLS = 2, FC_ITEMS = 3, FC_KEPT = 4, FC_NEW = 5 };
struct FrameCounts {
    uint32_t n[6];
    uint32_t overflow;
    uint32_t pad;
    unsigned long long produced;  // segments the rasterizer produced, kept or not
};

// The count `k` of a frame: `cap` itself without device counts (the host's
// exact count), else the device count clamped to `cap`.
__device__ __forceinline__ uint32_t fc_count(FrameCounts* fc, int k, uint32_t cap, bool report) {
    if (!fc) return cap;
    const uint32_t v = fc->n[k];
    if (v <= cap) return v;
    if (report) atomicOr(&fc->overflow, 1u << k);
    return cap;
}

// Device scratch shared by the stages of one composition handle.
struct Scratch {
    size_t budget = 0;  // 0 = unlimited
    size_t used = 0;    // bytes held by all DevBufs of the handle
    bool over_budget = false;
    // Grows `b` to at least `bytes` (geometric growth).  Fails with
    // cudaErrorMemoryAllocation (and sets over_budget) past the budget.
    cudaError_t ensure(DevBuf& b, size_t bytes);
    void release(DevBuf& b);
    DevBuf scan_sums;  // u64 per-block sums of scan_u32
    DevBuf sort_hist, sort_lookback, sort_counter;
    uint64_t* pinned = nullptr;  // small pinned host area for readbacks
};

// Process-wide count of kernels launched by this library.
void count_launches(uint64_t n);
uint64_t launches_total();
void uncount_launches(uint64_t n);  // launches captured into a graph, counted when replayed

// k_lines.cu
cudaError_t launch_flatten(int write, const uint32_t* kinds, const float* points, const uint64_t* cmd_off,
                           const uint64_t* pt_off, const float* transforms9, const uint8_t* has_t,
                           const uint32_t* path_layer, uint32_t n_paths, uint32_t* counts, const uint32_t* out_off,
                           float* p0x, float* p0y, float* p1x, float* p1y, uint32_t* lids, cudaStream_t st);
// cull != 0 (render mode) drops lines whose segments the painter never reads.
// order_flag (zeroed by the caller), if given, is set to 1 when some line of
// a scene has a lower order than the line before it; while it stays 0 the
// rasterizer's segments come out in non-decreasing order within each scene.
cudaError_t launch_build_lines(const BatchGeom& bg, int cull, LineRec* recs, uint32_t* lengths, cudaStream_t st,
                               uint32_t* order_flag = nullptr);
// mode: 0 = count, 1 = write.  render != 0: culled, re-keyed render format;
// else the reference segment format of the (single) scene.
// Rasterizes every pixel step (`items` consecutive steps per thread, 4 or 8);
// block b stores its kept segments at runs[b * raster_run_slots(block, items)...]
// and their count at run_count[b]; *produced (zeroed by the caller)
// accumulates all segments, kept or not.
// With fc, n_steps is the capacity and the step count is fc->n[FC_STEPS].
// sparse: most lines have length 0 (an incremental frame); their runs are
// searched instead of walked.
cudaError_t launch_rasterize(int render, const BatchGeom& bg, const LineRec* recs, const uint32_t* step_off,
                             uint32_t n_lines, uint64_t n_steps, uint32_t block, uint32_t items, uint64_t* runs,
                             uint32_t* run_count, unsigned long long* produced, cudaStream_t st,
                             FrameCounts* fc, bool sparse, uint32_t* block_lines);
uint32_t raster_run_slots(uint32_t block, uint32_t items);
// Keys n reference CompactSegments (cassia_render's input) of scene 0 into
// runs of import_run_slots() slots per block, as launch_rasterize does.
cudaError_t launch_import_segments(const uint64_t* segs, uint64_t n, const BatchGeom& bg, uint64_t* runs,
                                   uint32_t* run_count, unsigned long long* produced, cudaStream_t st);
uint32_t import_grid(uint64_t n);
uint32_t import_run_slots();
uint32_t raster_grid(uint64_t n_steps, uint32_t block, uint32_t items);
cudaError_t launch_compact_lines(const float* in4[4], const uint32_t* lid_in, uint32_t n, const LayerRec* layers,
                                 uint32_t n_layer_recs, float* out4[4], uint32_t* lid_out, uint32_t* flags,
                                 uint32_t* offsets, Scratch* s, cudaStream_t st, uint32_t* n_out_host);
// Appends copies of n line runs: run k starts at src4[*][src_first[k]] and
// lands at dst4[*][dst_off[k] .. dst_off[k + 1]) with layer id dst_ids[k];
// total = dst_off[n].
cudaError_t launch_copy_lines(const float* const src4[4], const uint64_t* src_first, const uint64_t* dst_off,
                              const uint32_t* dst_ids, uint32_t n, uint64_t total, float* const dst4[4],
                              uint32_t* dst_lids, cudaStream_t st);

// k_sort.cu
// Exclusive scan of n u32 values; out has n+1 entries (out[n] = total mod 2^32).
// *total_host receives the exact 64-bit total (synchronizes); *tail_dev, if
// given, receives the total on the device as well (no synchronization).
cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, Scratch* s, cudaStream_t st,
                     uint64_t* total_host, uint32_t* tail_dev = nullptr);
// Sizes the scan and sort scratch of `s` for scans of up to scan_n values and
// sorts of up to sort_n keys (before a frame graph is captured: nothing may
// allocate while a stream captures).
cudaError_t reserve_frame_scratch(Scratch* s, uint32_t scan_n, uint32_t sort_n);
// The key bits a sort orders by, [lo, hi), with the digit passes planned
// separately for [lo, mid) and for [mid, hi).  With skip_flag, the passes of
// [lo, mid) are skipped on the device while *skip_flag == 0: the caller's
// guarantee that wherever bits [mid, hi) tie the keys already come in
// non-decreasing [lo, mid) order, so that those stable passes would move no
// key (the result is bit for bit the full sort's).
struct SortBits {
    int lo, mid, hi;
    const uint32_t* skip_flag;
};
inline SortBits sort_bits(int lo, int hi) { return SortBits{lo, lo, hi, nullptr}; }
// Sort n u64 keys by bits [sb.lo, sb.hi).  `keys` and `tmp` hold n keys;
// on return *result points at the sorted array (keys or tmp).  With
// hist_ready the digit counts of every pass are already in s->sort_hist
// (from radix_gather_hist).
// With fc, n is the capacity of keys and tmp and the key count is fc->n[fc_which].
// Pass p ranks its tile's keys with warp ballots instead of match.any when bit
// p of ballot_passes is set: for digits that the lanes of a warp mostly hold
// distinct (the low digit of the work items' tile field).
cudaError_t radix_sort_u64(uint64_t* keys, uint64_t* tmp, uint32_t n, SortBits sb, int digit_bits, Scratch* s,
                           uint32_t* err_flag, cudaStream_t st, uint64_t** result, int* passes,
                           bool hist_ready = false, FrameCounts* fc = nullptr, int fc_which = 0,
                           uint32_t ballot_passes = 0);
// Runs one onesweep CTA whose predecessor tile never publishes; *flag_host
// receives the kernel's error flag (1 = the bounded wait gave up).
cudaError_t selftest_bounded_wait(cudaStream_t st, uint32_t* flag_host);
// Packs runs of keys (run r: run_count[r] keys at runs[r * run_slots...],
// placed at run_off[r] of out) and counts the digits of every pass of the sort
// by `sb` into s->sort_hist, for radix_sort_u64(hist_ready) with the same sb.
// Keys placed at or beyond out_cap are dropped (a graph frame whose segment
// count passed its capacity; the sort reports the overflow).
cudaError_t radix_gather_hist(const uint64_t* runs, uint32_t run_slots, const uint32_t* run_count,
                              const uint32_t* run_off, uint32_t n_runs, uint64_t* out, SortBits sb, int digit_bits,
                              Scratch* s, cudaStream_t st, uint32_t out_cap = 0xFFFFFFFFu);
// The sort of a frame's render keys (bits 22..63 of its segments): bits
// [22, 22 + order_bits) hold the order, the passes that order_flag lets the
// frame skip.
inline SortBits render_sort_bits(const BatchGeom& bg, const uint32_t* order_flag) {
    return SortBits{22, 22 + (int)bg.order_bits, 22 + (int)bg.key_bits, order_flag};
}

// k_incr.cu: incremental frames
// Local key layout of a composition's resident segments after a batched
// frame (bits 22..63): tile row (12 bits) | tile column + 1 (13) | order (17).
// After a frame of the composition alone they stay in that frame's layout.
constexpr int LOCAL_ORDER_BITS = 17;
constexpr int LOCAL_COL_BITS = 13;
constexpr uint32_t LOCAL_MAX_ROWS = 1u << (42 - LOCAL_ORDER_BITS - LOCAL_COL_BITS);
constexpr uint32_t MAX_KEEP_SOURCES = 256;  // scenes of one incremental frame
// Resident segments of one scene, flattened at `start` among all sources.
struct KeepSource {
    const uint64_t* seg;
    uint64_t start, n;
    const uint8_t* dirty;  // by order: 1 = the order's segments are rasterized again
    uint32_t n_dirty;
    uint32_t row_base;     // the scene's first tile row in the frame
    uint32_t order_bits, col_bits;  // the key layout the resident segments are stored in
};
// A scene's range of the sorted frame and where its resident copy goes.
struct ExtractTarget {
    uint64_t* dst;
    uint64_t start, n, cap;  // flattened start, count, capacity of dst
    uint32_t first;          // first segment of the range in the frame
    uint32_t row_base;
};
uint32_t keep_grid(uint64_t total);
uint32_t merge_tiles(uint64_t n);
// mode 0: per block of keep_grid(total), the kept (clean-order) resident
// segments; mode 1: write them at block_off, in order, in the frame's key
// layout (out holds out_cap keys).
cudaError_t launch_keep(int mode, const KeepSource* srcs, uint32_t n_srcs, uint64_t total, const BatchGeom& bg,
                        uint32_t* block_count, const uint32_t* block_off, uint64_t* out, uint64_t out_cap,
                        cudaStream_t st);
// Stable merge of two key-sorted arrays (by bits 22..63; a first on ties);
// split holds merge_tiles(na + nb) + 1 entries.  With fc, na and nb are
// capacities (counts fc->n[FC_KEPT], fc->n[FC_NEW]) and fc->n[FC_SEGS]
// receives the merged count.
cudaError_t launch_merge(const uint64_t* a, uint32_t na, const uint64_t* b, uint32_t nb, uint32_t* split,
                         uint64_t* out, cudaStream_t st, FrameCounts* fc = nullptr);
// ranges[2k], ranges[2k + 1]: the segments of scene scene_ids[k]'s tile rows in the sorted frame.
cudaError_t launch_scene_ranges(const uint64_t* segs, uint32_t n, const BatchGeom& bg, const uint32_t* scene_ids,
                                uint32_t n_ids, uint32_t* ranges, cudaStream_t st);
cudaError_t launch_extract(const uint64_t* segs, const ExtractTarget* tg, uint32_t n_tg, uint64_t total,
                           const BatchGeom& bg, cudaStream_t st);

// k_paint.cu
// The run-record sort ranks its first pass (the order's low digit) by warp
// ballots: consecutive TLs of a tile hold distinct, increasing orders, whose
// low bits differ (their high bits repeat: match.any ranks those).
constexpr uint32_t TL_SORT_BALLOT_PASSES = 1u;
// TLs (tile-layer groups) are numbered in segment order, which is
// tile-major; tl_rec lists them along the (row, order) runs that carry
// cover from tile to tile: entry s = run << idx_bits | TL index, sorted by
// run (stably, so each run's TLs go left to right).
struct CarryBuffers {
    uint32_t* tl_start;   // [G + 1] first segment of each tile-layer group (TL)
    uint64_t* tl_key;     // [G] its segment key (bits 22..63)
    uint64_t* tl_cover;   // [G] lane-wise cover sum of its segments
    uint64_t* tl_carry;   // [G] cover entering it along its (row, order) run
    uint64_t* tl_rec;     // [G] run << idx_bits | TL: written unsorted by the TL scan, then sorted
    uint64_t* tl_skey;    // [G] by position in tl_rec: the TL's key
    uint64_t* tl_sout;    // [G] by position in tl_rec: the cover leaving the TL
    uint32_t* item_count; // [G] by position in tl_rec
    uint32_t* item_off;   // [G + 1]
    uint64_t* items;      // [W]
    uint64_t* items_tmp;  // [W]
    uint32_t* tile_start; // [tiles + 1]
    uint64_t* blk_cover;  // [tl_scan_grid] per block: cover sum before its first TL head
    uint32_t* blk_head;   // [tl_scan_grid] per block: holds a TL head
    int order_bits;       // width of the order field of keys and items
    int col_bits;         // width of the tile column field of keys
    int idx_bits;         // width of the TL index in tl_rec and in items
    // graph frames: the device counts, and the TL and item capacities (TL
    // and item writes at or beyond them are dropped); without fc, the exact
    // G and W bound every write
    FrameCounts* fc;
    uint32_t tl_cap, items_cap;
};
// n: the segment count (with cb.fc, the capacity of the segment arrays).
cudaError_t launch_tl_scan(int mode, const uint64_t* segs, uint32_t n, uint32_t* block_counts,
                           const uint32_t* block_off, const CarryBuffers& cb, cudaStream_t st);
uint32_t tl_scan_grid(uint32_t n);
// Carries along the sorted run records and each record's work-item count
// (cb.item_count); also sets tl_start[G] = P.  G, P: the counts (with cb.fc,
// the capacities).
cudaError_t launch_tl_carry(uint32_t G, uint32_t P, const CarryBuffers& cb, const BatchGeom& bg, cudaStream_t st);
// The work items at cb.item_off (the scan of cb.item_count).
cudaError_t launch_items(uint32_t G, const BatchGeom& bg, const CarryBuffers& cb, int idx_bits, cudaStream_t st);
cudaError_t launch_tile_ranges(const uint64_t* items, uint32_t W, uint32_t n_tiles, int tile_shift,
                               uint32_t* tile_start, cudaStream_t st, FrameCounts* fc = nullptr);
// full: some scene of the frame has gradient fills or clips (selects the
// painter variant that handles them); item_state: one byte per work item
// (clip pass results), needed when a scene has clips.
cudaError_t launch_paint(const BatchGeom& bg, const uint64_t* segs, const uint64_t* items, int idx_bits, uint32_t G,
                         const uint32_t* tile_start, const CarryBuffers& cb, uint32_t warps, bool full,
                         uint8_t* item_state, cudaStream_t st);


}  // namespace cgb
