// Incremental frames: re-rasterize only the layers whose geometry changed.
//
// A composition in incremental mode keeps the sorted segments of its last
// frame on the device ("resident" segments): after a frame of its own, that
// frame's sorted segments as they are (a buffer swap); after a batched
// frame, its range of the batch re-keyed to a fixed local layout, bits
// 22..63 = row:12 | tile column + 1:13 | order:17.  The next
// frame rasterizes only the lines of changed layers (their orders are marked
// dirty; a layer whose order changed marks both orders), sorts those
// segments, keeps the resident segments of clean orders, re-keys them into
// the frame's key space and merges the two sorted streams (re-keying keeps
// the tile-major order: row, tile column, order).  Keys of one
// order never come from both streams, so the merge needs no tie rule beyond
// "kept first"; within one tile-layer group the order of segments does not
// change any pixel (their areas and covers are summed).  Afterwards the
// merged frame is the composition's new resident segments (a frame of its
// own), or each composition's range of it (its tile rows) is copied back,
// re-keyed to the local layout (a batched frame).
//
// In a batch, scenes occupy disjoint, increasing row ranges of the frame key,
// so the kept segments of all scenes, taken scene after scene, are already
// sorted: one merge serves the batch.
//
// Replaces the reference's full re-rasterization of every frame
// (mold/src/composition.rs:212-329 rebuilds all lines; LinesBuilder::build,
// surpass/src/segment.rs:91-237).  The painter's own incremental cache
// (tile_unchanged_pass) is independent of this.
#include <algorithm>

#include "cgb_internal.cuh"

namespace cgb {

namespace {

constexpr int KEEP_THREADS = 256;
constexpr int KEEP_ITEMS = 8;
constexpr int KEEP_TILE = KEEP_THREADS * KEEP_ITEMS;
constexpr int MERGE_THREADS = 256;
constexpr int MERGE_ITEMS = 4;
constexpr int MERGE_TILE = MERGE_THREADS * MERGE_ITEMS;

__device__ __forceinline__ uint64_t local_key(uint32_t row, uint32_t order, uint32_t col1) {
    return ((uint64_t)row << (LOCAL_ORDER_BITS + LOCAL_COL_BITS)) | ((uint64_t)col1 << LOCAL_ORDER_BITS) | order;
}

// The resident source of flattened index g: the last descriptor whose start is <= g.
__device__ __forceinline__ uint32_t keep_source(const KeepSource* s, uint32_t n, uint64_t g) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s[mid].start <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Whether resident segment v of source `src` is kept (its order is clean),
// and its key re-packed into the frame's layout.
__device__ __forceinline__ bool keep_segment(const KeepSource& src, const BatchGeom& bg, uint64_t v, uint64_t* out) {
    const uint64_t k = v >> 22;
    const uint32_t col1 = key_col1(k, src.order_bits, src.col_bits);
    const uint32_t order = key_order(k, src.order_bits);
    const uint32_t row = key_row(k, src.order_bits, src.col_bits);
    if (order >= src.n_dirty || src.dirty[order]) return false;
    *out = (make_render_key(bg, src.row_base + row, order, col1) << 22) | (v & 0x3FFFFFull);
    return true;
}

// mode 0: kept segments per block; mode 1: write them at block_off[block],
// in order, re-keyed.  Each thread owns KEEP_ITEMS consecutive segments.
template <int MODE>
__global__ void __launch_bounds__(KEEP_THREADS) k_keep(const KeepSource* __restrict__ srcs, uint32_t n_srcs,
                                                       uint64_t total, BatchGeom bg, uint32_t* __restrict__ block_count,
                                                       const uint32_t* __restrict__ block_off,
                                                       uint64_t* __restrict__ out, uint64_t out_cap) {
    __shared__ KeepSource s_src[MAX_KEEP_SOURCES];
    for (uint32_t i = threadIdx.x; i < n_srcs; i += blockDim.x) s_src[i] = srcs[i];
    __syncthreads();
    const uint64_t g0 = ((uint64_t)blockIdx.x * KEEP_THREADS + threadIdx.x) * KEEP_ITEMS;
    uint64_t keys[KEEP_ITEMS];
    uint32_t keep = 0, cnt = 0;
    if (g0 < total) {
        uint32_t si = keep_source(s_src, n_srcs, g0);
        const KeepSource& s0 = s_src[si];
        const uint64_t i0 = g0 - s0.start;
        const uint64_t* p0 = s0.seg + i0;
        if (i0 + KEEP_ITEMS <= s0.n && (((uintptr_t)p0) & 15) == 0) {
            // the thread's segments lie in one source: 16-byte pairs
            uint64_t v[KEEP_ITEMS];
            const ulonglong2* p2 = reinterpret_cast<const ulonglong2*>(p0);
#pragma unroll
            for (int k = 0; k < KEEP_ITEMS / 2; k++) {
                const ulonglong2 w = p2[k];
                v[2 * k] = w.x;
                v[2 * k + 1] = w.y;
            }
#pragma unroll
            for (int k = 0; k < KEEP_ITEMS; k++)
                if (keep_segment(s0, bg, v[k], &keys[k])) {
                    keep |= 1u << k;
                    cnt++;
                }
        } else {
#pragma unroll
            for (int k = 0; k < KEEP_ITEMS; k++) {
                const uint64_t g = g0 + k;
                if (g >= total) break;
                while (si + 1 < n_srcs && s_src[si + 1].start <= g) si++;
                const KeepSource& src = s_src[si];
                const uint64_t i = g - src.start;
                if (i < src.n && keep_segment(src, bg, src.seg[i], &keys[k])) {
                    keep |= 1u << k;
                    cnt++;
                }
            }
        }
    }
    // block-wide exclusive scan of the kept counts
    __shared__ uint32_t w_sum[KEEP_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) w_sum[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int w = 0; w < KEEP_THREADS / 32; w++) {
            const uint32_t v = w_sum[w];
            w_sum[w] = run;
            run += v;
        }
        if (MODE == 0) block_count[blockIdx.x] = run;
    }
    __syncthreads();
    if (MODE == 0) return;
    // the block's kept keys in order in shared memory, then out coalesced
    __shared__ uint64_t s_keep[KEEP_TILE];
    uint32_t o = w_sum[warp] + inc - cnt;
#pragma unroll
    for (int k = 0; k < KEEP_ITEMS; k++)
        if (keep & (1u << k)) s_keep[o++] = keys[k];
    __shared__ uint32_t s_total;
    if (threadIdx.x == KEEP_THREADS - 1) s_total = o;
    __syncthreads();
    const uint64_t base = block_off[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < s_total; i += KEEP_THREADS)
        if (base + i < out_cap) out[base + i] = s_keep[i];
}

__device__ __forceinline__ uint64_t mkey(uint64_t v) { return v >> 22; }

// Merge path: the number of elements of a taken from the first d outputs
// (ties: a first).
__device__ __forceinline__ uint32_t merge_split(const uint64_t* a, uint32_t na, const uint64_t* b, uint32_t nb,
                                                uint32_t d) {
    uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (mkey(a[mid]) <= mkey(b[d - 1 - mid])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// With fc (sync-free frames) na and nb are capacities and the counts are
// fc->n[FC_KEPT] and fc->n[FC_NEW]; thread 0 then records the merged count
// in fc->n[FC_SEGS] for the stages after the merge.
__global__ void k_merge_split(const uint64_t* __restrict__ a, uint32_t na, const uint64_t* __restrict__ b,
                              uint32_t nb, uint32_t n_tiles, uint32_t* __restrict__ split, FrameCounts* fc) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    na = fc_count(fc, FC_KEPT, na, false);
    nb = fc_count(fc, FC_NEW, nb, false);
    if (fc && t == 0) fc->n[FC_SEGS] = na + nb;
    if (t > n_tiles) return;
    const uint64_t d = min((uint64_t)t * MERGE_TILE, (uint64_t)na + nb);
    split[t] = merge_split(a, na, b, nb, (uint32_t)d);
}

// One MERGE_TILE of outputs per block: its parts of a and b in shared memory,
// each thread merges MERGE_ITEMS outputs from its own split of the tile, and
// the tile goes out coalesced.
__global__ void __launch_bounds__(MERGE_THREADS) k_merge(const uint64_t* __restrict__ a, uint32_t na,
                                                         const uint64_t* __restrict__ b, uint32_t nb,
                                                         const uint32_t* __restrict__ split,
                                                         uint64_t* __restrict__ out, const FrameCounts* fc) {
    __shared__ uint64_t s_in[MERGE_TILE];
    __shared__ uint64_t s_out[MERGE_TILE];
    if (fc) {  // the counts, clamped to the capacities the grid was sized for
        na = min(fc->n[FC_KEPT], na);
        nb = min(fc->n[FC_NEW], nb);
    }
    const uint64_t n = (uint64_t)na + nb;
    const uint64_t d0 = (uint64_t)blockIdx.x * MERGE_TILE;
    if (d0 >= n) return;
    const uint32_t dn = (uint32_t)min((uint64_t)MERGE_TILE, n - d0);
    // the tile's ranges: a[i0, i1), b[j0, j1) with (i1 - i0) + (j1 - j0) = dn
    const uint32_t i0 = min(split[blockIdx.x], na), i1 = min(max(split[blockIdx.x + 1], i0), na);
    const uint32_t ca = min(i1 - i0, dn);
    const uint32_t j0 = (uint32_t)min(d0 - i0, (uint64_t)nb);
    const uint32_t cb = min(dn - ca, nb - j0);
    for (uint32_t k = threadIdx.x; k < ca; k += MERGE_THREADS) s_in[k] = a[i0 + k];
    for (uint32_t k = threadIdx.x; k < cb; k += MERGE_THREADS) s_in[ca + k] = b[j0 + k];
    __syncthreads();
    const uint64_t* sa = s_in;
    const uint64_t* sb = s_in + ca;
    const uint32_t m = ca + cb;
    const uint32_t t0 = min((uint32_t)threadIdx.x * MERGE_ITEMS, m);
    uint32_t ia = merge_split(sa, ca, sb, cb, t0), ib = t0 - ia;
    for (int k = 0; k < MERGE_ITEMS; k++) {
        const uint32_t d = t0 + k;
        if (d >= m) break;
        const bool take_a = ib >= cb || (ia < ca && mkey(sa[ia]) <= mkey(sb[ib]));
        s_out[d] = take_a ? sa[ia++] : sb[ib++];
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < m; k += MERGE_THREADS) out[d0 + k] = s_out[k];
}

// Range [first, last) of the segments of each scene's tile rows in the
// sorted frame (lower bounds of the row-range keys).
__global__ void k_scene_ranges(const uint64_t* __restrict__ segs, uint32_t n, BatchGeom bg,
                               const uint32_t* __restrict__ scene_ids, uint32_t n_ids, uint32_t* __restrict__ ranges) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n_ids) return;
    const uint32_t s = scene_ids[t >> 1];
    const SceneDesc& S = bg.scenes[s];
    const uint64_t row = (uint64_t)S.row_base + ((t & 1) ? S.rows : 0u);
    const uint64_t key = row << (bg.order_bits + bg.col_bits);
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (mkey(segs[mid]) < key) lo = mid + 1;
        else hi = mid;
    }
    ranges[t] = lo;
}

// Copies each scene's range of the frame back to its resident segments,
// re-keyed to the local layout.  Flattened over the scenes (start prefix).
__global__ void k_extract(const uint64_t* __restrict__ segs, const ExtractTarget* __restrict__ tg, uint32_t n_tg,
                          uint64_t total, BatchGeom bg) {
    __shared__ ExtractTarget s_tg[MAX_KEEP_SOURCES];
    for (uint32_t i = threadIdx.x; i < n_tg; i += blockDim.x) s_tg[i] = tg[i];
    __syncthreads();
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    uint32_t lo = 0, hi = n_tg;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_tg[mid].start <= g) lo = mid;
        else hi = mid;
    }
    const ExtractTarget& T = s_tg[lo];
    const uint64_t i = g - T.start;
    if (i >= T.n || i >= T.cap) return;
    const uint64_t v = segs[T.first + i];
    const uint64_t k = v >> 22;
    const uint32_t col1 = key_col1(k, bg.order_bits, bg.col_bits);
    const uint32_t order = key_order(k, bg.order_bits), row = key_row(k, bg.order_bits, bg.col_bits) - T.row_base;
    T.dst[i] = (local_key(row, order, col1) << 22) | (v & 0x3FFFFFull);
}

}  // namespace

cudaError_t launch_keep(int mode, const KeepSource* srcs, uint32_t n_srcs, uint64_t total, const BatchGeom& bg,
                        uint32_t* block_count, const uint32_t* block_off, uint64_t* out, uint64_t out_cap,
                        cudaStream_t st) {
    if (total == 0) return cudaSuccess;
    if (n_srcs == 0 || n_srcs > MAX_KEEP_SOURCES) return cudaErrorInvalidValue;
    count_launches(1);
    const uint32_t grid = keep_grid(total);
    if (mode == 0)
        k_keep<0><<<grid, KEEP_THREADS, 0, st>>>(srcs, n_srcs, total, bg, block_count, block_off, out, out_cap);
    else
        k_keep<1><<<grid, KEEP_THREADS, 0, st>>>(srcs, n_srcs, total, bg, block_count, block_off, out, out_cap);
    return cudaGetLastError();
}

uint32_t keep_grid(uint64_t total) { return (uint32_t)((total + KEEP_TILE - 1) / KEEP_TILE); }

uint32_t merge_tiles(uint64_t n) { return (uint32_t)((n + MERGE_TILE - 1) / MERGE_TILE); }

cudaError_t launch_merge(const uint64_t* a, uint32_t na, const uint64_t* b, uint32_t nb, uint32_t* split,
                         uint64_t* out, cudaStream_t st, FrameCounts* fc) {
    const uint32_t tiles = merge_tiles((uint64_t)na + nb);
    if (tiles == 0 && !fc) return cudaSuccess;
    count_launches(2);
    k_merge_split<<<(tiles + 1 + 255) / 256, 256, 0, st>>>(a, na, b, nb, tiles, split, fc);
    if (tiles) k_merge<<<tiles, MERGE_THREADS, 0, st>>>(a, na, b, nb, split, out, fc);
    return cudaGetLastError();
}

cudaError_t launch_scene_ranges(const uint64_t* segs, uint32_t n, const BatchGeom& bg, const uint32_t* scene_ids,
                                uint32_t n_ids, uint32_t* ranges, cudaStream_t st) {
    if (n_ids == 0) return cudaSuccess;
    count_launches(1);
    k_scene_ranges<<<(2 * n_ids + 127) / 128, 128, 0, st>>>(segs, n, bg, scene_ids, n_ids, ranges);
    return cudaGetLastError();
}

cudaError_t launch_extract(const uint64_t* segs, const ExtractTarget* tg, uint32_t n_tg, uint64_t total,
                           const BatchGeom& bg, cudaStream_t st) {
    if (total == 0) return cudaSuccess;
    if (n_tg == 0 || n_tg > MAX_KEEP_SOURCES) return cudaErrorInvalidValue;
    count_launches(1);
    k_extract<<<(uint32_t)((total + 255) / 256), 256, 0, st>>>(segs, tg, n_tg, total, bg);
    return cudaGetLastError();
}

}  // namespace cgb
