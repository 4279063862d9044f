// Cover carries, per-tile work items and the tile painter.
//
// The reference paints each tile row sequentially (Painter::paint_tile_row,
// surpass/src/painter/mod.rs:495-596) and carries each layer's per-row cover
// from tile to tile through LayerWorkbench's queue
// (surpass/src/painter/layer_workbench.rs:134-198, 430-486).  Here the segments
// arrive sorted tile-major, by (tile row j, tile column i, order L), as the
// reference's sort key orders them, so every "tile-layer" group (TL) is
// contiguous.  The TLs' (j, L) run records, sorted by run, list each run's
// TLs left to right, and the carry into a TL is an exclusive prefix of its
// run's cover sums (8 x i8 lanes, wrapping).
//
// A layer L is painted in tile i of row j (is in the workbench's `ids`) iff
//   - L has segments in (j, i), or
//   - i is the first painted tile of the row and L has segments left of it
//     (the initial queue is pushed without an emptiness test,
//     painter/mod.rs:507-550, layer_workbench.rs:134-137), or
//   - the cumulative cover of L entering tile i is non-empty for L's fill rule
//     (the queue only keeps non-empty carries, layer_workbench.rs:194, 475).
// The exact cumulative cover equals the reference's queued cover up to
// multiples of 32 for EvenOdd (whose tests are mod 32) and exactly for NonZero,
// so every decision and coverage below is bit-identical.
//
// Work items are (tile, order) pairs, written along the sorted run records
// ((row, order, column) order) and sorted by tile with the (stable) radix
// sort, which leaves each tile's items in order.  The painter gives each tile one warp (2 pixels per lane), replicates
// tile_unchanged_pass and skip_fully_covered_layers (:200-222, :310-388),
// paints the surviving layers bottom-up in f32 with the reference's vector
// blend formulas, and writes RGBA8 with 128-bit stores.  Frames with gradient
// fills or clip layers use the FULL variant: per-pixel gradient colours
// (style.rs:96-174), skip_trivial_clips_pass (:224-308) as a lockstep warp
// pass, and the painter's clip mask (painter/mod.rs:260-317, 402-416).
#include "cgb_internal.cuh"

namespace cgb {

namespace {

constexpr int HEAD_THREADS = 256;
constexpr int HEAD_ITEMS = 8;
constexpr int HEAD_WARPS = HEAD_THREADS / 32;
constexpr int TL_STAGE = 64;  // TLs per warp staged for the TL scan's writes

// The cover of one segment as a packed 8 x i8 value (its row's lane).
__device__ __forceinline__ uint64_t seg_cover(uint32_t low) {
    return (uint64_t)(uint8_t)(int8_t)low_cover(low) << (8 * low_tile_y(low));
}

// TL heads and their cover sums in one pass over the sorted segments.
//
// Each thread owns HEAD_ITEMS consecutive segments; a segment starts a TL when
// its key (bits 22..63) differs from its predecessor's.  A TL's cover sum is
// the lane-wise sum of its segments' covers; the part of it that lies beyond
// the owning thread is R(t + 1), where R(t) = pre(t) + (t has a head ? 0 :
// R(t + 1)) and pre(t) is the sum of thread t's segments before its first
// head.  R is a reverse segmented scan: within a warp by shuffles, across
// warps in shared memory, and across blocks through each block's R(0)
// (blk_cover, written by the counting pass) and whether the block holds a head.
//
// mode 0: per block, the TL count, blk_cover and blk_head.
// mode 1: per TL g, its first segment, key, cover sum and run record
// (tl_rec[g] = (row, order) run << idx_bits | g, sorted afterwards).
template <int MODE>
__global__ void __launch_bounds__(HEAD_THREADS, 5) k_tl_scan(const uint64_t* __restrict__ segs, uint32_t n,
                                                          uint32_t* __restrict__ block_counts,
                                                          const uint32_t* __restrict__ block_off, CarryBuffers cb) {
    constexpr int mode = MODE;
    n = fc_count(cb.fc, FC_SEGS, n, false);
    // (graph frames launch blocks for the capacity: those past the count
    // hold no segments and are not walked)
    const uint32_t nb = min(gridDim.x, (uint32_t)((n + HEAD_THREADS * HEAD_ITEMS - 1) / (HEAD_THREADS * HEAD_ITEMS)));
    // mode 1: the next block's cover sum and head flag, loaded first so that
    // their latency passes while the segments load
    uint64_t next_cover = 0;
    uint32_t next_head = 1;
    if (mode == 1 && threadIdx.x == 0 && blockIdx.x + 1 < nb) {
        next_cover = cb.blk_cover[blockIdx.x + 1];
        next_head = cb.blk_head[blockIdx.x + 1];
    }
    const uint64_t s0 = ((uint64_t)blockIdx.x * HEAD_THREADS + threadIdx.x) * HEAD_ITEMS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t key[HEAD_ITEMS];
    uint32_t low[HEAD_ITEMS];
    uint32_t flags = 0, cnt = 0;
    uint64_t prev = ~0ull;
    if (s0 < n && s0 > 0) prev = segs[s0 - 1] >> 22;
    // the thread's segments as 16-byte pairs (s0 is a multiple of HEAD_ITEMS)
    uint64_t sv[HEAD_ITEMS];
    if (s0 + HEAD_ITEMS <= n) {
        const ulonglong2* p2 = reinterpret_cast<const ulonglong2*>(segs + s0);
#pragma unroll
        for (int k = 0; k < HEAD_ITEMS / 2; k++) {
            const ulonglong2 v = p2[k];
            sv[2 * k] = v.x;
            sv[2 * k + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < HEAD_ITEMS; k++) sv[k] = s0 + k < n ? segs[s0 + k] : 0ull;
    }
#pragma unroll
    for (int k = 0; k < HEAD_ITEMS; k++) {
        const uint64_t s = s0 + k;
        key[k] = ~0ull;
        low[k] = 0;
        if (s < n) {
            const uint64_t v = sv[k];
            key[k] = v >> 22;
            low[k] = (uint32_t)v;
            if (key[k] != prev) {
                flags |= 1u << k;
                cnt++;
            }
            prev = key[k];
        }
    }
    // TL counts: inclusive scan within the warp
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += a;
    }
    // mode 1: the warp's TLs are consecutive from its first: staged in shared
    // memory and written by the warp together after the scans (a thread's own
    // TLs are few and sparse across the lanes); a warp with more TLs than the
    // stage writes them directly once its offset is known.
    __shared__ uint32_t st_start[HEAD_WARPS][TL_STAGE];
    __shared__ uint64_t st_key[HEAD_WARPS][TL_STAGE], st_cover[HEAD_WARPS][TL_STAGE];
    const uint32_t wn = __shfl_sync(0xffffffffu, inc, 31);  // the warp's TL count
    const bool staged = mode == 1 && wn <= (uint32_t)TL_STAGE;
    // pre(t): covers before the thread's first head (all of them without
    // one); staged: acc = covers since its last head, whose cover is closed
    // once the following covers are known
    uint64_t pre = 0, acc = 0;
    uint32_t last = 0;  // staged: the stage index of the thread's last TL
    if (staged) {
        uint32_t i = inc - cnt;
        bool open = false;
#pragma unroll
        for (int k = 0; k < HEAD_ITEMS; k++) {
            if (flags & (1u << k)) {
                if (open) st_cover[warp][i++] = acc;
                else pre = acc;
                open = true;
                acc = 0;
                st_start[warp][i] = (uint32_t)(s0 + k);
                st_key[warp][i] = key[k];
            }
            if (s0 + k < n) acc = cover_add(acc, seg_cover(low[k]));
        }
        if (!open) pre = acc;
        last = i;
    } else {
#pragma unroll
        for (int k = 0; k < HEAD_ITEMS; k++)
            if ((flags & ((2u << k) - 1)) == 0) pre = cover_add(pre, seg_cover(low[k]));
    }

    // reverse segmented scan of (pre, has head) within the warp
    uint64_t r = pre;
    bool stop = flags != 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t nr = __shfl_down_sync(0xffffffffu, r, o);
        const bool ns = __shfl_down_sync(0xffffffffu, stop ? 1 : 0, o) != 0;
        if (!stop && lane + o < 32) {
            r = cover_add(r, nr);
            stop = ns;
        }
    }
    __shared__ uint64_t w_r[HEAD_WARPS], w_carry[HEAD_WARPS];
    __shared__ uint32_t w_stop[HEAD_WARPS], w_sums[HEAD_WARPS];
    __shared__ uint64_t s_next;  // R of the first thread of the next block
    if (lane == 0) {
        w_r[warp] = r;
        w_stop[warp] = stop ? 1u : 0u;
    }
    if (lane == 31) w_sums[warp] = inc;
    if (mode == 1 && threadIdx.x == 0) {
        // the covers of the following blocks up to the first with a head
        uint64_t x = next_cover;
        if (!next_head)
            for (uint32_t b = blockIdx.x + 2; b < nb; b++) {
                x = cover_add(x, cb.blk_cover[b]);
                if (cb.blk_head[b]) break;
            }
        s_next = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // carry into each warp from the warps after it (and the next block)
        uint64_t c = mode == 1 ? s_next : 0;
        for (int w = HEAD_WARPS - 1; w >= 0; w--) {
            w_carry[w] = c;
            c = w_stop[w] ? w_r[w] : cover_add(w_r[w], c);
        }
        uint32_t run = 0;
        for (int w = 0; w < HEAD_WARPS; w++) {
            const uint32_t v = w_sums[w];
            w_sums[w] = run;
            run += v;
        }
        if (mode == 0) {
            block_counts[blockIdx.x] = run;
            cb.blk_cover[blockIdx.x] = c;  // R(0) up to the block end
            cb.blk_head[blockIdx.x] = run != 0 ? 1u : 0u;
        }
    }
    __syncthreads();
    if (mode == 0) return;
    const uint64_t R = stop ? r : cover_add(r, w_carry[warp]);
    const uint64_t r_next_lane = __shfl_down_sync(0xffffffffu, R, 1);
    const uint64_t cont = lane == 31 ? w_carry[warp] : r_next_lane;  // R(t + 1)
    const uint32_t cap = cb.fc ? cb.tl_cap : 0xFFFFFFFFu;
    const uint32_t o0 = block_off[blockIdx.x] + w_sums[warp];
    if (!staged) {
        // the thread's TLs from o0 + its first, written directly
        uint32_t i = inc - cnt;
        bool open = false;
#pragma unroll
        for (int k = 0; k < HEAD_ITEMS; k++) {
            if (flags & (1u << k)) {
                if (open) {
                    if (o0 + i < cap) cb.tl_cover[o0 + i] = acc;
                    i++;
                }
                open = true;
                acc = 0;
                if (o0 + i < cap) {
                    const uint32_t o = o0 + i;
                    cb.tl_start[o] = (uint32_t)(s0 + k);
                    cb.tl_key[o] = key[k];
                    cb.tl_rec[o] = (key_run(key[k], cb.order_bits, cb.col_bits) << cb.idx_bits) | o;
                }
            }
            if (s0 + k < n) acc = cover_add(acc, seg_cover(low[k]));
        }
        if (flags && o0 + i < cap) cb.tl_cover[o0 + i] = cover_add(acc, cont);
        return;
    }
    if (flags) st_cover[warp][last] = cover_add(acc, cont);
    __syncwarp();
    for (uint32_t t = lane; t < wn; t += 32) {
        const uint32_t o = o0 + t;
        if (o >= cap) break;
        const uint64_t k = st_key[warp][t];
        cb.tl_start[o] = st_start[warp][t];
        cb.tl_key[o] = k;
        cb.tl_rec[o] = (key_run(k, cb.order_bits, cb.col_bits) << cb.idx_bits) | o;
        cb.tl_cover[o] = st_cover[warp][t];
    }
}

// Work-item payload bits above the TL index: the item holds only a cover carry;
// its layer is full in the tile; and it is also an opaque Solid Over layer.
constexpr uint32_t ITEM_OWN = 0u;
constexpr uint32_t ITEM_OPAQUE = 1u;
constexpr uint32_t ITEM_FULL = 2u;
constexpr uint32_t ITEM_CARRY = 4u;
constexpr int ITEM_FLAG_BITS = 3;

// The work items of TL g: its own (tile, order) pair, when its tile is
// painted, and cover-carry-only items for the tiles [ta, tb) of its row, up
// to the next TL of its (row, order) run.
struct TlItems {
    uint64_t row_tile;  // global index of the first tile of the TL's row
    int32_t own;        // tile column of the own item, or -1
    int32_t ta, tb;     // the carry-only items' tile columns (none if ta >= tb)
    uint32_t flags;     // the carry-only items' flags
    uint32_t L;
    uint32_t g;         // the TL (its index in segment order)
    __device__ __forceinline__ uint32_t count() const {
        return (own >= 0 ? 1u : 0u) + (tb > ta ? (uint32_t)(tb - ta) : 0u);
    }
};

// The work items of TL g, of key `key` and leaving cover `carry_out`;
// next_col: the column of the next TL of its run, or -1 at the run's end.
__device__ __forceinline__ TlItems tl_items_of(uint32_t g, uint64_t key, uint64_t carry_out, int32_t next_col,
                                               const BatchGeom& bg) {
    TlItems r{0, -1, 0, 0, 0, 0, 0};
    r.g = g;
    const int32_t i = (int32_t)key_col1(key, bg.order_bits, bg.col_bits) - 1;
    const uint32_t L = key_order(key, bg.order_bits);
    const uint32_t grow = key_row(key, bg.order_bits, bg.col_bits);
    // fields out of range only come from a sort that gave up (its error
    // flag is reported after the frame): no items rather than a stray access
    if (grow >= bg.total_rows) return r;
    // (one scene: no row-to-scene lookup on the way to the scene's fields)
    const SceneDesc& S = bg.scenes[bg.n_scenes == 1 ? 0u : bg.row_scene[grow]];
    const uint32_t j = grow - S.row_base;
    if (j < S.crop_v0 || j >= S.crop_v1 || L >= S.n_orders) return r;
    r.L = L;
    r.row_tile = (uint64_t)S.tile_base + (uint64_t)j * S.row_len;
    int32_t next = next_col >= 0 ? next_col : (int32_t)S.row_len;
    const int32_t h0 = (int32_t)S.crop_h0, h1 = (int32_t)S.crop_h1;
    if (next > h1) next = h1;
    if (i >= h0 && i < h1) r.own = i;  // a layer with segments is never "full" (layer_workbench.rs:164-175)
    if (next <= i + 1) return r;
    const PaintProps pp = S.props[L];
    const bool nonempty = !cover_is_empty(carry_out, pp.fill_rule);
    // payload of a cover-carry-only item: its layer_is_full and the opaque
    // Solid Over test of skip_fully_covered_layers (:335-356)
    const bool full = cover_is_full(carry_out, pp.fill_rule);
    r.flags = ITEM_CARRY | (full ? ITEM_FULL : 0u) | (full && (pp.flags & PROPS_OPAQUE_OVER) ? ITEM_OPAQUE : 0u);
    if (i < h0) {
        // the first painted tile of the row holds every layer with segments
        // to its left, empty or not
        if (next <= h0) return r;
        r.ta = h0;
        r.tb = nonempty ? next : h0 + 1;
        return r;
    }
    if (nonempty) {
        r.ta = i + 1;
        r.tb = next;
    }
    return r;
}

// The work items of the TL at position s of the sorted run records.
__device__ __forceinline__ TlItems tl_items(uint32_t s, uint32_t G, const CarryBuffers& cb, const BatchGeom& bg) {
    const int ib = cb.idx_bits;
    // every load issued before any is used (the next record's key whether or
    // not it continues the run)
    const bool has_next = s + 1 < G;
    const uint64_t rec = cb.tl_rec[s];
    const uint64_t rec1 = has_next ? cb.tl_rec[s + 1] : 0;
    const uint64_t key1 = has_next ? cb.tl_skey[s + 1] : 0;
    const uint64_t key = cb.tl_skey[s], sout = cb.tl_sout[s];
    const uint32_t g = (uint32_t)(rec & ((1ull << ib) - 1));
    if (g >= G) return TlItems{0, -1, 0, 0, 0, 0, 0};
    int32_t next_col = -1;
    if (has_next && (rec1 >> ib) == (rec >> ib)) next_col = (int32_t)key_col1(key1, bg.order_bits, bg.col_bits) - 1;
    return tl_items_of(g, key, sout, next_col, bg);
}

// Exclusive prefix of the cover sums along each (j, L) run, taken in the
// sorted run records (runs are a layer's tile groups in one tile row, left
// to right): one thread per record, a segmented scan across the warp, and
// for a run that began before the warp, the sum of its earlier records,
// taken 32 at a time by the warp.  Each TL's entering cover goes to the
// TL's own index, where the painter reads it; the key and the leaving cover
// go to the record's position (tl_skey, tl_sout), where the item expansion
// reads them in sequence, and each record's count of work items (TlItems)
// goes to item_count.  Thread 0 also closes the TL segment ranges:
// tl_start[G] = P.
__global__ void __launch_bounds__(256) k_tl_carry(uint32_t G, uint32_t P, CarryBuffers cb, BatchGeom bg) {
    const uint32_t Gcap = G;
    G = fc_count(cb.fc, FC_TLS, G, blockIdx.x == 0 && threadIdx.x == 0);
    P = fc_count(cb.fc, FC_SEGS, P, false);
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    if (s == 0) cb.tl_start[G] = P;
    // graph frames: the item counts past the device count stay zero for the scan over the capacity
    if (s >= G && s < Gcap) cb.item_count[s] = 0;
    const uint32_t s0 = s - lane;  // the warp's first record
    if (s0 >= G) return;           // (whole warps only: the shuffles below take every lane)
    const int ib = cb.idx_bits;
    const uint64_t mask = (1ull << ib) - 1;
    const bool valid = s < G;
    uint64_t run = ~0ull, cov = 0, key = ~0ull;  // no row: no items (g beyond G only after a failed sort)
    uint32_t g = 0xFFFFFFFFu;
    if (valid) {
        const uint64_t r = cb.tl_rec[s];
        run = r >> ib;
        g = (uint32_t)(r & mask);
        if (g < G) {
            key = cb.tl_key[g];
            cov = cb.tl_cover[g];
        }
    }
    uint64_t prev_run = __shfl_up_sync(0xffffffffu, run, 1);
    if (lane == 0) prev_run = s > 0 ? (cb.tl_rec[s - 1] >> ib) : ~run;
    const bool head = run != prev_run;
    // segmented inclusive scan of the covers (restart at each head)
    uint64_t incl = cov;
    bool f = head;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t tv = __shfl_up_sync(0xffffffffu, incl, o);
        const bool tf = __shfl_up_sync(0xffffffffu, f ? 1 : 0, o) != 0;
        if (lane >= o) {
            if (!f) incl = cover_add(tv, incl);
            f = f || tf;
        }
    }
    // the run open at the warp's start: its records before the warp
    uint64_t pre = 0;
    const uint64_t run0 = __shfl_sync(0xffffffffu, run, 0);
    if (!__shfl_sync(0xffffffffu, head ? 1 : 0, 0)) {
        int64_t h0 = (int64_t)s0 - 1;
        while (true) {
            const int64_t h = h0 - lane;
            bool in = false;
            uint64_t c = 0;
            if (h >= 0) {
                const uint64_t r = cb.tl_rec[h];
                in = (r >> ib) == run0;
                const uint64_t hg = r & mask;
                if (in && hg < G) c = cb.tl_cover[hg];
            }
            const uint32_t m = __ballot_sync(0xffffffffu, in);
            const int n_in = m == 0xffffffffu ? 32 : __ffs(~m) - 1;  // the run's records are lanes [0, n_in)
            if (lane >= n_in) c = 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c = cover_add(c, __shfl_xor_sync(0xffffffffu, c, o));
            pre = cover_add(pre, c);
            if (n_in < 32) break;
            h0 -= 32;
        }
    }
    const uint64_t incl_prev = __shfl_up_sync(0xffffffffu, incl, 1);
    uint64_t carry = (head || lane == 0) ? 0 : incl_prev;
    if (!f && !head) carry = cover_add(carry, pre);  // still in the warp's open run
    // the run's next TL: the next lane's, or (last lane) loaded
    const uint64_t next_run = __shfl_down_sync(0xffffffffu, run, 1);
    uint64_t next_key = __shfl_down_sync(0xffffffffu, key, 1);
    bool more = lane < 31 ? next_run == run : false;
    if (lane == 31 && valid && s + 1 < G) {
        const uint64_t r = cb.tl_rec[s + 1];
        const uint64_t ng = r & mask;
        more = (r >> ib) == run && ng < G;
        if (more) next_key = cb.tl_key[ng];
    }
    if (!valid) return;
    const uint64_t out = cover_add(carry, cov);
    if (g < G) cb.tl_carry[g] = carry;
    cb.tl_skey[s] = key;
    cb.tl_sout[s] = out;
    uint32_t items = 0;
    if (g < G) {
        const int32_t next_col = more ? (int32_t)key_col1(next_key, bg.order_bits, bg.col_bits) - 1 : -1;
        items = tl_items_of(g, key, out, next_col, bg).count();
    }
    cb.item_count[s] = items;
}

// Item = tile | order | flags | TL index, high to low; the tile field is the
// sort key.  The items of a tile are written in ascending order (they are
// written along the sorted run records: by row, then order), so a stable
// sort on the tile alone leaves each tile's items in paint order.  Each
// block expands the items of 256 run records together: thread t writes
// items t, t + 256, ... of the block's range.
constexpr int IW_THREADS = 256;
constexpr int IW_PER = 8;                      // items built per thread and chunk
constexpr int IW_CHUNK = IW_THREADS * IW_PER;  // items per chunk

__global__ void __launch_bounds__(IW_THREADS) k_items_write(uint32_t G, CarryBuffers cb, BatchGeom bg, int idx_bits) {
    __shared__ uint32_t s_off[IW_THREADS + 1];  // item offsets of the block's TLs, from its first item
    __shared__ uint64_t s_row[IW_THREADS];
    __shared__ int32_t s_own[IW_THREADS], s_ta[IW_THREADS];
    __shared__ uint32_t s_lf[IW_THREADS];  // order << 3 | carry-only flags
    __shared__ uint32_t s_g[IW_THREADS];   // the TL
    G = fc_count(cb.fc, FC_TLS, G, false);
    const uint32_t g0 = blockIdx.x * IW_THREADS, g = g0 + threadIdx.x;
    if (g0 >= G) return;  // graph frames: blocks past the TL count
    const uint32_t icap = cb.fc ? cb.items_cap : 0xFFFFFFFFu;
    const uint32_t nt = min(G - g0, (uint32_t)IW_THREADS);
    const uint32_t base = cb.item_off[g0];
    if (g < G) {
        const TlItems r = tl_items(g, G, cb, bg);
        s_off[threadIdx.x] = cb.item_off[g] - base;
        s_row[threadIdx.x] = r.row_tile;
        s_own[threadIdx.x] = r.own;
        s_ta[threadIdx.x] = r.ta;
        s_lf[threadIdx.x] = (r.L << ITEM_FLAG_BITS) | r.flags;
        s_g[threadIdx.x] = r.g;
    }
    if (threadIdx.x == 0) s_off[nt] = cb.item_off[g0 + nt] - base;
    __syncthreads();
    const uint32_t total = s_off[nt];
    const int ob = cb.order_bits;
    // Chunks of IW_CHUNK items: each thread builds IW_PER consecutive items
    // (one search for the TL of the first, then a walk), into shared memory;
    // the block then writes the chunk out together.
    __shared__ uint64_t s_items[IW_CHUNK];
    for (uint32_t c0 = 0; c0 < total; c0 += IW_CHUNK) {
        const uint32_t cn = min((uint32_t)IW_CHUNK, total - c0);
        const uint32_t i0 = threadIdx.x * IW_PER;
        if (i0 < cn) {
            uint32_t idx = c0 + i0;
            // the TL q with s_off[q] <= idx < s_off[q + 1] (the last one with s_off[q] <= idx)
            uint32_t lo = 0, hi = nt;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_off[mid] <= idx) lo = mid;
                else hi = mid;
            }
            const uint32_t iend = min(i0 + (uint32_t)IW_PER, cn);
            for (uint32_t i = i0; i < iend; i++, idx++) {
                while (s_off[lo + 1] <= idx) lo++;  // (past TLs without items too)
                const uint32_t k = idx - s_off[lo];
                const int32_t own = s_own[lo];
                const uint32_t lf = s_lf[lo];
                int32_t col;
                uint32_t fl;
                if (own >= 0 && k == 0) {
                    col = own;
                    fl = ITEM_OWN;
                } else {
                    col = s_ta[lo] + (int32_t)(k - (own >= 0 ? 1u : 0u));
                    fl = lf & 7u;
                }
                const uint64_t tile = s_row[lo] + (uint64_t)col;
                const uint64_t key = (((tile << ob) | (lf >> ITEM_FLAG_BITS)) << ITEM_FLAG_BITS) | fl;
                s_items[i] = (key << idx_bits) | s_g[lo];
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < cn; i += IW_THREADS)
            if (base + c0 + i < icap) cb.items[base + c0 + i] = s_items[i];
        __syncthreads();
    }
}

// tile_start from the items sorted by tile: each thread takes TR_ITEMS
// consecutive items (two 16-byte loads) and writes the start of every tile
// from the one before its first item's up to each item's tile.
constexpr int TR_ITEMS = 4;
__global__ void k_tile_ranges(const uint64_t* __restrict__ items, uint32_t W, uint32_t n_tiles, int tile_shift,
                              uint32_t* __restrict__ tile_start, FrameCounts* fc) {
    W = fc_count(fc, FC_ITEMS, W, blockIdx.x == 0 && threadIdx.x == 0);
    const uint64_t k0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * TR_ITEMS;
    if (k0 > W) return;
    uint64_t v[TR_ITEMS];
    if (k0 + TR_ITEMS <= W) {
        const ulonglong2* p2 = reinterpret_cast<const ulonglong2*>(items + k0);
        const ulonglong2 a = p2[0], b = p2[1];
        v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
    } else {
#pragma unroll
        for (int j = 0; j < TR_ITEMS; j++) v[j] = k0 + j < W ? items[k0 + j] : 0;
    }
    int64_t prev = k0 > 0 ? (int64_t)min(items[k0 - 1] >> tile_shift, (uint64_t)n_tiles) : -1;
#pragma unroll
    for (int j = 0; j < TR_ITEMS; j++) {
        const uint64_t k = k0 + j;
        if (k > W) break;
        const int64_t cur = k < W ? (int64_t)min(v[j] >> tile_shift, (uint64_t)n_tiles) : (int64_t)n_tiles;
        for (int64_t t = prev + 1; t <= cur; t++) tile_start[t] = (uint32_t)k;
        prev = cur;
    }
}

// ---------------------------------------------------------------------------
// painter numerics (surpass/src/painter/mod.rs:53-123, style.rs:206-418)
// ---------------------------------------------------------------------------

// from_area (painter/mod.rs:53-71)
__device__ __forceinline__ float from_area(int32_t area, uint32_t fill_rule) {
    if (fill_rule == CGB_FILL_NONZERO) return fminf(fabsf((float)area * (1.0f / 256.0f)), 1.0f);
    float capped = (float)(area & 255) * (1.0f / 256.0f);
    return ((area >> 8) & 1) == 0 ? capped : 1.0f - capped;
}

// Packed pixel pairs.  Each lane holds two pixels of a tile row, so every
// per-pixel operation of the blend is issued as one f32x2 instruction; each
// element is rounded exactly as the scalar f32 operation (.rn, no flush).
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b is a + (-b) in IEEE arithmetic: the negation is exact
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 sel2(bool a, bool b, float2 x, float2 y) {
    return make_float2(a ? x.x : y.x, b ? x.y : y.y);
}

// SoftLight's per-channel constants of a source colour (style.rs:365-418):
// (s (1 - s), d - s) with d = ((16 s - 12) s + 4) s for s <= 1/4, else sqrt(s).
// They depend on the item alone, so the stage computes them once per item.
__device__ __forceinline__ void soft_light_consts(const float4& c, float4 (&k)[2]) {
    float sk[3], dk[3];
    const float sv[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float s = sv[q];
        const float dd = s <= 0.25f ? __fmaf_rn(__fmaf_rn(16.0f, s, -12.0f), s, 4.0f) * s : sqrtf(s);
        sk[q] = s * (1.0f - s);
        dk[q] = dd - s;
    }
    k[0] = make_float4(sk[0], sk[1], sk[2], dk[0]);
    k[1] = make_float4(dk[1], dk[2], 0.0f, 0.0f);
}

// blend_function! (style.rs:288-418) for a pixel pair
template <int MODE>
__device__ __forceinline__ float2 blend_vec2(float2 d, float s) {
    const float2 S = splat(s);
    if (MODE == CGB_BLEND_OVER) return S;
    if (MODE == CGB_BLEND_MULTIPLY) return mul2(d, S);
    if (MODE == CGB_BLEND_SCREEN) return add2(fma2(d, splat(-s), d), S);
    if (MODE == CGB_BLEND_OVERLAY) {
        if (s <= 0.5f) return mul2(mul2(d, S), splat(2.0f));
        return mul2(splat(2.0f), sub2(add2(S, d), fma2(S, d, splat(0.5f))));
    }
    if (MODE == CGB_BLEND_DARKEN) return make_float2(fminf(d.x, s), fminf(d.y, s));
    if (MODE == CGB_BLEND_LIGHTEN) return make_float2(fmaxf(d.x, s), fmaxf(d.y, s));
    if (MODE == CGB_BLEND_COLOR_DODGE) {
        if (s == 0.0f) return splat(0.0f);
        const float2 om = sub2(splat(1.0f), d);
        return make_float2(fminf(1.0f, s / om.x), fminf(1.0f, s / om.y));
    }
    if (MODE == CGB_BLEND_COLOR_BURN) {
        if (s == 1.0f) return splat(1.0f);
        const float t = 1.0f - s;
        return sub2(splat(1.0f), make_float2(fminf(1.0f, t / d.x), fminf(1.0f, t / d.y)));
    }
    if (MODE == CGB_BLEND_HARD_LIGHT) {
        const float2 lo = mul2(mul2(d, S), splat(2.0f));
        const float2 hi = mul2(splat(2.0f), sub2(add2(S, d), fma2(S, d, splat(0.5f))));
        return sel2(d.x <= 0.5f, d.y <= 0.5f, lo, hi);
    }
    if (MODE == CGB_BLEND_SOFT_LIGHT) {
        const float dd = s <= 0.25f ? __fmaf_rn(__fmaf_rn(16.0f, s, -12.0f), s, 4.0f) * s : sqrtf(s);
        const float2 k = fma2(splat(2.0f), d, splat(-1.0f));
        const float2 lo = fma2(splat(s * (1.0f - s)), k, S);
        const float2 hi = fma2(splat(dd - s), k, S);
        return sel2(d.x <= 0.5f, d.y <= 0.5f, lo, hi);
    }
    if (MODE == CGB_BLEND_DIFFERENCE) {
        const float2 t = sub2(d, S);
        return make_float2(fabsf(t.x), fabsf(t.y));
    }
    return add2(fma2(mul2(splat(-2.0f), d), S, d), S);  // EXCLUSION
}

// blend_function! (style.rs:288-418) for the three colour channels of a
// lane's pixel pair: the only part of blend_at that depends on the mode.  The
// switch holds just these few operations per mode, so that the painter's hot
// code stays small when a tile's layers use many modes.
template <int MODE>
__device__ __forceinline__ void blend_channels(const float2 (&C)[4], const float4& src, float2 (&B)[3]) {
    B[0] = blend_vec2<MODE>(C[0], src.x);
    B[1] = blend_vec2<MODE>(C[1], src.y);
    B[2] = blend_vec2<MODE>(C[2], src.z);
}

// SoftLight from the item's constants (soft_light_consts): the vector
// formula's operations on the pixel pair.
__device__ __forceinline__ void blend_soft_light(const float2 (&C)[4], const float4& src, const float4* hk,
                                                 float2 (&B)[3]) {
    const float4 k0 = hk[0], k1 = hk[1];
    const float sk[3] = {k0.x, k0.y, k0.z}, dk[3] = {k0.w, k1.x, k1.y}, sv[3] = {src.x, src.y, src.z};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float2 d = C[q];
        const float2 k = fma2(splat(2.0f), d, splat(-1.0f));
        const float2 lo = fma2(splat(sk[q]), k, splat(sv[q]));
        const float2 hi = fma2(splat(dk[q]), k, splat(sv[q]));
        B[q] = sel2(d.x <= 0.5f, d.y <= 0.5f, lo, hi);
    }
}

// hk: the item's SoftLight constants (read only for that mode).
__device__ __forceinline__ void blend_channels(uint32_t mode, const float2 (&C)[4], const float4& src,
                                               const float4* hk, float2 (&B)[3]) {
    switch (mode) {
        case CGB_BLEND_OVER: blend_channels<CGB_BLEND_OVER>(C, src, B); break;
        case CGB_BLEND_MULTIPLY: blend_channels<CGB_BLEND_MULTIPLY>(C, src, B); break;
        case CGB_BLEND_SCREEN: blend_channels<CGB_BLEND_SCREEN>(C, src, B); break;
        case CGB_BLEND_OVERLAY: blend_channels<CGB_BLEND_OVERLAY>(C, src, B); break;
        case CGB_BLEND_DARKEN: blend_channels<CGB_BLEND_DARKEN>(C, src, B); break;
        case CGB_BLEND_LIGHTEN: blend_channels<CGB_BLEND_LIGHTEN>(C, src, B); break;
        case CGB_BLEND_COLOR_DODGE: blend_channels<CGB_BLEND_COLOR_DODGE>(C, src, B); break;
        case CGB_BLEND_COLOR_BURN: blend_channels<CGB_BLEND_COLOR_BURN>(C, src, B); break;
        case CGB_BLEND_HARD_LIGHT: blend_channels<CGB_BLEND_HARD_LIGHT>(C, src, B); break;
        case CGB_BLEND_SOFT_LIGHT: blend_soft_light(C, src, hk, B); break;
        case CGB_BLEND_DIFFERENCE: blend_channels<CGB_BLEND_DIFFERENCE>(C, src, B); break;
        default: blend_channels<CGB_BLEND_EXCLUSION>(C, src, B); break;
    }
}

// blend_at for one lane's pixel pair of a tile row (painter/mod.rs:364-400).
// C[q] holds channel q of the two pixels; a pixel whose column is not blended
// keeps its color.  MASKED = false when both columns of every lane are
// blended (cover-carry-only items: every column has the same per-row coverage).
// al = src.w * coverage, the pixel pair's alpha; hk: the item's SoftLight constants.
template <bool MASKED>
__device__ __forceinline__ void blend_dispatch_al(uint32_t mode, float2 (&C)[4], const float4& src,
                                                  const float4* hk, float2 al, bool col0, bool col1) {
    float2 B[3];
    blend_channels(mode, C, src, hk, B);
    const float2 inv = sub2(splat(1.0f), al);
    const float2 n0 = fma2(C[0], inv, mul2(B[0], al));
    const float2 n1 = fma2(C[1], inv, mul2(B[1], al));
    const float2 n2 = fma2(C[2], inv, mul2(B[2], al));
    const float2 n3 = fma2(C[3], inv, al);
    if (MASKED) {
        C[0] = sel2(col0, col1, n0, C[0]);
        C[1] = sel2(col0, col1, n1, C[1]);
        C[2] = sel2(col0, col1, n2, C[2]);
        C[3] = sel2(col0, col1, n3, C[3]);
    } else {
        C[0] = n0;
        C[1] = n1;
        C[2] = n2;
        C[3] = n3;
    }
}

template <bool MASKED>
__device__ __forceinline__ void blend_dispatch(uint32_t mode, float2 (&C)[4], const float4& src, const float4* hk,
                                               float2 cov, bool col0, bool col1) {
    blend_dispatch_al<MASKED>(mode, C, src, hk, mul2(splat(src.w), cov), col0, col1);
}

// blend_function! (style.rs:288-418) for one pixel: blend_vec2's operations
// on one element.
template <int MODE>
__device__ __forceinline__ float blend_vec1(float d, float s) {
    if (MODE == CGB_BLEND_OVER) return s;
    if (MODE == CGB_BLEND_MULTIPLY) return d * s;
    if (MODE == CGB_BLEND_SCREEN) return __fmaf_rn(d, -s, d) + s;
    if (MODE == CGB_BLEND_OVERLAY) return s <= 0.5f ? (d * s) * 2.0f : 2.0f * ((s + d) - __fmaf_rn(s, d, 0.5f));
    if (MODE == CGB_BLEND_DARKEN) return fminf(d, s);
    if (MODE == CGB_BLEND_LIGHTEN) return fmaxf(d, s);
    if (MODE == CGB_BLEND_COLOR_DODGE) return s == 0.0f ? 0.0f : fminf(1.0f, s / (1.0f - d));
    if (MODE == CGB_BLEND_COLOR_BURN) return s == 1.0f ? 1.0f : 1.0f - fminf(1.0f, (1.0f - s) / d);
    if (MODE == CGB_BLEND_HARD_LIGHT) return d <= 0.5f ? (d * s) * 2.0f : 2.0f * ((s + d) - __fmaf_rn(s, d, 0.5f));
    if (MODE == CGB_BLEND_SOFT_LIGHT) {
        const float dd = s <= 0.25f ? __fmaf_rn(__fmaf_rn(16.0f, s, -12.0f), s, 4.0f) * s : sqrtf(s);
        const float k = __fmaf_rn(2.0f, d, -1.0f);
        return d <= 0.5f ? __fmaf_rn(s * (1.0f - s), k, s) : __fmaf_rn(dd - s, k, s);
    }
    if (MODE == CGB_BLEND_DIFFERENCE) return fabsf(d - s);
    return __fmaf_rn(-2.0f * d, s, d) + s;  // EXCLUSION
}

// Gradient::get_t + color_at (style.rs:96-174) for one pixel.  x is the
// column argument the painter passes (the pixel's column + 1, as
// paint_layer's loop does), y the tile's top row, k the row in the tile.
// Stop lanes are merged by OR-ing float bits, as the vector code does.
__device__ float4 gradient_color(const GradRec& g, const GradStop* __restrict__ stops, float x, float y,
                                             int k) {
    const float dx = g.end[0] - g.start[0];
    const float dy = g.end[1] - g.start[1];
    const float dot = dx * dx + dy * dy;
    const float dot_recip = 1.0f / dot;
    float t;
    if (g.type == CGB_GRADIENT_LINEAR) {
        const float tx = (x - g.start[0]) * dx * dot_recip;
        const float ty = y - g.start[1];
        t = __fmaf_rn(((float)k + ty) * dy, dot_recip, tx);
    } else {
        const float px = x - g.start[0];
        const float px2 = px * px;
        const float py = (float)k + (y - g.start[1]);
        t = sqrtf(__fmaf_rn(py, py, px2) * dot_recip);
    }
    uint32_t out[4] = {0u, 0u, 0u, 0u};
    const GradStop* st = stops + g.first;
    bool acc = t <= st[0].stop;
    if (acc)
        for (int c = 0; c < 4; c++) out[c] |= __float_as_uint(st[0].color[c]);
    float start_stop = 0.0f;
    float sc[4] = {st[0].color[0], st[0].color[1], st[0].color[2], st[0].color[3]};
    for (uint32_t si = 1; si < g.n_stops; si++) {
        const float end_stop = st[si].stop;
        const bool m = acc ^ (t < end_stop);
        if (m) {
            const float d = end_stop - start_stop;
            const float dr = 1.0f / d;
            const float lt = (t - start_stop) * dr;
            for (int c = 0; c < 4; c++)
                out[c] |= __float_as_uint(__fmaf_rn(lt, st[si].color[c], __fmaf_rn(-lt, sc[c], sc[c])));
        }
        acc = acc || m;
        start_stop = end_stop;
        for (int c = 0; c < 4; c++) sc[c] = st[si].color[c];
    }
    if (!acc)
        for (int c = 0; c < 4; c++) out[c] |= __float_as_uint(st[g.n_stops - 1].color[c]);
    return make_float4(__uint_as_float(out[0]), __uint_as_float(out[1]), __uint_as_float(out[2]),
                       __uint_as_float(out[3]));
}

// blend_function! for a per-pixel source: the three channels of both pixels.
template <int MODE>
__device__ __forceinline__ void blend_channels_src(const float2 (&C)[4], const float4 (&src)[2], float (&B)[2][3]) {
    B[0][0] = blend_vec1<MODE>(C[0].x, src[0].x);
    B[0][1] = blend_vec1<MODE>(C[1].x, src[0].y);
    B[0][2] = blend_vec1<MODE>(C[2].x, src[0].z);
    B[1][0] = blend_vec1<MODE>(C[0].y, src[1].x);
    B[1][1] = blend_vec1<MODE>(C[1].y, src[1].y);
    B[1][2] = blend_vec1<MODE>(C[2].y, src[1].z);
}

__device__ __forceinline__ void blend_channels_src(uint32_t mode, const float2 (&C)[4], const float4 (&src)[2],
                                                   float (&B)[2][3]) {
    switch (mode) {
        case CGB_BLEND_OVER: blend_channels_src<CGB_BLEND_OVER>(C, src, B); break;
        case CGB_BLEND_MULTIPLY: blend_channels_src<CGB_BLEND_MULTIPLY>(C, src, B); break;
        case CGB_BLEND_SCREEN: blend_channels_src<CGB_BLEND_SCREEN>(C, src, B); break;
        case CGB_BLEND_OVERLAY: blend_channels_src<CGB_BLEND_OVERLAY>(C, src, B); break;
        case CGB_BLEND_DARKEN: blend_channels_src<CGB_BLEND_DARKEN>(C, src, B); break;
        case CGB_BLEND_LIGHTEN: blend_channels_src<CGB_BLEND_LIGHTEN>(C, src, B); break;
        case CGB_BLEND_COLOR_DODGE: blend_channels_src<CGB_BLEND_COLOR_DODGE>(C, src, B); break;
        case CGB_BLEND_COLOR_BURN: blend_channels_src<CGB_BLEND_COLOR_BURN>(C, src, B); break;
        case CGB_BLEND_HARD_LIGHT: blend_channels_src<CGB_BLEND_HARD_LIGHT>(C, src, B); break;
        case CGB_BLEND_SOFT_LIGHT: blend_channels_src<CGB_BLEND_SOFT_LIGHT>(C, src, B); break;
        case CGB_BLEND_DIFFERENCE: blend_channels_src<CGB_BLEND_DIFFERENCE>(C, src, B); break;
        default: blend_channels_src<CGB_BLEND_EXCLUSION>(C, src, B); break;
    }
}

// blend_at with a per-pixel source (gradient fills) and, for clipped layers,
// the clip mask (alpha = fill alpha * coverage * mask, in that order).
__device__ void blend_dispatch_src(uint32_t mode, float2 (&C)[4], const float4 (&src)[2], float2 cov, bool col0,
                                   bool col1, bool clipped, float2 mask) {
    float B[2][3];
    blend_channels_src(mode, C, src, B);
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float cv = h ? cov.y : cov.x;
        const bool on = h ? col1 : col0;
        float c[4] = {h ? C[0].y : C[0].x, h ? C[1].y : C[1].x, h ? C[2].y : C[2].x, h ? C[3].y : C[3].x};
        float al = src[h].w * cv;
        if (clipped) al *= h ? mask.y : mask.x;
        const float inv = 1.0f - al;
        const float n0 = __fmaf_rn(c[0], inv, B[h][0] * al);
        const float n1 = __fmaf_rn(c[1], inv, B[h][1] * al);
        const float n2 = __fmaf_rn(c[2], inv, B[h][2] * al);
        const float n3 = __fmaf_rn(c[3], inv, al);
        if (on) {
            if (h) C[0].y = n0, C[1].y = n1, C[2].y = n2, C[3].y = n3;
            else C[0].x = n0, C[1].x = n1, C[2].x = n2, C[3].x = n3;
        }
    }
}

// BlendMode::blend_fn (style.rs:206-267)
__device__ float blend_fn(uint32_t mode, float dst, float src) {
    switch (mode) {
        case CGB_BLEND_OVER: return src;
        case CGB_BLEND_MULTIPLY: return dst * src;
        case CGB_BLEND_SCREEN: return dst + src - (dst * src);
        case CGB_BLEND_OVERLAY:
            return src <= 0.5f ? (2.0f * src) * dst : (2.0f * src - 1.0f) + dst - ((2.0f * src - 1.0f) * dst);
        case CGB_BLEND_DARKEN: return fminf(dst, src);
        case CGB_BLEND_LIGHTEN: return fmaxf(dst, src);
        case CGB_BLEND_COLOR_DODGE:
            if (src == 0.0f) return 0.0f;
            if (dst == 1.0f) return 1.0f;
            return fminf(1.0f, src / (1.0f - dst));
        case CGB_BLEND_COLOR_BURN:
            if (src == 1.0f) return 1.0f;
            if (dst == 0.0f) return 0.0f;
            return 1.0f - fminf(1.0f, (1.0f - src) / dst);
        case CGB_BLEND_HARD_LIGHT:
            return dst <= 0.5f ? (2.0f * dst) * src : (2.0f * dst - 1.0f) + src - ((2.0f * dst - 1.0f) * src);
        case CGB_BLEND_SOFT_LIGHT: {
            float d = src <= 0.25f ? ((16.0f * src - 12.0f) * src + 4.0f) * src : sqrtf(src);
            if (dst <= 0.5f) return src - (1.0f - 2.0f * dst) * src * (1.0f - src);
            return src + (2.0f * dst - 1.0f) * (d - src);
        }
        case CGB_BLEND_DIFFERENCE: return fabsf(dst - src);
        default: return dst + src - 2.0f * dst * src;
    }
}

// linear_to_srgb_approx[_simd] (painter/mod.rs:73-106)
__device__ __forceinline__ float linear_to_srgb(float l) {
    float s = sqrtf(l);
    float s3 = l * s;
    float n = __fmaf_rn(0.20101772f, s3, __fmaf_rn(-0.51280147f, l, __fmaf_rn(1.344401f, s, -0.030656587f)));
    return l <= 0.0031308f ? l * 12.92f : n;
}
__device__ __forceinline__ uint32_t round_u8(float v) { return f2u8(roundf(v)); }
__device__ __forceinline__ uint32_t to_byte(float n) { return f2u8(__fmaf_rn(n, 255.0f, 0.5f)); }

// compute_srgb for one pixel (painter/mod.rs:418-453)
__device__ __forceinline__ uint32_t pixel_bytes(float c0, float c1, float c2, float a) {
    uint32_t r = round_u8((linear_to_srgb(c0) * a) * 255.0f);
    uint32_t g = round_u8((linear_to_srgb(c1) * a) * 255.0f);
    uint32_t b = round_u8((linear_to_srgb(c2) * a) * 255.0f);
    uint32_t al = round_u8(__fmaf_rn(a, 255.0f, 0.5f));
    return r | (g << 8) | (b << 16) | (al << 24);
}

// to_bytes (painter/mod.rs:108-123)
__device__ __forceinline__ uint32_t solid_bytes(const float c[4]) {
    float ar = 1.0f / c[3];
    return to_byte(linear_to_srgb(c[0] * ar)) | (to_byte(linear_to_srgb(c[1] * ar)) << 8) |
           (to_byte(linear_to_srgb(c[2] * ar)) << 16) | (to_byte(c[3]) << 24);
}

__device__ __forceinline__ void item_decode(uint64_t item, int idx_bits, int order_bits, uint32_t& L,
                                            uint32_t& flags, uint32_t& g) {
    g = (uint32_t)(item & ((1ull << idx_bits) - 1));
    uint64_t k = item >> idx_bits;
    flags = (uint32_t)(k & 7u);
    L = (uint32_t)((k >> ITEM_FLAG_BITS) & ((1ull << order_bits) - 1));
}

struct PaintArgs {
    BatchGeom bg;
    const uint64_t* segs;
    const uint64_t* items;
    int idx_bits;
    int order_bits;
    uint32_t G;  // TL count (item TL indices are below it)
    uint8_t* item_state;  // per work item: ISTATE_* from the clip pass (scenes with clips)
    const uint32_t* tile_start;
    const uint32_t* tl_start;
    const uint64_t* tl_cover;
    const uint64_t* tl_carry;
    const FrameCounts* fc;  // graph frames: nothing is painted after an overflow
};

constexpr int SEGCAP = 256;     // staged segments per warp and chunk of 32 items
static_assert(SEGCAP == 8 * 32, "the staging owner map gives each lane 8 positions");

constexpr uint32_t META_CARRY_ONLY = 32u;  // the item only carries cover through the tile
constexpr uint32_t META_ACTIVE = 64u;      // carry-only: some tile row has non-zero coverage
constexpr uint32_t META_GRAD = 128u;       // a gradient fill (its GradRec index in color.x's bits)
constexpr uint32_t META_SKIP = 256u;       // masked out by the clip pass: not painted
constexpr uint32_t META_CLIP = 512u;       // a clip layer (the last layer it clips in color.x's bits)
constexpr uint32_t META_APPLY_CLIP = 1024u;  // a clipped Draw layer whose clip is not trivially full
// item_state bits written by the clip pass (skip_trivial_clips_pass)
constexpr uint8_t ISTATE_MASKED = 1;     // masked out
constexpr uint8_t ISTATE_SKIP_CLIP = 2;  // clipped, but its clip is full: drawn unclipped

// Per-warp staging of 32 work items.
struct WarpStage {
    float4 color[32];
    float4 rowcov[32][2];  // carry-only items: coverage (FULL) or alpha of each tile row
    float4 hoist[32][2];   // SoftLight items: soft_light_consts of the colour
    uint64_t carry[32];    // cover entering the tile (TL items)
    uint32_t meta[32];     // blend_mode | fill_rule << 4 | META_*
    uint32_t order[32];    // the item's layer order
    uint32_t sb[32];     // first segment (global index)
    uint32_t cnt[32];    // segments of the item
    uint32_t soff[32];   // staging offset of its segments
    uint32_t seg[SEGCAP];
    alignas(8) uint8_t owner[SEGCAP];  // item of each staged segment
    alignas(8) int32_t area[64];    // per-pixel area sums (y * 8 + x)
    int32_t cov[64];     // per-pixel cover sums, added to the columns right of x
};

// Loads items [c0, c0 + n) into the stage; all loads of the chunk are in flight together.
template <bool FULL>
__device__ __forceinline__ void stage_items(const PaintArgs& a, const SceneDesc& scene, WarpStage& S, uint32_t c0,
                                            uint32_t n, int lane, bool with_segments) {
    const PaintProps* __restrict__ props = scene.props;
    const uint32_t n_orders = scene.n_orders;
    uint32_t meta = 0, sb = 0, cnt = 0;
    uint64_t carry = 0;
    float4 col = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t L = 0, fl = 0, g = 0;
    if ((uint32_t)lane < n) item_decode(a.items[c0 + lane], a.idx_bits, a.order_bits, L, fl, g);
    if ((uint32_t)lane < n && L < n_orders && g < a.G) {  // out of range only after a failed sort
        const float4* pp = reinterpret_cast<const float4*>(props + L);
        const uint4 hdr = *reinterpret_cast<const uint4*>(pp);
        col = pp[1];
        carry = a.tl_carry[g];
        const uint32_t co = (fl & ITEM_CARRY) ? 1u : 0u;
        const uint32_t fr = hdr.x & 1u;
        meta = (hdr.y & 15u) | (fr << 4);
        if ((hdr.y & 15u) == CGB_BLEND_SOFT_LIGHT) soft_light_consts(col, S.hoist[lane]);
        if (FULL) {
            if (hdr.z & PROPS_CLIP) {
                // `layer + *layers as u16` (mold's u16 arithmetic; 17 bits in the widened format)
                meta |= META_CLIP;
                col.x = __uint_as_float((L + hdr.w) & (scene.wide ? 0x1FFFFu : 0xFFFFu));
            } else if (!(hdr.z & PROPS_SOLID)) {
                meta |= META_GRAD;
                col.x = __uint_as_float(hdr.w);
            }
            if (scene.features & FEAT_CLIPS) {
                const uint32_t st = a.item_state[c0 + lane];
                if (st & ISTATE_MASKED) meta |= META_SKIP;
                if ((hdr.z & PROPS_DRAW) && (hdr.z & PROPS_CLIPPED) && !(st & ISTATE_SKIP_CLIP)) meta |= META_APPLY_CLIP;
            }
        }
        if (co) {
            carry = cover_add(carry, a.tl_cover[g]);
            meta |= META_CARRY_ONLY;
            if (with_segments) {
                // every pixel of a tile row has the row's coverage; the
                // layer's columns are blended iff some row is covered
                // (the plain painter stores each row's alpha, fill alpha x
                // coverage, the first product of blend_at)
                float rc[8];
                bool any = false;
#pragma unroll
                for (int yy = 0; yy < 8; yy++) {
                    rc[yy] = from_area(PIXEL_WIDTH * cover_lane(carry, yy), fr);
                    any |= rc[yy] != 0.0f;
                    if (!FULL) rc[yy] = col.w * rc[yy];
                }
                S.rowcov[lane][0] = make_float4(rc[0], rc[1], rc[2], rc[3]);
                S.rowcov[lane][1] = make_float4(rc[4], rc[5], rc[6], rc[7]);
                if (any) meta |= META_ACTIVE;
            }
        } else if (with_segments) {
            sb = a.tl_start[g];
            cnt = a.tl_start[g + 1] - sb;
        }
    }
    // exclusive scan of the segment counts -> staging offsets
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    S.color[lane] = col;
    S.carry[lane] = carry;
    S.meta[lane] = meta;
    S.order[lane] = L;
    S.sb[lane] = sb;
    S.cnt[lane] = cnt;
    S.soff[lane] = inc - cnt;
    __syncwarp();
    if (!with_segments) return;
    const uint32_t staged = min(total, (uint32_t)SEGCAP);
    const uint32_t soff = inc - cnt;
    // Segments are sorted tile-major, so a tile's TLs, in order, are
    // consecutive TLs with consecutive segment ranges: the chunk's segments
    // are then one run from its first TL item's first segment.
    {
        const uint32_t with = __ballot_sync(0xffffffffu, cnt > 0);
        const uint32_t base = __shfl_sync(0xffffffffu, sb, with ? __ffs(with) - 1 : 0);
        if (__all_sync(0xffffffffu, cnt == 0 || sb == base + soff)) {
#pragma unroll
            for (int r = 0; r < SEGCAP / 32; r++) {
                const uint32_t pos = lane + 32 * r;
                if (pos < staged) S.seg[pos] = (uint32_t)a.segs[base + pos];
            }
            __syncwarp();
            return;
        }
    }
    // Otherwise staged segment s belongs to the last item q with soff[q] <= s
    // among the items with segments: mark each such item at its offset, take
    // a running maximum over the offsets, then copy 32 segments per round.
    *reinterpret_cast<uint2*>(&S.owner[8 * lane]) = make_uint2(0u, 0u);
    __syncwarp();
    if (cnt > 0 && soff < (uint32_t)SEGCAP) S.owner[soff] = (uint8_t)lane;
    __syncwarp();
    {
        uint2 w = *reinterpret_cast<const uint2*>(&S.owner[8 * lane]);
        uint32_t run = 0, b[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t v = ((k < 4 ? w.x : w.y) >> (8 * (k & 3))) & 0xFFu;
            run = max(run, v);
            b[k] = run;
        }
        uint32_t scan = run;  // inclusive max over lanes <= this one
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, scan, o);
            if (lane >= o) scan = max(scan, t);
        }
        uint32_t carry = __shfl_up_sync(0xffffffffu, scan, 1);
        if (lane == 0) carry = 0;
        uint32_t lo = 0, hi = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t v = max(carry, b[k]);
            if (k < 4) lo |= v << (8 * k);
            else hi |= v << (8 * (k - 4));
        }
        *reinterpret_cast<uint2*>(&S.owner[8 * lane]) = make_uint2(lo, hi);
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < SEGCAP / 32; r++) {
        const uint32_t pos = lane + 32 * r;
        const uint32_t q = pos < staged ? S.owner[pos] : 0u;
        const uint32_t qsb = __shfl_sync(0xffffffffu, sb, q);
        const uint32_t qoff = __shfl_sync(0xffffffffu, soff, q);
        if (pos < staged) S.seg[pos] = (uint32_t)a.segs[qsb + (pos - qoff)];
    }
    __syncwarp();
}

// PAINT_WARPS tiles per CTA; FULL: the frame holds gradient fills or clips
template <int PAINT_WARPS, bool FULL>
__global__ void __launch_bounds__(PAINT_WARPS * 32) k_paint(PaintArgs a) {
    __shared__ WarpStage stages[PAINT_WARPS];
    const int lane = threadIdx.x & 31;
    WarpStage& S = stages[threadIdx.x >> 5];
    const uint32_t t = blockIdx.x * PAINT_WARPS + (threadIdx.x >> 5);
    if (t >= a.bg.total_tiles) return;
    if (a.fc && a.fc->overflow) return;
    // the scene holding global tile t
    uint32_t lo = 0, hi = a.bg.n_scenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a.bg.scenes[mid].tile_base <= t) lo = mid;
        else hi = mid;
    }
    const SceneDesc& p = a.bg.scenes[lo];
    const uint32_t lt = t - p.tile_base;
    const uint32_t j = lt / p.row_len, i = lt % p.row_len;
    if (i < p.crop_h0 || i >= p.crop_h1 || j < p.crop_v0 || j >= p.crop_v1) return;
    const uint32_t b = a.tile_start[t], e = a.tile_start[t + 1];

    // tile_unchanged_pass (layer_workbench.rs:200-222)
    if (p.prev_layers) {
        const int32_t layers = (int32_t)((e - b) & 0xFFFF);
        const int32_t old = p.prev_layers[lt];
        __syncwarp();
        if (lane == 0) p.prev_layers[lt] = layers;
        if (old >= 0 && old == layers) {
            bool all = true;
            for (uint32_t k = b + lane; k < e; k += 32) {
                uint32_t L, fl, g;
                item_decode(a.items[k], a.idx_bits, a.order_bits, L, fl, g);
                all &= L < p.n_orders && p.unchanged[L] != 0;
            }
            if (__all_sync(0xffffffffu, all)) return;  // TileWriteOp::None
        }
    }

    // skip_trivial_clips_pass (layer_workbench.rs:224-308): a sequential pass
    // over the tile's layers in order, run by the whole warp in lockstep (each
    // lane holds one item of the chunk); lane 0 records each item's state.
    const bool clips = FULL && (p.features & FEAT_CLIPS);
    if (clips) {
        const uint32_t lmask = p.wide ? 0x1FFFFu : 0xFFFFu;
        bool has = false, c_full = false, c_used = false;
        uint32_t c_last = 0, c_idx = 0;
        for (uint32_t c0 = b; c0 < e; c0 += 32) {
            const uint32_t n = min(32u, e - c0);
            uint32_t L = 0, fl = 0, g = 0, pf = 0, aux = 0;
            if ((uint32_t)lane < n) {
                item_decode(a.items[c0 + lane], a.idx_bits, a.order_bits, L, fl, g);
                if (L < p.n_orders) {
                    pf = p.props[L].flags;
                    aux = p.props[L].aux;
                }
            }
            for (uint32_t q = 0; q < n; q++) {
                const uint32_t qL = __shfl_sync(0xffffffffu, L, q);
                const uint32_t qpf = __shfl_sync(0xffffffffu, pf, q);
                const uint32_t qfl = __shfl_sync(0xffffffffu, fl, q);
                const uint32_t qaux = __shfl_sync(0xffffffffu, aux, q);
                uint8_t st = 0;
                if (qpf & PROPS_CLIP) {
                    has = true;
                    c_full = (qfl & ITEM_FULL) != 0;  // layer_is_full: no segments, full carried cover
                    c_last = (qL + qaux) & lmask;
                    c_idx = c0 + q;
                    c_used = false;
                    if (c_full) st |= ISTATE_MASKED;
                }
                if ((qpf & PROPS_DRAW) && (qpf & PROPS_CLIPPED)) {
                    if (has && qL <= c_last) {
                        if (c_full) st |= ISTATE_SKIP_CLIP;
                        else c_used = true;
                    } else {
                        st |= ISTATE_MASKED;
                    }
                }
                if (lane == 0) a.item_state[c0 + q] = st;
                if (has && qL > c_last) {
                    has = false;
                    if (!c_used && lane == 0) a.item_state[c_idx] |= ISTATE_MASKED;
                }
            }
        }
        if (has && !c_used && lane == 0) a.item_state[c_idx] |= ISTATE_MASKED;
        __syncwarp();
    }

    // skip_fully_covered_layers (layer_workbench.rs:310-388), top-down over
    // the items' precomputed full / opaque bits.
    int64_t k_op = -1;
    int first = 0;  // 0 none, 1 opaque, 2 incomplete
    for (int64_t c0 = (int64_t)e - 1; c0 >= (int64_t)b; c0 -= 32) {
        const int64_t idx = c0 - lane;
        bool inc = false, op = false;
        if (idx >= (int64_t)b) {
            const uint32_t fl = (uint32_t)(a.items[idx] >> a.idx_bits) & 7u;
            inc = !(fl & ITEM_FULL);
            op = (fl & ITEM_OPAQUE) != 0;
            if (clips) {
                const uint32_t st = a.item_state[idx];
                uint32_t L, f2, g;
                item_decode(a.items[idx], a.idx_bits, a.order_bits, L, f2, g);
                const uint32_t pf = L < p.n_orders ? p.props[L].flags : 0u;
                const bool clipped = (pf & PROPS_DRAW) && (pf & PROPS_CLIPPED) && !(st & ISTATE_SKIP_CLIP);
                if (st & ISTATE_MASKED) {
                    inc = op = false;
                } else {
                    inc = inc || clipped;
                    op = op && !clipped;
                }
            }
        }
        const uint32_t bi = __ballot_sync(0xffffffffu, inc), bo = __ballot_sync(0xffffffffu, op);
        const uint32_t any = bi | bo;
        if (first == 0 && any) first = (bo & (any & (0u - any))) ? 1 : 2;  // lowest lane = topmost item
        if (bo) {
            k_op = c0 - (__ffs(bo) - 1);
            break;
        }
    }

    const uint32_t y = lane & 7, xg = lane >> 3;
    const uint32_t x0 = 2 * xg;
    uint32_t px0 = 0, px1 = 0;
    bool painted = true;
    // the gradient column argument of the lane's first pixel, less one, and the tile's top row
    const float gx0 = (float)(i * 8 + x0), gy0 = (float)(j * 8);
    if (FULL && first != 2) {
        // the fold takes (unmasked) Solid Draw layers only (skip_fully_covered_layers, :376-383)
        const uint32_t from0 = first == 1 ? (uint32_t)k_op + 1 : b;
        for (uint32_t c0 = from0; c0 < e && first != 2; c0 += 32) {
            bool ok = true;
            if (c0 + lane < e) {
                uint32_t L, fl, g;
                item_decode(a.items[c0 + lane], a.idx_bits, a.order_bits, L, fl, g);
                const bool masked = clips && (a.item_state[c0 + lane] & ISTATE_MASKED);
                ok = masked || (L < p.n_orders && (p.props[L].flags & PROPS_SOLID) && (p.props[L].flags & PROPS_DRAW));
            }
            if (!__all_sync(0xffffffffu, ok)) first = 2;
        }
    }
    if (first != 2) {
        // Solid: fold BlendMode::blend (scalar, style.rs:269-285) over the
        // full layers above the opaque one (or above the clear color).
        float dst[4];
        uint32_t from;
        if (first == 1) {
            uint32_t L, fl, g;
            item_decode(a.items[k_op], a.idx_bits, a.order_bits, L, fl, g);
            const float4 c = reinterpret_cast<const float4*>(p.props + min(L, p.n_orders - 1))[1];
            dst[0] = c.x, dst[1] = c.y, dst[2] = c.z, dst[3] = c.w;
            from = (uint32_t)k_op + 1;
        } else {
            for (int q = 0; q < 4; q++) dst[q] = p.clear[q];
            from = b;
        }
        for (uint32_t c0 = from; c0 < e; c0 += 32) {
            const uint32_t n = min(32u, e - c0);
            stage_items<FULL>(a, p, S, c0, n, lane, false);
            for (uint32_t q = 0; q < n; q++) {
                if (FULL && (S.meta[q] & META_SKIP)) continue;
                const float4 col = S.color[q];
                const uint32_t mode = S.meta[q] & 15u;
                const float al = col.w, inv = 1.0f - al;
                const float o0 = __fmaf_rn(dst[0], inv, blend_fn(mode, dst[0], col.x) * al);
                const float o1 = __fmaf_rn(dst[1], inv, blend_fn(mode, dst[1], col.y) * al);
                const float o2 = __fmaf_rn(dst[2], inv, blend_fn(mode, dst[2], col.z) * al);
                const float o3 = __fmaf_rn(dst[3], inv, al);
                dst[0] = o0, dst[1] = o1, dst[2] = o2, dst[3] = o3;
            }
            __syncwarp();
        }
        px0 = px1 = solid_bytes(dst);
        painted = false;
    }
    if (painted) {
        // ColorBuffer: paint the unculled layers bottom-up (drive_tile_painting, :449-481).
        float2 C[4];
#pragma unroll
        for (int q = 0; q < 4; q++) C[q] = splat(p.clear[q]);
        // Painter's clip state (painter/mod.rs:260-317): a mask per pixel and
        // the last layer it applies to
        bool has_clip = false;
        uint32_t clip_last = 0;
        float2 clip_mask = splat(0.0f);
        const uint32_t start = k_op >= 0 ? (uint32_t)k_op : b;
        S.area[lane] = 0;
        S.area[lane + 32] = 0;
        S.cov[lane] = 0;
        S.cov[lane + 32] = 0;
        for (uint32_t c0 = start; c0 < e; c0 += 32) {
            const uint32_t n = min(32u, e - c0);
            stage_items<FULL>(a, p, S, c0, n, lane, true);
            for (uint32_t q = 0; q < n; q++) {
                // every lane reads the same word; the warp reduction makes
                // that visible to the compiler (a uniform value), so the
                // item's branches need no convergence barriers
                const uint32_t meta = __reduce_or_sync(0xffffffffu, S.meta[q]);
                const uint32_t mode = meta & 15u, fr = (meta >> 4) & 1u;
                bool apply = false;
                if (clips) {
                    if (meta & META_SKIP) continue;  // masked: its cover is carried, nothing is painted
                    if (has_clip && clip_last < S.order[q]) has_clip = false;
                    apply = (meta & META_APPLY_CLIP) != 0;
                    if (apply && !has_clip) continue;  // a clipped layer with no clip in effect
                }
                float2 cov;
                bool col0, col1;
                if (meta & META_CARRY_ONLY) {
                    if (!FULL) {
                        if (!(meta & META_ACTIVE)) continue;
                        blend_dispatch_al<false>(mode, C, S.color[q], S.hoist[q],
                                                 splat(reinterpret_cast<const float*>(&S.rowcov[q][0])[y]), true,
                                                 true);
                        continue;
                    }
                    cov = splat(reinterpret_cast<const float*>(&S.rowcov[q][0])[y]);
                    if (clips && (meta & META_CLIP)) {
                        if (!has_clip) {
                            has_clip = true;
                            clip_last = __float_as_uint(S.color[q].x);
                        }
                        clip_mask = cov;
                        continue;
                    }
                    if (!(meta & META_ACTIVE)) continue;
                    if (FULL && ((meta & META_GRAD) || apply)) {
                        float4 src[2] = {S.color[q], S.color[q]};
                        if (meta & META_GRAD) {
                            const GradRec g = p.grads[__float_as_uint(S.color[q].x)];
                            src[0] = gradient_color(g, p.stops, gx0 + 1.0f, gy0, (int)y);
                            src[1] = gradient_color(g, p.stops, gx0 + 2.0f, gy0, (int)y);
                        }
                        blend_dispatch_src(mode, C, src, cov, true, true, apply, clip_mask);
                    } else {
                        blend_dispatch<false>(mode, C, S.color[q], S.hoist[q], cov, true, true);
                    }
                    continue;
                } else {
                    // acc_segment / acc_cover / compute_areas (painter/mod.rs:229-243, 347-362):
                    // per-cell sums in shared memory, then each lane reads
                    // (and clears) the cells of its two pixels
                    const int32_t cy = cover_lane(S.carry[q], y);
                    const uint32_t cnt = S.cnt[q], so = S.soff[q], sb = S.sb[q];
                    for (uint32_t s = lane; s < cnt; s += 32) {
                        const uint32_t low = so + s < SEGCAP ? S.seg[so + s] : (uint32_t)a.segs[sb + s];
                        const uint32_t cell = low_cell(low);
                        atomicAdd(&S.area[cell], low_area(low));
                        atomicAdd(&S.cov[cell], low_cover(low));
                    }
                    __syncwarp();
                    // the lane's two pixels are adjacent cells: one 64-bit access each
                    const uint32_t c0i = y * 8 + x0;
                    const int2 aa = *reinterpret_cast<const int2*>(&S.area[c0i]);
                    const int2 vv = *reinterpret_cast<const int2*>(&S.cov[c0i]);
                    *reinterpret_cast<int2*>(&S.area[c0i]) = make_int2(0, 0);
                    *reinterpret_cast<int2*>(&S.cov[c0i]) = make_int2(0, 0);
                    const int32_t a0 = aa.x, a1 = aa.y, v0 = vv.x, v1 = vv.y;
                    // covers of the columns left of x0: prefix over the lane's column pairs
                    int32_t pre = v0 + v1;
                    int32_t t = __shfl_up_sync(0xffffffffu, pre, 8);
                    if (xg >= 1) pre += t;
                    t = __shfl_up_sync(0xffffffffu, pre, 16);
                    if (xg >= 2) pre += t;
                    const int32_t cv = cy + pre - (v0 + v1);
                    const int32_t cv1 = cv + v0;
                    cov.x = from_area(PIXEL_WIDTH * (int32_t)(int8_t)cv + (int32_t)(int16_t)a0, fr);
                    cov.y = from_area(PIXEL_WIDTH * (int32_t)(int8_t)cv1 + (int32_t)(int16_t)a1, fr);
                    __syncwarp();
                    if (clips && (meta & META_CLIP)) {  // clip_at: every column, zero or not
                        if (!has_clip) {
                            has_clip = true;
                            clip_last = __float_as_uint(S.color[q].x);
                        }
                        clip_mask = cov;
                        continue;
                    }
                    // A column is blended when any of its 8 coverages is non-zero
                    // (painter/mod.rs:287-289).
                    const uint32_t b0 = __ballot_sync(0xffffffffu, cov.x != 0.0f);
                    const uint32_t b1 = __ballot_sync(0xffffffffu, cov.y != 0.0f);
                    if (!(b0 | b1)) continue;
                    col0 = ((b0 >> (8 * xg)) & 0xFFu) != 0;
                    col1 = ((b1 >> (8 * xg)) & 0xFFu) != 0;
                }
                if (FULL && ((meta & META_GRAD) || apply)) {
                    float4 src[2] = {S.color[q], S.color[q]};
                    if (meta & META_GRAD) {
                        const GradRec g = p.grads[__float_as_uint(S.color[q].x)];
                        src[0] = gradient_color(g, p.stops, gx0 + 1.0f, gy0, (int)y);
                        src[1] = gradient_color(g, p.stops, gx0 + 2.0f, gy0, (int)y);
                    }
                    blend_dispatch_src(mode, C, src, cov, col0, col1, apply, clip_mask);
                } else {
                    blend_dispatch<true>(mode, C, S.color[q], S.hoist[q], cov, col0, col1);
                }
            }
            __syncwarp();
        }
        px0 = pixel_bytes(C[0].x, C[1].x, C[2].x, C[3].x);
        px1 = pixel_bytes(C[0].y, C[1].y, C[2].y, C[3].y);
    }

    if (p.written && lane == 0) p.written[lt] = 1;
    // RGBA8 store: a full tile goes out as 16 x 16-byte half rows.
    const uint32_t gx = i * 8 + x0, gy = j * 8 + y;
    const bool full_tile = (i * 8 + 8 <= p.width) && (j * 8 + 8 <= p.height) && ((p.stride & 3) == 0) &&
                           ((((uintptr_t)p.out) & 15) == 0);
    if (full_tile) {
        const uint32_t q0 = __shfl_down_sync(0xffffffffu, px0, 8);
        const uint32_t q1 = __shfl_down_sync(0xffffffffu, px1, 8);
        if ((xg & 1) == 0) {
            uint4 v = make_uint4(px0, px1, q0, q1);
            *reinterpret_cast<uint4*>(p.out + ((size_t)gy * p.stride + gx) * 4) = v;
        }
    } else if (gy < p.height) {
        uint32_t* row = reinterpret_cast<uint32_t*>(p.out + (size_t)gy * p.stride * 4);
        if (gx < p.width) row[gx] = px0;
        if (gx + 1 < p.width) row[gx + 1] = px1;
    }
}

}  // namespace

cudaError_t launch_tl_scan(int mode, const uint64_t* segs, uint32_t n, uint32_t* block_counts,
                           const uint32_t* block_off, const CarryBuffers& cb, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    count_launches(1);
    if (mode == 0)
        k_tl_scan<0><<<tl_scan_grid(n), HEAD_THREADS, 0, st>>>(segs, n, block_counts, block_off, cb);
    else
        k_tl_scan<1><<<tl_scan_grid(n), HEAD_THREADS, 0, st>>>(segs, n, block_counts, block_off, cb);
    return cudaGetLastError();
}

uint32_t tl_scan_grid(uint32_t n) { return (n + HEAD_THREADS * HEAD_ITEMS - 1) / (HEAD_THREADS * HEAD_ITEMS); }

cudaError_t launch_tl_carry(uint32_t G, uint32_t P, const CarryBuffers& cb, const BatchGeom& bg, cudaStream_t st) {
    count_launches(1);
    k_tl_carry<<<std::max<uint32_t>(1, (G + 255) / 256), 256, 0, st>>>(G, P, cb, bg);
    return cudaGetLastError();
}

cudaError_t launch_items(uint32_t G, const BatchGeom& bg, const CarryBuffers& cb, int idx_bits, cudaStream_t st) {
    if (G == 0) return cudaSuccess;
    count_launches(1);
    k_items_write<<<(G + IW_THREADS - 1) / IW_THREADS, IW_THREADS, 0, st>>>(G, cb, bg, idx_bits);
    return cudaGetLastError();
}

cudaError_t launch_tile_ranges(const uint64_t* items, uint32_t W, uint32_t n_tiles, int tile_shift,
                               uint32_t* tile_start, cudaStream_t st, FrameCounts* fc) {
    count_launches(1);
    k_tile_ranges<<<(W + 1 + 256 * TR_ITEMS - 1) / (256 * TR_ITEMS), 256, 0, st>>>(items, W, n_tiles, tile_shift,
                                                                                   tile_start, fc);
    return cudaGetLastError();
}

cudaError_t launch_paint(const BatchGeom& bg, const uint64_t* segs, const uint64_t* items, int idx_bits, uint32_t G,
                         const uint32_t* tile_start, const CarryBuffers& cb, uint32_t warps, bool full,
                         uint8_t* item_state, cudaStream_t st) {
    if (bg.total_tiles == 0) return cudaSuccess;
    PaintArgs a{bg,         segs,       items,       idx_bits,    cb.order_bits, G,
                item_state, tile_start, cb.tl_start, cb.tl_cover, cb.tl_carry,   cb.fc};
    count_launches(1);
    const uint32_t T = bg.total_tiles;
    if (full) {
        switch (warps) {
            case 2: k_paint<2, true><<<(T + 1) / 2, 64, 0, st>>>(a); break;
            case 4: k_paint<4, true><<<(T + 3) / 4, 128, 0, st>>>(a); break;
            case 8: k_paint<8, true><<<(T + 7) / 8, 256, 0, st>>>(a); break;
            default: return cudaErrorInvalidValue;
        }
    } else {
        switch (warps) {
            case 2: k_paint<2, false><<<(T + 1) / 2, 64, 0, st>>>(a); break;
            case 4: k_paint<4, false><<<(T + 3) / 4, 128, 0, st>>>(a); break;
            case 8: k_paint<8, false><<<(T + 7) / 8, 256, 0, st>>>(a); break;
            default: return cudaErrorInvalidValue;
        }
    }
    return cudaGetLastError();
}

}  // namespace cgb
