// Device-wide scan and the onesweep LSD radix sort of 64-bit pixel-segment keys.
//
// Replaces Rasterizer::sort (surpass/src/rasterizer/mod.rs:287-290), a rayon
// par_sort_unstable_by_key over `segment >> 22`.  The GPU sort is an LSD radix
// sort over a caller-chosen bit range with one "onesweep" kernel per digit:
// each CTA ranks a tile of keys in shared memory (warp multi-split: match.any,
// or ten ballots for a pass whose digits are mostly distinct within a warp),
// publishes its digit counts, resolves its global digit offsets with a
// decoupled look-back over the preceding tiles, and scatters the tile through
// shared memory so that each digit run is written contiguously.  The sort is
// stable, so sorting bits [22, 64) keeps rasterizer order among equal keys.
//
// Every spin on a predecessor's status is bounded: past the limit the kernel
// sets the handle's error flag and stops waiting (the host reports
// CGB_ERR_DEVICE_TIMEOUT), so a failed GPU never hangs on it.
#include <algorithm>
#include <mutex>

#include "cgb_internal.cuh"

namespace cgb {

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Block-wide exclusive scan (blockDim.x a multiple of 32, <= 1024).  Every
// thread of the block must call it.
template <class T>
__device__ T block_exclusive_scan(T v, T* total) {
    __shared__ T warp_sums[32];
    __shared__ T s_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? warp_sums[lane] : T(0);
        T wi = warp_inclusive_scan(w);
        if (lane < nw) warp_sums[lane] = wi - w;
        if (lane == 31) s_total = wi;
    }
    __syncthreads();
    T res = warp_sums[warp] + inc - v;
    if (total) *total = s_total;
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in, uint32_t n,
                                                             uint64_t* __restrict__ sums) {
    uint64_t s = 0;
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        uint64_t i = base + (uint64_t)k * SCAN_THREADS + threadIdx.x;
        if (i < n) s += in[i];
    }
    __shared__ uint64_t red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint64_t v = threadIdx.x < (SCAN_THREADS >> 5) ? red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = v;
    }
}

// Exclusive scan of nb u64 block sums in place; sums[nb] = total; out_tail
// (and tail2, if given) = total (u32).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(uint64_t* sums, uint32_t nb, uint32_t* out_tail,
                                                           uint32_t* tail2) {
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
        uint32_t i = b0 + threadIdx.x;
        uint64_t v = i < nb ? sums[i] : 0;
        uint64_t tot;
        uint64_t ex = block_exclusive_scan<uint64_t>(v, &tot);
        uint64_t c = carry;
        if (i < nb) sums[i] = c + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        sums[nb] = carry;
        if (out_tail) *out_tail = (uint32_t)carry;
        if (tail2) *tail2 = (uint32_t)carry;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const uint32_t* __restrict__ in, uint32_t n,
                                                            const uint64_t* __restrict__ sums,
                                                            uint32_t* __restrict__ out) {
    // Blocked arrangement: thread t owns elements [t*ITEMS, (t+1)*ITEMS) of the tile.
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        uint64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    uint64_t ex = block_exclusive_scan<uint64_t>(s, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        uint64_t i = base + k;
        if (i < n) out[i] = (uint32_t)ex;
        ex += v[k];
    }
}

// ---------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------

constexpr int RADIX = 512;  // up to 9-bit digits
constexpr int MAX_PASSES = 12;  // 42 key bits in 4-bit digits, split in two groups
// 512 threads (one digit each) x 14 keys: 7,168-key tiles, 2 CTAs per SM at 64
// registers.  Measured against 8 keys at 3 CTAs per SM, 12 and 16 keys at 2,
// and 256-thread CTAs: this shape sorts fastest.
constexpr int SORT_THREADS = RADIX;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_ITEMS = 14;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;  // keys per CTA
constexpr int SORT_MIN_BLOCKS = 2;
static_assert(SORT_TILE < 65536, "per-warp digit offsets are 16-bit");
constexpr uint32_t ST_AGG = 1u << 30;
constexpr uint32_t ST_INC = 2u << 30;
constexpr uint32_t ST_VAL = (1u << 30) - 1;
constexpr uint32_t SPIN_LIMIT = 1u << 22;  // ~ a second with the back-off below
constexpr int LB_WINDOW = 4;      // look-back entries loaded per round
constexpr unsigned LB_SLEEP = 32;  // back-off (ns) after a round with no published entry

struct PassPlan {
    int n;
    int skip;  // the first `skip` passes may be skipped (SortBits::skip_flag)
    int shift[MAX_PASSES];
    int bits[MAX_PASSES];
};

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One pass over the keys that histograms every digit of every pass (passes
// unrolled as in k_gather_hist; NP = 0: any number).
template <int NP>
__global__ void __launch_bounds__(512) k_radix_hist(const uint64_t* __restrict__ keys, uint32_t n, PassPlan plan,
                                                    uint32_t* __restrict__ hist, FrameCounts* fc, int fc_which) {
    __shared__ uint32_t sh[MAX_PASSES][RADIX];
    const int np = NP > 0 ? NP : plan.n;
    n = fc_count(fc, fc_which, n, false);
    for (int i = threadIdx.x; i < np * RADIX; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
#pragma unroll
        for (int p = 0; p < (NP > 0 ? NP : MAX_PASSES); p++) {
            if (NP == 0 && p >= np) break;
            const uint32_t d = (uint32_t)(k >> plan.shift[p]) & ((1u << plan.bits[p]) - 1);
            atomicAdd(&sh[p][d], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < np * RADIX; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Launches k_radix_hist for the plan's number of passes.
void launch_radix_hist(uint32_t blocks, cudaStream_t st, const uint64_t* keys, uint32_t n, const PassPlan& plan,
                       uint32_t* hist, FrameCounts* fc, int fc_which) {
    switch (plan.n) {
        case 1: k_radix_hist<1><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
        case 2: k_radix_hist<2><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
        case 3: k_radix_hist<3><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
        case 4: k_radix_hist<4><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
        case 5: k_radix_hist<5><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
        case 6: k_radix_hist<6><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
        default: k_radix_hist<0><<<blocks, 512, 0, st>>>(keys, n, plan, hist, fc, fc_which); break;
    }
}

// Packs the rasterizer's runs into one array and histograms every pass's
// digits on the way (the counting pass of the sort, fused with the copy).
// NP > 0: the plan has NP passes, unrolled so that each pass's shift and mask
// stay in registers; NP = 0: any number of passes.
template <int NP>
__global__ void __launch_bounds__(512) k_gather_hist(const uint64_t* __restrict__ runs, uint32_t run_slots,
                                                     const uint32_t* __restrict__ run_count,
                                                     const uint32_t* __restrict__ run_off, uint32_t n_runs,
                                                     uint64_t* __restrict__ out, uint32_t out_cap, PassPlan plan,
                                                     uint32_t* __restrict__ hist, const uint32_t* skip_flag) {
    __shared__ uint32_t sh[MAX_PASSES][RADIX];
    const int np = NP > 0 ? NP : plan.n;
    // passes the sort will skip need no digit counts
    const int p0 = (skip_flag && *skip_flag == 0) ? plan.skip : 0;
    for (int i = threadIdx.x; i < np * RADIX; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t r = blockIdx.x; r < n_runs; r += gridDim.x) {
        const uint32_t o = run_off[r];
        const uint32_t cnt = o < out_cap ? min(run_count[r], out_cap - o) : 0u;
        const uint64_t* src = runs + (uint64_t)r * run_slots;
        uint64_t* dst = out + o;
        for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
            const uint64_t k = src[i];
            dst[i] = k;
#pragma unroll
            for (int p = 0; p < (NP > 0 ? NP : MAX_PASSES); p++) {
                if (NP == 0 && p >= np) break;
                if (p < p0) continue;
                const uint32_t d = (uint32_t)(k >> plan.shift[p]) & ((1u << plan.bits[p]) - 1);
                atomicAdd(&sh[p][d], 1u);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < np * RADIX; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Exclusive scan of each pass's RADIX bins (one CTA of RADIX threads per pass).
__global__ void __launch_bounds__(RADIX) k_radix_hist_scan(uint32_t* hist) {
    uint32_t* h = hist + blockIdx.x * RADIX;
    uint32_t v = h[threadIdx.x];
    uint32_t ex = block_exclusive_scan<uint32_t>(v, nullptr);
    h[threadIdx.x] = ex;
}

// Digit `mask` of a key at bit `shift`: from the high word alone (HI, shift
// >= 32) or funnel-shifted out of both words.
template <bool HI>
__device__ __forceinline__ uint32_t key_digit(uint64_t k, int sh, uint32_t mask) {
    const uint32_t lo = (uint32_t)k, hi = (uint32_t)(k >> 32);
    return (HI ? __funnelshift_r(hi, 0u, sh) : __funnelshift_r(lo, hi, sh)) & mask;
}

// The lanes of the warp that hold digit d (d < 1024), from ten ballots: a
// fixed cost, where match.any slows down when the lanes' digits are mostly
// distinct.
__device__ __forceinline__ uint32_t ballot_peers(uint32_t d) {
    uint32_t peers = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < 10; b++) {
        const bool bit = (d >> b) & 1u;
        const uint32_t v = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? v : ~v;
    }
    return peers;
}

// One LSD pass over a tile of SORT_TILE keys.  HI: the digit lies in the high
// word (`sh` = shift - 32); else `sh` = shift < 32.  BALLOT: the warp's peers
// of a digit come from ballots rather than match.any.
// skip_mode 1: while *skip_flag == 0 the pass is skipped (it would move no
// key); skip_mode 2: likewise, but the tile is copied to `out` (the last of
// an odd number of skipped passes, so the keys end in the buffer the next
// pass reads).
template <bool HI, bool BALLOT>
__global__ void __launch_bounds__(SORT_THREADS, SORT_MIN_BLOCKS)
    k_onesweep(const uint64_t* __restrict__ in, uint64_t* __restrict__ out, uint32_t n, int sh, int bits,
               const uint32_t* __restrict__ global_off, uint32_t* lookback, uint32_t* tile_counter, uint32_t* err,
               FrameCounts* fc, int fc_which, const uint32_t* skip_flag, int skip_mode) {
    if (skip_mode && *skip_flag == 0) {
        if (skip_mode == 2) {
            const uint32_t nk = fc_count(fc, fc_which, n, false);
            const uint64_t b = (uint64_t)blockIdx.x * SORT_TILE;
            for (uint32_t i = threadIdx.x; i < SORT_TILE; i += SORT_THREADS)
                if (b + i < nk) out[b + i] = in[b + i];
        }
        return;
    }
    // per-warp digit counts, then the warp's offsets within each digit; the
    // column past the digits counts the keys past the end of the last tile
    __shared__ __align__(16) uint16_t s_hist[SORT_WARPS][RADIX + 2];
    __shared__ uint32_t s_start[RADIX];  // tile-local start of each digit
    __shared__ uint32_t s_off[RADIX];    // global start minus tile-local start (mod 2^32)
    extern __shared__ uint64_t s_keys[];  // SORT_TILE keys
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t mask = (1u << bits) - 1;
    if (tid == 0) {
        s_tile = atomicAdd(tile_counter, 1u);
        s_abort = 0;
    }
    {
        uint32_t* h = reinterpret_cast<uint32_t*>(&s_hist[0][0]);
        for (int i = tid; i < SORT_WARPS * (RADIX + 2) / 2; i += SORT_THREADS) h[i] = 0;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * SORT_TILE;
    // graph frames launch one CTA per tile of the capacity: the tiles past
    // the count have no keys and no successor that waits for them
    n = fc_count(fc, fc_which, n, tile == 0 && tid == 0);
    if (fc && base >= n && tile > 0) return;

    // Keys stay in registers; ranks are packed two per register and digits
    // recomputed from the keys, which keeps 14 keys per thread unspilled.
    uint64_t key[SORT_ITEMS];
    uint32_t rk[(SORT_ITEMS + 1) / 2];
    const uint64_t wbase = base + (uint64_t)warp * 32 * SORT_ITEMS + lane;
    const bool full = base + SORT_TILE <= n;
    if (full) {
#pragma unroll
        for (int k = 0; k < SORT_ITEMS; k++) key[k] = in[wbase + k * 32];
    } else {
#pragma unroll
        for (int k = 0; k < SORT_ITEMS; k++) key[k] = wbase + k * 32 < n ? in[wbase + k * 32] : 0;
    }
    // Warp-level multi-split ranking, in key order within the warp (stable);
    // keys past the end count in the spare digit column.
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint32_t d = full || wbase + k * 32 < n ? key_digit<HI>(key[k], sh, mask) : (uint32_t)RADIX;
        const uint32_t peers = BALLOT ? ballot_peers(d) : __match_any_sync(0xffffffffu, d);
        const uint32_t r = __popc(peers & lt);
        const uint32_t cnt = s_hist[warp][d];
        __syncwarp();
        if (r == 0) s_hist[warp][d] = (uint16_t)(cnt + __popc(peers));
        __syncwarp();
        if (k & 1)
            rk[k >> 1] |= (cnt + r) << 16;
        else
            rk[k >> 1] = cnt + r;
    }
    __syncthreads();
    // Per digit (one per thread): exclusive offsets across warps and the tile's count.
    const int d0 = tid;
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; w++) {
        const uint32_t v = s_hist[w][d0];
        s_hist[w][d0] = (uint16_t)cnt;
        cnt += v;
    }
    // The tile's digit counts are published at once (aggregate status; the
    // first tile's are already inclusive), so that later tiles can sum them
    // while this one places its keys in shared memory.
    uint32_t* mine = lookback + (uint64_t)tile * RADIX + d0;
    st_relaxed(mine, (tile == 0 ? ST_INC : ST_AGG) | cnt);
    // Tile-local digit starts: exclusive scan of the counts over the digits.
    s_start[d0] = block_exclusive_scan<uint32_t>(cnt, nullptr);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint32_t d = full || wbase + k * 32 < n ? key_digit<HI>(key[k], sh, mask) : (uint32_t)RADIX;
        const uint32_t rank = (rk[k >> 1] >> ((k & 1) * 16)) & 0xFFFFu;
        if (d < RADIX) s_keys[s_start[d] + s_hist[warp][d] + rank] = key[k];
    }
    // Decoupled look-back for the tile's global digit offsets: each thread
    // walks back over the predecessors of its digit, LB_WINDOW entries per
    // load round, summing until an inclusive prefix, and publishes its own.
    uint32_t excl = 0;
    if (tile > 0) {
        int t = (int)tile - 1;  // tiles < 2^30 / SORT_TILE
        uint32_t spins = 0;
        while (t >= 0) {
            uint32_t v[LB_WINDOW];
#pragma unroll
            for (int k = 0; k < LB_WINDOW; k++)
                v[k] = t - k >= 0 ? ld_relaxed(lookback + (size_t)(uint32_t)(t - k) * RADIX + d0) : (ST_INC | 0u);
            int used = 0;
            bool inc = false;
#pragma unroll
            for (int k = 0; k < LB_WINDOW; k++) {
                if (inc || used < k) break;  // stop at the first inclusive or unpublished entry
                const uint32_t stt = v[k] & ~ST_VAL;
                if (stt == 0) break;
                excl += v[k] & ST_VAL;
                used++;
                if (stt == ST_INC) inc = true;
            }
            if (inc) break;
            if (used == 0) {
                if (++spins > SPIN_LIMIT) {  // a predecessor never published
                    atomicExch(err, 1u);
                    s_abort = 1;
                    break;
                }
                __nanosleep(LB_SLEEP);
            }
            t -= used;
        }
        st_relaxed(mine, ST_INC | ((excl + cnt) & ST_VAL));
    }
    s_off[d0] = global_off[d0] + excl - s_start[d0];
    __syncthreads();
    if (s_abort) return;  // a predecessor never published: leave the output, the host reports the timeout
    const uint32_t valid = (n - base) < (uint64_t)SORT_TILE ? (uint32_t)(n - base) : (uint32_t)SORT_TILE;
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint32_t i = k * SORT_THREADS + tid;
        if (i < valid) {
            const uint64_t v = s_keys[i];
            const uint32_t pos = s_off[key_digit<HI>(v, sh, mask)] + i;
            if (pos < n) out[pos] = v;
        }
    }
}

constexpr size_t ONESWEEP_DYN_SMEM = SORT_TILE * sizeof(uint64_t);

// Opts the onesweep kernels into their dynamic shared memory (once per device).
cudaError_t onesweep_setup() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!done[dev]) {
        const void* fns[4] = {(const void*)k_onesweep<false, false>, (const void*)k_onesweep<true, false>,
                              (const void*)k_onesweep<false, true>, (const void*)k_onesweep<true, true>};
        for (int i = 0; i < 4 && e == cudaSuccess; i++)
            e = cudaFuncSetAttribute(fns[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ONESWEEP_DYN_SMEM);
        if (e != cudaSuccess) return e;
        done[dev] = true;
    }
    return cudaSuccess;
}

// One onesweep pass over the digit of `bits` bits at bit `shift`.
void launch_onesweep(uint32_t grid, cudaStream_t st, const uint64_t* in, uint64_t* out, uint32_t n, int shift,
                     int bits, const uint32_t* global_off, uint32_t* lookback, uint32_t* tile_counter, uint32_t* err,
                     FrameCounts* fc, int fc_which, bool ballot = false, const uint32_t* skip_flag = nullptr,
                     int skip_mode = 0) {
    const bool hi = shift >= 32;
    const int sh = hi ? shift - 32 : shift;
    auto k = hi ? (ballot ? k_onesweep<true, true> : k_onesweep<true, false>)
                : (ballot ? k_onesweep<false, true> : k_onesweep<false, false>);
    k<<<grid, SORT_THREADS, ONESWEEP_DYN_SMEM, st>>>(in, out, n, sh, bits, global_off, lookback, tile_counter, err,
                                                      fc, fc_which, skip_flag, skip_flag ? skip_mode : 0);
}

}  // namespace

size_t scan_scratch_bytes(uint32_t n) { return ((size_t)n / SCAN_TILE + 2) * sizeof(uint64_t); }

cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, Scratch* s, cudaStream_t st,
                     uint64_t* total_host, uint32_t* tail_dev) {
    uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    cudaError_t e = s->ensure(s->scan_sums, ((size_t)nb + 1) * sizeof(uint64_t));
    if (e != cudaSuccess) return e;
    uint64_t* sums = s->scan_sums.as<uint64_t>();
    count_launches(nb > 0 ? 3 : 1);
    if (nb > 0) k_scan_reduce<<<nb, SCAN_THREADS, 0, st>>>(in, n, sums);
    k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(sums, nb, out + n, tail_dev);
    if (nb > 0) k_scan_apply<<<nb, SCAN_THREADS, 0, st>>>(in, n, sums, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (total_host) {
        e = cudaMemcpyAsync(s->pinned, sums + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        *total_host = s->pinned[0];
    }
    return cudaSuccess;
}

cudaError_t reserve_frame_scratch(Scratch* s, uint32_t scan_n, uint32_t sort_n) {
    const size_t tiles = ((size_t)sort_n + SORT_TILE - 1) / SORT_TILE;
    cudaError_t e = s->ensure(s->scan_sums, ((size_t)scan_n / SCAN_TILE + 2) * sizeof(uint64_t));
    if (e == cudaSuccess) e = s->ensure(s->sort_hist, (size_t)MAX_PASSES * RADIX * 4);
    if (e == cudaSuccess) e = s->ensure(s->sort_lookback, std::max<size_t>(tiles, 1) * RADIX * 4);
    if (e == cudaSuccess) e = s->ensure(s->sort_counter, MAX_PASSES * 4);
    if (e == cudaSuccess) e = onesweep_setup();
    return e;
}

cudaError_t scan_block_counts(const uint32_t* counts, uint32_t* offsets, uint32_t n_blocks, Scratch* s,
                              cudaStream_t st, uint64_t* total_host) {
    return scan_u32(counts, offsets, n_blocks, s, st, total_host);
}

static PassPlan make_plan(int bit_lo, int bit_hi, int digit_bits) {
    PassPlan p{};
    p.skip = 0;
    int bits = std::max(0, bit_hi - bit_lo);
    digit_bits = std::min(9, std::max(1, digit_bits));
    p.n = (bits + digit_bits - 1) / digit_bits;
    if (p.n > MAX_PASSES) p.n = MAX_PASSES;
    int sh = bit_lo;
    for (int i = 0; i < p.n; i++) {
        int b = bits / p.n + (i < bits % p.n ? 1 : 0);  // even split, e.g. 42 bits -> 6 x 7
        p.shift[i] = sh;
        p.bits[i] = b;
        sh += b;
    }
    return p;
}

// The passes of [lo, mid), then those of [mid, hi); the first group may be skipped.
static PassPlan make_plan(const SortBits& sb, int digit_bits) {
    const PassPlan a = make_plan(sb.lo, sb.mid, digit_bits), b = make_plan(sb.mid, sb.hi, digit_bits);
    PassPlan p = a;
    for (int i = 0; i < b.n && p.n < MAX_PASSES; i++, p.n++) {
        p.shift[p.n] = b.shift[i];
        p.bits[p.n] = b.bits[i];
    }
    p.skip = sb.skip_flag ? a.n : 0;
    return p;
}

size_t radix_sort_scratch_bytes(uint32_t n, int bit_lo, int bit_hi, int digit_bits) {
    PassPlan p = make_plan(bit_lo, bit_hi, digit_bits);
    size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    return (size_t)p.n * RADIX * 4 + tiles * RADIX * 4 + 64;
}

static int sm_count() {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

cudaError_t radix_gather_hist(const uint64_t* runs, uint32_t run_slots, const uint32_t* run_count,
                              const uint32_t* run_off, uint32_t n_runs, uint64_t* out, SortBits sb, int digit_bits,
                              Scratch* s, cudaStream_t st, uint32_t out_cap) {
    const PassPlan plan = make_plan(sb, digit_bits);
    cudaError_t e = s->ensure(s->sort_hist, (size_t)MAX_PASSES * RADIX * 4);
    if (e != cudaSuccess) return e;
    uint32_t* hist = s->sort_hist.as<uint32_t>();
    if ((e = cudaMemsetAsync(hist, 0, (size_t)MAX_PASSES * RADIX * 4, st)) != cudaSuccess) return e;
    if (n_runs == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>(n_runs, (uint32_t)sm_count() * 4);
    count_launches(1);
#define CGB_GATHER(NP) \
    k_gather_hist<NP><<<blocks, 512, 0, st>>>(runs, run_slots, run_count, run_off, n_runs, out, out_cap, plan, hist, \
                                              sb.skip_flag)
    switch (plan.n) {
        case 1: CGB_GATHER(1); break;
        case 2: CGB_GATHER(2); break;
        case 3: CGB_GATHER(3); break;
        case 4: CGB_GATHER(4); break;
        case 5: CGB_GATHER(5); break;
        case 6: CGB_GATHER(6); break;
        default: CGB_GATHER(0); break;
    }
#undef CGB_GATHER
    return cudaGetLastError();
}

cudaError_t radix_sort_u64(uint64_t* keys, uint64_t* tmp, uint32_t n, SortBits sb, int digit_bits, Scratch* s,
                           uint32_t* err_flag, cudaStream_t st, uint64_t** result, int* passes, bool hist_ready,
                           FrameCounts* fc, int fc_which, uint32_t ballot_passes) {
    const PassPlan plan = make_plan(sb, digit_bits);
    *result = keys;
    if (passes) *passes = plan.n;
    if (n <= 1 || plan.n == 0) return cudaSuccess;
    if (n >= ST_VAL) return cudaErrorInvalidValue;
    uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    cudaError_t e = onesweep_setup();
    if (e != cudaSuccess) return e;
    if ((e = s->ensure(s->sort_hist, (size_t)MAX_PASSES * RADIX * 4)) != cudaSuccess) return e;
    if ((e = s->ensure(s->sort_lookback, (size_t)tiles * RADIX * 4)) != cudaSuccess) return e;
    if ((e = s->ensure(s->sort_counter, MAX_PASSES * 4)) != cudaSuccess) return e;
    uint32_t* hist = s->sort_hist.as<uint32_t>();
    uint32_t* lb = s->sort_lookback.as<uint32_t>();
    uint32_t* ctr = s->sort_counter.as<uint32_t>();
    if ((e = cudaMemsetAsync(ctr, 0, MAX_PASSES * 4, st)) != cudaSuccess) return e;
    if (!hist_ready) {
        if ((e = cudaMemsetAsync(hist, 0, (size_t)plan.n * RADIX * 4, st)) != cudaSuccess) return e;
        uint32_t hist_blocks = std::min<uint32_t>((n + 511) / 512, (uint32_t)sm_count() * 4);
        count_launches(1);
        launch_radix_hist(hist_blocks, st, keys, n, plan, hist, fc, fc_which);
    }
    count_launches(1 + plan.n);
    k_radix_hist_scan<<<plan.n, RADIX, 0, st>>>(hist);
    uint64_t* src = keys;
    uint64_t* dst = tmp;
    for (int p = 0; p < plan.n; p++) {
        if ((e = cudaMemsetAsync(lb, 0, (size_t)tiles * RADIX * 4, st)) != cudaSuccess) return e;
        // skippable passes: the last of an odd number copies its keys across
        const int skip_mode = p < plan.skip ? (p == plan.skip - 1 && (plan.skip & 1) ? 2 : 1) : 0;
        launch_onesweep(tiles, st, src, dst, n, plan.shift[p], plan.bits[p], hist + p * RADIX, lb, ctr + p, err_flag,
                        fc, fc_which, ((ballot_passes >> p) & 1u) != 0, sb.skip_flag, skip_mode);
        std::swap(src, dst);
    }
    *result = src;
    return cudaGetLastError();
}

// Self-test of the bounded wait: one CTA is given tile 1 of a two-tile pass
// (the tile counter starts at 1), so the predecessor it looks back at never
// publishes.  Its digit threads give up after SPIN_LIMIT rounds, set the error
// flag and return without writing; nothing traps or hangs.  Returns the flag.
cudaError_t selftest_bounded_wait(cudaStream_t st, uint32_t* flag_host) {
    cudaError_t e = onesweep_setup();
    if (e != cudaSuccess) return e;
    const uint32_t n = 2 * SORT_TILE;
    const size_t keys_b = (size_t)n * 8, hist_b = RADIX * 4, lb_b = 2 * RADIX * 4;
    void* buf = nullptr;
    if ((e = cudaMalloc(&buf, 2 * keys_b + hist_b + lb_b + 64)) != cudaSuccess) return e;
    uint8_t* b = static_cast<uint8_t*>(buf);
    uint64_t* in = reinterpret_cast<uint64_t*>(b);
    uint64_t* out = reinterpret_cast<uint64_t*>(b + keys_b);
    uint32_t* hist = reinterpret_cast<uint32_t*>(b + 2 * keys_b);
    uint32_t* lb = reinterpret_cast<uint32_t*>(b + 2 * keys_b + hist_b);
    uint32_t* ctr = reinterpret_cast<uint32_t*>(b + 2 * keys_b + hist_b + lb_b);
    uint32_t* err = ctr + 1;
    const uint32_t one = 1;
    e = cudaMemsetAsync(buf, 0, 2 * keys_b + hist_b + lb_b + 64, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctr, &one, 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        count_launches(1);
        launch_onesweep(1, st, in, out, n, 0, 8, hist, lb, ctr, err, nullptr, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(flag_host, err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaError_t e2 = cudaFree(buf);
    return e != cudaSuccess ? e : e2;
}

}  // namespace cgb

// ---------------------------------------------------------------------------
// Allocation-free sort entry point.
//
// For callers that cannot allocate device memory while they run: a render
// thread that has reserved its memory up front, or a host process whose
// device memory is owned by another allocator (a framework's caching pool),
// where a cudaMalloc either fails or, like cudaFree, synchronizes the whole
// device and stalls every other stream.  The sort's scratch (digit
// histograms, tile counters, the look-back table and the error flag) lives in
// one file-scope device array instead, sized for at most
// NOALLOC_MAX_KEYS keys; every GPU that loads this library holds it (about
// 5 MB) until the process exits.  Every call shares that array and leaves its
// contents behind: each call clears what must start at zero, and calls whose
// work overlaps on the GPU (two streams, or two host threads) race on it.
// ---------------------------------------------------------------------------

namespace cgb {
namespace {

constexpr uint32_t NOALLOC_MAX_KEYS = 1u << 24;                    // 16,777,216 keys
constexpr uint32_t NOALLOC_TILES = (NOALLOC_MAX_KEYS + SORT_TILE - 1) / SORT_TILE;  // onesweep tiles
constexpr uint32_t NOALLOC_HIST_WORDS = MAX_PASSES * RADIX;
constexpr uint32_t NOALLOC_CTR_OFF = NOALLOC_HIST_WORDS;            // MAX_PASSES tile counters
constexpr uint32_t NOALLOC_ERR_OFF = NOALLOC_CTR_OFF + 64;          // error flag
constexpr uint32_t NOALLOC_LB_OFF = NOALLOC_ERR_OFF + 64;           // look-back table
constexpr uint32_t NOALLOC_WORDS = NOALLOC_LB_OFF + NOALLOC_TILES * RADIX;

static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_WORDS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the array's name is only a host-side stand-in).
cudaError_t noalloc_scratch(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = (uint32_t*)p;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

}  // namespace

}  // namespace cgb

extern "C" CGB_EXPORT cgb_status cgb_sort_keys_noalloc(uint64_t* keys, uint64_t* out, size_t n, uint32_t bit_lo,
                                                       uint32_t bit_hi, void* stream) {
    using namespace cgb;
    if (n > NOALLOC_MAX_KEYS) return CGB_ERR_CAPACITY;
    if (bit_lo >= bit_hi || bit_hi > 64) return CGB_ERR_INVALID_ARG;
    if (n > 0 && (!keys || !out)) return CGB_ERR_INVALID_ARG;
    // the two buffers ping-pong, so any overlap of [keys, keys+n) and [out, out+n) would corrupt the keys
    if (n > 0 && (uintptr_t)keys < (uintptr_t)(out + n) && (uintptr_t)out < (uintptr_t)(keys + n))
        return CGB_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    // The call reads its error flag back and waits for the stream, neither of
    // which a capturing stream allows: refuse it before any work.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        return CGB_ERR_INVALID_ARG;
    }
    if (cap != cudaStreamCaptureStatusNone) return CGB_ERR_INVALID_ARG;
    if (n <= 1) {
        if (n == 1 && cudaMemcpyAsync(out, keys, 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return CGB_ERR_DEVICE;
        return cudaStreamSynchronize(st) == cudaSuccess ? CGB_OK : CGB_ERR_DEVICE;
    }
    uint32_t* scratch = nullptr;
    if (noalloc_scratch(&scratch) != cudaSuccess) return CGB_ERR_DEVICE;
    if (onesweep_setup() != cudaSuccess) return CGB_ERR_DEVICE;
    uint32_t* hist = scratch;
    uint32_t* ctr = scratch + NOALLOC_CTR_OFF;
    uint32_t* err = scratch + NOALLOC_ERR_OFF;
    uint32_t* lb = scratch + NOALLOC_LB_OFF;
    const PassPlan plan = make_plan((int)bit_lo, (int)bit_hi, 9);
    const uint32_t nn = (uint32_t)n;
    const uint32_t tiles = (nn + SORT_TILE - 1) / SORT_TILE;
    cudaError_t e = cudaMemsetAsync(scratch, 0, (size_t)NOALLOC_LB_OFF * 4, st);  // hist, counters, error flag
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t hist_blocks = std::min<uint32_t>((nn + 511) / 512, (uint32_t)sms * 4);
    if (e == cudaSuccess) {
        count_launches(1);
        launch_radix_hist(hist_blocks, st, keys, nn, plan, hist, nullptr, 0);
        count_launches(1 + plan.n);
        k_radix_hist_scan<<<plan.n, RADIX, 0, st>>>(hist);
        e = cudaGetLastError();
    }
    // Ping-pong between the caller's two buffers; the result must end in `out`.
    uint64_t* src = keys;
    uint64_t* dst = out;
    for (int p = 0; p < plan.n && e == cudaSuccess; p++) {
        e = cudaMemsetAsync(lb, 0, (size_t)tiles * RADIX * 4, st);
        if (e != cudaSuccess) break;
        launch_onesweep(tiles, st, src, dst, nn, plan.shift[p], plan.bits[p], hist + p * RADIX, lb, ctr + p, err,
                        nullptr, 0);
        e = cudaGetLastError();
        std::swap(src, dst);
    }
    if (e == cudaSuccess && src != out) e = cudaMemcpyAsync(out, src, (size_t)nn * 8, cudaMemcpyDeviceToDevice, st);
    uint32_t flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return CGB_ERR_DEVICE;
    return flag ? CGB_ERR_DEVICE_TIMEOUT : CGB_OK;
}
