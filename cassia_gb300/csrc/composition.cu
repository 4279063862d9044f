// C ABI of cassia_gb300: mold's Composition / Layer / Props API
// (mold/src/composition.rs, mold/src/layer.rs) over the GPU pipeline
//   build lines -> rasterize -> radix sort -> carries / work items -> paint.
//
// Host state mirrors mold: layers by id (FxHashMap<u16, Layer> in the
// reference), an IdSet of free ids, orders_to_layers, per-cache layer counts.
// Lines live on the device (the LinesBuilder SoA, surpass/src/segment.rs:30-89)
// and are garbage-collected by the reference's rule (composition.rs:124-142).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "cgb_internal.cuh"

using namespace cgb;

namespace {

thread_local std::string g_last_error;

cgb_status fail(cgb_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

cgb_status from_cuda(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return CGB_OK;
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(CGB_ERR_OUT_OF_MEMORY, m);
    return fail(CGB_ERR_DEVICE, m);
}

#define CK(expr)                                                  \
    do {                                                          \
        cudaError_t _e = (expr);                                  \
        if (_e != cudaSuccess) return c->cuda_fail(_e, #expr);   \
    } while (0)

int bits_for(uint64_t max_value) {  // bits to hold values in [0, max_value]
    int b = 0;
    while (b < 64 && (max_value >> b) != 0) b++;
    return std::max(b, 1);
}

struct HostProps {
    cgb_props c{};
    std::vector<float> stops;
    bool operator==(const HostProps& o) const {
        if (c.fill_rule != o.c.fill_rule || c.func != o.c.func) return false;
        if (c.func == CGB_FUNC_CLIP) return c.clip_layers == o.c.clip_layers;
        if (c.is_clipped != o.c.is_clipped || c.blend_mode != o.c.blend_mode || c.fill_kind != o.c.fill_kind)
            return false;
        if (c.fill_kind == CGB_FILL_SOLID) return std::memcmp(c.color, o.c.color, sizeof(c.color)) == 0;
        return c.gradient_type == o.c.gradient_type && c.n_stops == o.c.n_stops &&
               std::memcmp(c.gradient_start, o.c.gradient_start, 8) == 0 &&
               std::memcmp(c.gradient_end, o.c.gradient_end, 8) == 0 && stops == o.stops;
    }
};

HostProps default_props() {
    HostProps p;
    p.c.fill_rule = CGB_FILL_NONZERO;
    p.c.func = CGB_FUNC_DRAW;
    p.c.blend_mode = CGB_BLEND_OVER;
    p.c.fill_kind = CGB_FILL_SOLID;
    p.c.color[3] = 1.0f;  // Fill::default (style.rs:183-187)
    return p;
}

// The fields a per-frame transform update touches share the first cache line.
struct alignas(64) HostLayer {
    bool present = false;  // the layer exists in mold's `layers` map
    bool enabled = true;
    bool has_transform = false;
    bool has_order = false;
    uint32_t order = 0;
    uint32_t unchanged = 0;  // SmallBitSet of cache ids (mold/src/layer.rs:101-142)
    float t[6] = {1, 0, 0, 1, 0, 0};
    uint64_t len = 0;
    HostProps props = default_props();
};

struct CacheState {
    DevBuf prev;  // int32 per tile, -1 = None
    uint64_t tiles = 0;
};

// Page-locked host storage for the layer table mirror, so that its upload is
// one asynchronous DMA instead of a staged pageable copy.  Falls back to
// pageable memory if pinning fails.
template <class T>
struct PinnedAllocator {
    using value_type = T;
    PinnedAllocator() = default;
    template <class U>
    PinnedAllocator(const PinnedAllocator<U>&) {}
    T* allocate(size_t n) {
        void* p = nullptr;
        if (cudaMallocHost(&p, n * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            p = std::malloc(n * sizeof(T));
            if (!p) throw std::bad_alloc();
            std::lock_guard<std::mutex> lock(registry_mutex());
            pageable().insert(p);
        }
        return static_cast<T*>(p);
    }
    void deallocate(T* p, size_t) {
        bool was_pageable = false;
        {
            std::lock_guard<std::mutex> lock(registry_mutex());
            auto it = pageable().find(p);
            if (it != pageable().end()) {
                pageable().erase(it);
                was_pageable = true;
            }
        }
        if (was_pageable) std::free(p);
        else cudaFreeHost(p);
    }
    static std::mutex& registry_mutex() {  // handles are used from several threads
        static std::mutex m;
        return m;
    }
    static std::set<void*>& pageable() {
        static std::set<void*> s;
        return s;
    }
    template <class U>
    bool operator==(const PinnedAllocator<U>&) const { return true; }
    template <class U>
    bool operator!=(const PinnedAllocator<U>&) const { return false; }
};

}  // namespace

// Capacities of a frame graph's buffers: the counts of the frame it was
// captured after, plus headroom.
struct FrameCaps {
    uint32_t steps = 0, segs = 0, tls = 0, items = 0;
};

// A captured frame: replayed while the frame geometry (its signature) and
// every buffer it uses (pointer and size) stay the same.
struct FrameGraph {
    cudaGraphExec_t exec = nullptr;
    FrameCaps caps;
    std::vector<std::pair<const void*, size_t>> bufs;
    uint64_t launches = 0;
    uint32_t sort_passes = 0, item_sort_passes = 0;
};

struct cgb_composition {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool wide = false;
    uint32_t max_ids = 1u << 16;
    Scratch s;
    cgb_tuning tuning{9, 256, 2048, 4};  // radix bits, raster block, steps per block, painter warps
    cgb_stats stats{};

    // LinesBuilder (device SoA)
    DevBuf p0x, p0y, p1x, p1y, lids;
    uint64_t n_lines = 0, line_cap = 0;
    bool has_default_transform = false;
    float default_transform[6] = {1, 0, 0, 1, 0, 0};

    // mold's `layers: FxHashMap<u16, Layer>` as a dense array by id, and its
    // IdSet as a used-flag array, the freed ids below next_fresh, and next_fresh.
    std::vector<HostLayer> layers;
    std::vector<uint8_t> used;
    std::set<uint32_t> released;
    uint32_t next_fresh = 0;
    uint64_t enabled_len = 0;            // Composition::actual_len, kept incrementally
    std::vector<LayerRec, PinnedAllocator<LayerRec>> layer_recs;  // host mirror of the device layer table
    uint32_t dirty_lo = UINT32_MAX, dirty_hi = 0;
    bool layers_grew = true;
    DevBuf d_layers;
    uint32_t n_layer_recs = 0;
    // LayerProps by order (orders_to_layers + Layer::props), rebuilt when dirty
    bool props_dirty = true;
    std::vector<PaintProps> props_host;
    std::vector<GradRec> grads_host;
    std::vector<GradStop> stops_host;
    std::vector<uint32_t> order_layer;
    uint32_t n_orders = 1;
    uint32_t features = 0;     // FEAT_* of the enabled layers' props
    // cassia_render input of the current frame (import mode: no lines, props from stylings)
    const uint64_t* import_segs = nullptr;
    uint64_t import_n = 0;
    DevBuf d_import;
    uint64_t props_version = 1, props_uploaded = 0;

    // frame buffers
    DevBuf recs, lengths, step_off, bcounts, boff, segs_a, segs_b;
    DevBuf tl_start, tl_key, tl_cover, tl_carry, tl_flags, item_count, item_off, items_a, items_b, tile_start;
    DevBuf blk_cover, blk_head, rlb, item_state, written;
    DevBuf d_props, d_grads, d_stops, d_unchanged, out_rgba, err, dflt_t, d_scenes, d_row_scene;
    // flatten staging
    DevBuf f_kinds, f_points, f_cmd_off, f_pt_off, f_t9, f_has_t, f_path_layer, f_counts, f_off;
    // GC staging
    DevBuf g_flags, g_off, g_tmp[5];

    uint32_t caches_used = 0;
    std::map<int32_t, CacheState> caches;

    cudaEvent_t ev[8] = {};
    nvtxRangeId_t nvtx_range = 0;  // the open stage range (visible in Nsight tools)
    bool nvtx_open = false;

    // frame graphs (cgb_set_graph_mode), by frame signature
    bool graph_mode = false;
    float graph_headroom = 0.125f;
    std::map<std::string, FrameGraph> graphs;
    DevBuf d_counts;                // FrameCounts of the frame in flight
    FrameCounts* h_counts = nullptr;  // pinned readback of d_counts
    bool last_replayed = false;
    bool capturing = false;         // the stream is capturing a frame graph

    // incremental frames (cgb_set_incremental): the sorted segments of the
    // last frame stay resident and only changed layers are rasterized again
    bool incremental = false;
    std::vector<uint32_t> rast_ids;   // layers whose geometry changed since the last frame
    std::vector<uint8_t> rast_flag;   // by id: listed in rast_ids
    std::vector<int32_t> rast_order;  // by id: the order its resident segments carry, -1 none
    std::vector<uint8_t, PinnedAllocator<uint8_t>> h_rast_dirty;  // uploaded asynchronously
    DevBuf d_rast_dirty;              // by order (max_ids bytes): 1 = rasterize again
    DevBuf resident;                  // sorted segments of the last frame, local key layout
    uint64_t resident_n = 0;
    uint32_t resident_ob = LOCAL_ORDER_BITS, resident_cb = LOCAL_COL_BITS;  // its key layout
    bool resident_valid = false;
    uint32_t resident_rows = 0, resident_row_len = 0;
    // frame-level buffers of an incremental frame (on the handle that renders it)
    DevBuf segs_k, segs_m, d_keep, d_scene_ids, d_ranges, d_extract, merge_split;
    // sync-free incremental frames: capacities from the earlier incremental
    // frames (steps and segs: those of the changed layers; tls and items:
    // the whole frame's), with headroom
    FrameCaps incr_caps;
    bool incr_caps_valid = false;
    uint64_t last_new_segs = 0;  // segments the last staged frame rasterized
    uint32_t incr_form = 0;      // the last frame: 0 full, 1 incremental staged, 2 incremental sync-free

    cgb_status cuda_fail(cudaError_t e, const char* where) {
        if (e == cudaErrorMemoryAllocation && s.over_budget) {
            s.over_budget = false;
            return fail(CGB_ERR_OVER_BUDGET, std::string(where) + ": HBM budget exceeded");
        }
        return from_cuda(e, where);
    }
};

namespace cgb {

static std::atomic<uint64_t> g_launches{0};
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaError_t Scratch::ensure(DevBuf& b, size_t bytes) {
    if (bytes <= b.cap) return cudaSuccess;
    size_t want = std::max(bytes, b.cap + b.cap / 4);
    want = (want + 255) & ~(size_t)255;
    if (budget && used - b.cap + want > budget) {
        want = bytes;
        if (used - b.cap + want > budget) {
            over_budget = true;
            return cudaErrorMemoryAllocation;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e;
    }
    if (b.p) cudaFree(b.p);
    used = used - b.cap + want;
    b.p = p;
    b.cap = want;
    return cudaSuccess;
}

void Scratch::release(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    used -= b.cap;
    b.p = nullptr;
    b.cap = 0;
}

}  // namespace cgb

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Grows a device buffer while keeping its first `keep` bytes.
cudaError_t grow_keep(cgb_composition* c, DevBuf& b, size_t bytes, size_t keep) {
    if (bytes <= b.cap) return cudaSuccess;
    DevBuf nb;
    size_t want = std::max(bytes, b.cap * 2);
    cudaError_t e = c->s.ensure(nb, want);
    if (e != cudaSuccess) {
        e = c->s.ensure(nb, bytes);
        if (e != cudaSuccess) return e;
    }
    if (keep && b.p) {
        e = cudaMemcpyAsync(nb.p, b.p, keep, cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return e;
    }
    c->s.release(b);
    b = nb;
    return cudaSuccess;
}

cudaError_t ensure_lines(cgb_composition* c, uint64_t n) {
    if (n <= c->line_cap) return cudaSuccess;
    uint64_t cap = std::max<uint64_t>(n, c->line_cap * 2);
    cap = std::max<uint64_t>(cap, 1024);
    DevBuf* arrs[5] = {&c->p0x, &c->p0y, &c->p1x, &c->p1y, &c->lids};
    for (DevBuf* a : arrs) {
        cudaError_t e = grow_keep(c, *a, cap * 4, c->n_lines * 4);
        if (e != cudaSuccess) return e;
    }
    c->line_cap = cap;
    return cudaSuccess;
}

HostLayer* find_layer(cgb_composition* c, uint32_t id) {
    return id < c->layers.size() && c->layers[id].present ? &c->layers[id] : nullptr;
}

// Incremental frames: layer `id`'s geometry changed (transform, enabled,
// order, lines, removal), so its old and new orders are rasterized again.
void mark_raster(cgb_composition* c, uint32_t id) {
    if (!c->incremental) return;
    if (id >= c->rast_flag.size()) c->rast_flag.resize((size_t)id + 1, 0);
    if (!c->rast_flag[id]) {
        c->rast_flag[id] = 1;
        c->rast_ids.push_back(id);
    }
}

// Refreshes the device-table record of layer `id` and marks it for upload.
void touch(cgb_composition* c, uint32_t id) {
    mark_raster(c, id);
    if (id >= c->layer_recs.size()) {
        c->layer_recs.resize((size_t)id + 1);
        c->layers_grew = true;
    }
    const HostLayer& l = c->layers[id];
    LayerRec& r = c->layer_recs[id];
    r.flags = l.present ? (LAYER_PRESENT | (l.enabled ? LAYER_ENABLED : 0u) | (l.has_transform ? LAYER_HAS_TRANSFORM : 0u) |
                           (l.has_order ? LAYER_HAS_ORDER : 0u))
                        : 0u;
    r.order = l.order;
    std::memcpy(r.t, l.t, sizeof(r.t));
    c->dirty_lo = std::min(c->dirty_lo, id);
    c->dirty_hi = std::max(c->dirty_hi, id + 1);
}

void mark_used(cgb_composition* c, uint32_t id) {
    if (id >= c->used.size()) c->used.resize((size_t)id + 1, 0);
    if (!c->used[id]) {
        c->used[id] = 1;
        c->released.erase(id);
    }
}

// IdSet::release (mold/src/layer.rs:74-98)
void release_id(cgb_composition* c, uint32_t id) {
    if (id < c->used.size()) c->used[id] = 0;
    if (id < c->next_fresh) c->released.insert(id);
}

// insert_segments bookkeeping (mold/src/composition.rs:58-79)
void insert_bookkeeping(cgb_composition* c, uint32_t id, uint64_t n) {
    if (id >= c->layers.size()) c->layers.resize((size_t)id + 1);
    HostLayer& l = c->layers[id];
    if (!l.present) {
        l = HostLayer();
        l.present = true;
    }
    const uint64_t before = l.enabled ? l.len : 0;
    l.has_order = true;
    l.order = id;
    l.enabled = true;
    l.len += n;
    c->enabled_len += l.len - before;
    mark_used(c, id);
    touch(c, id);
    c->props_dirty = true;
}

uint64_t actual_len(cgb_composition* c) { return c->enabled_len; }

cgb_status upload_layers(cgb_composition* c) {
    if (c->dirty_lo >= c->dirty_hi && !c->layers_grew) return CGB_OK;
    const size_t n = std::max<size_t>(c->layer_recs.size(), 1);
    if (c->layer_recs.empty()) c->layer_recs.resize(1);
    size_t lo = c->dirty_lo, hi = c->dirty_hi;
    if (c->layers_grew || c->d_layers.cap < n * sizeof(LayerRec)) {
        CK(c->s.ensure(c->d_layers, n * sizeof(LayerRec)));
        lo = 0;
        hi = n;
    }
    if (hi > lo)
        CK(cudaMemcpyAsync(c->d_layers.as<LayerRec>() + lo, c->layer_recs.data() + lo, (hi - lo) * sizeof(LayerRec),
                           cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->n_layer_recs = (uint32_t)c->layer_recs.size();
    c->dirty_lo = UINT32_MAX;
    c->dirty_hi = 0;
    c->layers_grew = false;
    return CGB_OK;
}

// LayerProps by order (composition.rs:229-237, 247-284): orders_to_layers over
// the enabled layers, ascending ids, so that the highest id wins a shared order.
void rebuild_props(cgb_composition* c) {
    uint32_t n_orders = 1;
    for (size_t id = 0; id < c->layers.size(); id++) {
        const HostLayer& l = c->layers[id];
        if (l.present && l.enabled) n_orders = std::max(n_orders, l.order + 1);
    }
    c->order_layer.assign(n_orders, UINT32_MAX);
    for (size_t id = 0; id < c->layers.size(); id++) {
        const HostLayer& l = c->layers[id];
        if (l.present && l.enabled) c->order_layer[l.order] = (uint32_t)id;
    }
    c->props_host.assign(n_orders, PaintProps{CGB_FILL_NONZERO, CGB_BLEND_OVER,
                                              PROPS_SOLID | PROPS_DRAW | PROPS_OPAQUE_OVER, 0, {0, 0, 0, 1}});
    c->features = 0;
    c->grads_host.clear();
    c->stops_host.clear();
    for (uint32_t o = 0; o < n_orders; o++) {
        if (c->order_layer[o] == UINT32_MAX) continue;
        const HostProps& hp = c->layers[c->order_layer[o]].props;
        const cgb_props& p = hp.c;
        PaintProps& pp = c->props_host[o];
        pp.fill_rule = p.fill_rule;
        pp.blend_mode = p.blend_mode;
        pp.flags = PROPS_PRESENT;
        pp.aux = 0;
        std::memcpy(pp.color, p.color, sizeof(pp.color));
        if (p.func == CGB_FUNC_CLIP) {  // Func::Clip(n): masks the next n layers
            pp.flags |= PROPS_CLIP;
            pp.aux = p.clip_layers;
            c->features |= FEAT_CLIPS;
            continue;
        }
        pp.flags |= PROPS_DRAW;
        if (p.is_clipped) {
            pp.flags |= PROPS_CLIPPED;
            c->features |= FEAT_CLIPS;
        }
        if (p.fill_kind == CGB_FILL_SOLID) {
            pp.flags |= PROPS_SOLID;
            if (p.blend_mode == CGB_BLEND_OVER && p.color[3] == 1.0f) pp.flags |= PROPS_OPAQUE_OVER;
        } else {
            // GradientBuilder::build (style.rs:66-84): a stop given as 0 takes
            // its evenly spaced default position
            GradRec g{p.gradient_type, p.n_stops, (uint32_t)c->stops_host.size(), 0,
                      {p.gradient_start[0], p.gradient_start[1]}, {p.gradient_end[0], p.gradient_end[1]}};
            const float inc = 1.0f / (float)(p.n_stops - 1);
            for (uint32_t i = 0; i < p.n_stops; i++) {
                const float* st = hp.stops.data() + 5 * (size_t)i;
                GradStop gs{{st[0], st[1], st[2], st[3]}, st[4] == -0.0f ? (float)i * inc : st[4], {0, 0, 0}};
                c->stops_host.push_back(gs);
            }
            pp.aux = (uint32_t)c->grads_host.size();
            c->grads_host.push_back(g);
            c->features |= FEAT_GRADIENTS;
        }
    }
    c->n_orders = n_orders;
    c->props_dirty = false;
    c->props_version++;
}

// Composition::remove_disabled (mold/src/composition.rs:124-142)
cgb_status remove_disabled(cgb_composition* c) {
    if (c->n_lines < actual_len(c) * 2) return CGB_OK;
    cgb_status st = upload_layers(c);
    if (st) return st;
    uint32_t n = (uint32_t)c->n_lines;
    if (n > 0) {
        CK(c->s.ensure(c->g_flags, (size_t)n * 4));
        CK(c->s.ensure(c->g_off, ((size_t)n + 1) * 4));
        for (int k = 0; k < 5; k++) CK(c->s.ensure(c->g_tmp[k], (size_t)n * 4));
        const float* in4[4] = {c->p0x.as<float>(), c->p0y.as<float>(), c->p1x.as<float>(), c->p1y.as<float>()};
        float* out4[4] = {c->g_tmp[0].as<float>(), c->g_tmp[1].as<float>(), c->g_tmp[2].as<float>(),
                          c->g_tmp[3].as<float>()};
        uint32_t kept = 0;
        CK(launch_compact_lines(in4, c->lids.as<uint32_t>(), n, c->d_layers.as<LayerRec>(), c->n_layer_recs, out4,
                                c->g_tmp[4].as<uint32_t>(), c->g_flags.as<uint32_t>(), c->g_off.as<uint32_t>(), &c->s,
                                c->stream, &kept));
        DevBuf* arrs[5] = {&c->p0x, &c->p0y, &c->p1x, &c->p1y, &c->lids};
        for (int k = 0; k < 5; k++)
            CK(cudaMemcpyAsync(arrs[k]->p, c->g_tmp[k].p, (size_t)kept * 4, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->n_lines = kept;
    }
    for (uint32_t id = 0; id < c->layers.size(); id++) {
        HostLayer& l = c->layers[id];
        if (l.present && !l.enabled) {
            l = HostLayer();
            release_id(c, id);
            touch(c, id);
        }
    }
    c->props_dirty = true;
    return CGB_OK;
}

// Validates a command stream; returns the float count or -1.
int64_t count_floats(const uint32_t* kinds, size_t n) {
    int64_t f = 0;
    for (size_t i = 0; i < n; i++) {
        switch (kinds[i]) {
            case CGB_CMD_LINE: f += 4; break;
            case CGB_CMD_QUAD: f += 6; break;
            case CGB_CMD_RAT_QUAD: f += 9; break;
            case CGB_CMD_CUBIC: f += 8; break;
            case CGB_CMD_RAT_CUBIC: f += 12; break;
            case CGB_CMD_CLOSE: break;
            default: return -1;
        }
    }
    return f;
}

cgb_status insert_paths(cgb_composition* c, size_t n_paths, const uint32_t* layer_ids, const uint64_t* cmd_offsets,
                        const uint32_t* kinds, const uint64_t* point_offsets, const float* points,
                        const float* transforms9, const uint8_t* has_transform) {
    if (n_paths == 0) return CGB_OK;
    if (!layer_ids || !cmd_offsets || !kinds || !point_offsets || !points)
        return fail(CGB_ERR_INVALID_ARG, "insert_paths: null array");
    for (size_t k = 0; k < n_paths; k++) {
        if (layer_ids[k] >= c->max_ids) return fail(CGB_ERR_LAYER_LIMIT, "insert_paths: layer id out of range");
        if (cmd_offsets[k + 1] < cmd_offsets[k] || point_offsets[k + 1] < point_offsets[k])
            return fail(CGB_ERR_INVALID_ARG, "insert_paths: offsets not monotone");
        int64_t f = count_floats(kinds + cmd_offsets[k], cmd_offsets[k + 1] - cmd_offsets[k]);
        if (f < 0) return fail(CGB_ERR_INVALID_ARG, "insert_paths: unknown command kind");
        if ((uint64_t)f != point_offsets[k + 1] - point_offsets[k])
            return fail(CGB_ERR_INVALID_ARG, "insert_paths: point count does not match the commands");
    }
    if (n_paths >= (1u << 31)) return fail(CGB_ERR_INVALID_ARG, "insert_paths: too many paths");
    const uint64_t n_cmds = cmd_offsets[n_paths] - cmd_offsets[0];
    const uint64_t n_floats = point_offsets[n_paths] - point_offsets[0];
    // rebase offsets to the uploaded slices
    std::vector<uint64_t> co(n_paths + 1), po(n_paths + 1);
    for (size_t k = 0; k <= n_paths; k++) {
        co[k] = cmd_offsets[k] - cmd_offsets[0];
        po[k] = point_offsets[k] - point_offsets[0];
    }
    CK(c->s.ensure(c->f_kinds, std::max<size_t>(n_cmds, 1) * 4));
    CK(c->s.ensure(c->f_points, std::max<size_t>(n_floats, 1) * 4));
    CK(c->s.ensure(c->f_cmd_off, (n_paths + 1) * 8));
    CK(c->s.ensure(c->f_pt_off, (n_paths + 1) * 8));
    CK(c->s.ensure(c->f_path_layer, n_paths * 4));
    CK(c->s.ensure(c->f_counts, n_paths * 4));
    CK(c->s.ensure(c->f_off, (n_paths + 1) * 4));
    cudaStream_t st = c->stream;
    CK(cudaMemcpyAsync(c->f_kinds.p, kinds + cmd_offsets[0], n_cmds * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->f_points.p, points + point_offsets[0], n_floats * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->f_cmd_off.p, co.data(), (n_paths + 1) * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->f_pt_off.p, po.data(), (n_paths + 1) * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->f_path_layer.p, layer_ids, n_paths * 4, cudaMemcpyHostToDevice, st));
    const float* dt = nullptr;
    const uint8_t* dh = nullptr;
    if (transforms9 && has_transform) {
        CK(c->s.ensure(c->f_t9, n_paths * 9 * 4));
        CK(c->s.ensure(c->f_has_t, n_paths));
        CK(cudaMemcpyAsync(c->f_t9.p, transforms9, n_paths * 9 * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(c->f_has_t.p, has_transform, n_paths, cudaMemcpyHostToDevice, st));
        dt = c->f_t9.as<float>();
        dh = c->f_has_t.as<uint8_t>();
    }
    CK(launch_flatten(0, c->f_kinds.as<uint32_t>(), c->f_points.as<float>(), c->f_cmd_off.as<uint64_t>(),
                      c->f_pt_off.as<uint64_t>(), dt, dh, c->f_path_layer.as<uint32_t>(), (uint32_t)n_paths,
                      c->f_counts.as<uint32_t>(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, st));
    uint64_t total = 0;
    CK(scan_u32(c->f_counts.as<uint32_t>(), c->f_off.as<uint32_t>(), (uint32_t)n_paths, &c->s, st, &total));
    if (c->n_lines + total >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "insert_paths: more than 2^32 lines");
    CK(ensure_lines(c, c->n_lines + total));
    const uint64_t base = c->n_lines;
    CK(launch_flatten(1, c->f_kinds.as<uint32_t>(), c->f_points.as<float>(), c->f_cmd_off.as<uint64_t>(),
                      c->f_pt_off.as<uint64_t>(), dt, dh, c->f_path_layer.as<uint32_t>(), (uint32_t)n_paths, nullptr,
                      c->f_off.as<uint32_t>(), c->p0x.as<float>() + base, c->p0y.as<float>() + base,
                      c->p1x.as<float>() + base, c->p1y.as<float>() + base, c->lids.as<uint32_t>() + base, st));
    std::vector<uint32_t> counts(n_paths);
    CK(cudaMemcpyAsync(counts.data(), c->f_counts.p, n_paths * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c->n_lines += total;
    for (size_t k = 0; k < n_paths; k++) insert_bookkeeping(c, layer_ids[k], counts[k]);
    return CGB_OK;
}

// One scene of a frame as the host prepares it.
struct SceneInput {
    cgb_composition* comp;
    const cgb_buffer* buf;
    const float* bg;
    const cgb_rect* crop;
    CacheState* cache;
    SceneDesc d;
    size_t staging_off;  // offset in the frame's host-output staging buffer
    // incremental frames: 0 no; 1 all lines rasterized, the resident
    // segments rebuilt; 2 only changed layers rasterized, the resident ones kept
    int incr = 0;
};

// Stage boundary: records CUDA event k on the stream (the stage times of
// cgb_stats) and closes the open NVTX range, opening `next` if given.
cudaError_t stage_mark(cgb_composition* c, int k, cudaStream_t st, const char* next) {
    // in a frame graph the event is a node of the graph, recorded at each replay
    if (c->capturing) return cudaEventRecordWithFlags(c->ev[k], st, cudaEventRecordExternal);
    if (c->nvtx_open) nvtxRangeEnd(c->nvtx_range);
    c->nvtx_open = next != nullptr;
    if (next) c->nvtx_range = nvtxRangeStartA(next);
    return cudaEventRecord(c->ev[k], st);
}

// LinesBuilder::build + Rasterizer::rasterize (+ re-keying / culling in
// render mode) over every scene of the frame.  Leaves n_segs keys packed at
// *keys (segs_b; segs_a is free for the sort) with the digit histogram of the
// sort by bits [sort_lo, sort_hi) counted.  sparse: only changed layers'
// lines have steps (an incremental frame).
cgb_status build_and_rasterize(cgb_composition* c, int render, const BatchGeom& bg, int sort_lo, int sort_hi,
                               uint64_t* n_segs, uint64_t* n_total, uint64_t** keys, bool sparse = false) {
    cudaStream_t st = c->stream;
    if (bg.total_lines >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^32 lines in a frame");
    const uint32_t L = (uint32_t)bg.total_lines;
    c->stats.lines = L;
    CK(c->s.ensure(c->recs, std::max<size_t>(L, 1) * sizeof(LineRec)));
    CK(c->s.ensure(c->lengths, std::max<size_t>(L, 1) * 4));
    CK(c->s.ensure(c->step_off, ((size_t)L + 1) * 4));
    CK(stage_mark(c, 0, st, "cgb:build_lines"));
    CK(launch_build_lines(bg, render, c->recs.as<LineRec>(), c->lengths.as<uint32_t>(), st));
    uint64_t S = 0;
    CK(scan_u32(c->lengths.as<uint32_t>(), c->step_off.as<uint32_t>(), L, &c->s, st, &S));
    CK(stage_mark(c, 1, st, "cgb:rasterize"));
    if (S >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^32 pixel steps");
    c->stats.steps = S;
    const uint32_t block = c->tuning.raster_block;
    const uint32_t items = c->tuning.steps_per_block / block;
    const uint32_t grid = raster_grid(S, block, items);
    const uint32_t slots = raster_run_slots(block, items);
    CK(c->s.ensure(c->segs_a, std::max<size_t>((size_t)grid * slots, 1) * 8));
    CK(c->s.ensure(c->bcounts, ((size_t)grid + 1) * 4));
    CK(c->s.ensure(c->boff, ((size_t)grid + 1) * 4));
    CK(c->s.ensure(c->rlb, 8));
    CK(cudaMemsetAsync(c->rlb.p, 0, 8, st));
    unsigned long long* produced = c->rlb.as<unsigned long long>();
    CK(launch_rasterize(render, bg, c->recs.as<LineRec>(), c->step_off.as<uint32_t>(), L, S, block, items,
                        c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(), produced, st, nullptr, sparse));
    CK(cudaMemcpyAsync(&c->s.pinned[3], produced, 8, cudaMemcpyDeviceToHost, st));
    uint64_t P = 0;
    if (grid) CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid, &c->s, st, &P));
    const uint64_t PT = S ? c->s.pinned[3] : 0;
    if (P >= (1ull << 30) - 1) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^30 pixel segments");
    CK(c->s.ensure(c->segs_b, std::max<size_t>(P, 1) * 8));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), slots, c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid,
                         c->segs_b.as<uint64_t>(), sort_lo, sort_hi, (int)c->tuning.radix_bits, &c->s, st));
    CK(stage_mark(c, 2, st, "cgb:sort"));
    *n_segs = P;
    *n_total = PT;
    *keys = c->segs_b.as<uint64_t>();
    c->stats.segments = PT;
    return CGB_OK;
}

// cassia_render's segments (host memory) into packed keys of scene 0, with
// the sort's digit histogram counted, like build_and_rasterize.
cgb_status import_segments(cgb_composition* c, const BatchGeom& bg, int sort_lo, int sort_hi, uint64_t* n_segs,
                           uint64_t* n_total, uint64_t** keys) {
    cudaStream_t st = c->stream;
    const uint64_t n = c->import_n;
    if (n >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "cassia_render: more than 2^32 segments");
    c->stats.lines = 0;
    c->stats.steps = 0;
    CK(stage_mark(c, 0, st, "cgb:import"));
    CK(c->s.ensure(c->d_import, std::max<size_t>(n, 1) * 8));
    if (n) CK(cudaMemcpyAsync(c->d_import.p, c->import_segs, n * 8, cudaMemcpyHostToDevice, st));
    CK(stage_mark(c, 1, st, "cgb:import_keys"));
    const uint32_t grid = import_grid(n), slots = import_run_slots();
    CK(c->s.ensure(c->segs_a, std::max<size_t>((size_t)grid * slots, 1) * 8));
    CK(c->s.ensure(c->bcounts, ((size_t)grid + 1) * 4));
    CK(c->s.ensure(c->boff, ((size_t)grid + 1) * 4));
    CK(c->s.ensure(c->rlb, 8));
    CK(cudaMemsetAsync(c->rlb.p, 0, 8, st));
    unsigned long long* produced = c->rlb.as<unsigned long long>();
    CK(launch_import_segments(c->d_import.as<uint64_t>(), n, bg, c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(),
                              produced, st));
    CK(cudaMemcpyAsync(&c->s.pinned[3], produced, 8, cudaMemcpyDeviceToHost, st));
    uint64_t P = 0;
    if (grid) CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid, &c->s, st, &P));
    else CK(cudaStreamSynchronize(st));
    if (P >= (1ull << 30) - 1) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^30 pixel segments");
    CK(c->s.ensure(c->segs_b, std::max<size_t>(P, 1) * 8));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), slots, c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid,
                         c->segs_b.as<uint64_t>(), sort_lo, sort_hi, (int)c->tuning.radix_bits, &c->s, st));
    CK(stage_mark(c, 2, st, "cgb:sort"));
    *n_segs = P;
    *n_total = n ? c->s.pinned[3] : 0;
    *keys = c->segs_b.as<uint64_t>();
    c->stats.segments = *n_total;
    return CGB_OK;
}

cgb_status check_device_error(cgb_composition* c) {
    uint32_t v = 0;
    CK(cudaMemcpyAsync(&v, c->err.p, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (v) {
        CK(cudaMemsetAsync(c->err.p, 0, 4, c->stream));
        return fail(CGB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait expired");
    }
    return CGB_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        return 0.0f;
    }
    return ms;
}

// Incremental frames: which orders of composition c are rasterized again.
// The resident segments are usable when the canvas (tile rows and row
// length) is the one they were made for; the orders to redo are the old and
// new orders of every layer whose geometry changed since the last frame,
// and every order no present layer holds.
cgb_status prepare_incremental(cgb_composition* c, SceneInput& in) {
    in.incr = 0;
    in.d.rast_dirty = nullptr;
    if (!c->incremental || c->import_segs) return CGB_OK;
    const uint32_t rows = in.d.rows, row_len = in.d.row_len;
    if (rows > LOCAL_MAX_ROWS || row_len + 1 >= (1u << LOCAL_COL_BITS)) {  // beyond the local key layout
        c->resident_valid = false;
        return CGB_OK;
    }
    const bool valid = c->resident_valid && c->resident_rows == rows && c->resident_row_len == row_len;
    // from the device-table mirror (32 bytes per layer; touch() keeps it current)
    auto current_order = [&](uint32_t id) -> int32_t {
        if (id >= c->layer_recs.size()) return -1;
        const LayerRec& r = c->layer_recs[id];
        const bool live = (r.flags & LAYER_PRESENT) && (r.flags & LAYER_ENABLED);
        return live ? (int32_t)((r.flags & LAYER_HAS_ORDER) ? r.order : id) : -1;
    };
    if (!valid) {  // every line rasterized; the resident segments are rebuilt after the frame
        c->rast_order.assign(c->layers.size(), -1);
        for (uint32_t id = 0; id < c->layers.size(); id++) c->rast_order[id] = current_order(id);
        for (uint32_t id : c->rast_ids) c->rast_flag[id] = 0;
        c->rast_ids.clear();
        in.incr = 1;
        return CGB_OK;
    }
    c->h_rast_dirty.assign(c->max_ids, 0);
    for (uint32_t o = c->n_orders; o < c->max_ids; o++) c->h_rast_dirty[o] = 1;  // orders no layer holds
    if (c->rast_order.size() < c->layers.size()) c->rast_order.resize(c->layers.size(), -1);
    for (uint32_t id : c->rast_ids) {
        if (id < c->rast_order.size() && c->rast_order[id] >= 0) c->h_rast_dirty[(uint32_t)c->rast_order[id]] = 1;
        const int32_t cur = current_order(id);
        if (cur >= 0 && (uint32_t)cur < c->max_ids) c->h_rast_dirty[(uint32_t)cur] = 1;
        if (id >= c->rast_order.size()) c->rast_order.resize((size_t)id + 1, -1);
        c->rast_order[id] = cur;
        c->rast_flag[id] = 0;
    }
    c->rast_ids.clear();
    CK(c->s.ensure(c->d_rast_dirty, c->max_ids));
    // pinned source, rewritten only by the next frame (every render returns
    // after its frame is done)
    CK(cudaMemcpyAsync(c->d_rast_dirty.p, c->h_rast_dirty.data(), c->max_ids, cudaMemcpyHostToDevice, c->stream));
    in.d.rast_dirty = c->d_rast_dirty.as<uint8_t>();
    in.incr = 2;
    return CGB_OK;
}

// Host-side preparation of one composition for a frame: mold's
// remove_disabled, orders_to_layers / props, the layer table and the layer
// cache (composition.rs:212-241).
cgb_status prepare_scene(cgb_composition* c, SceneInput& in) {
    const cgb_buffer* buf = in.buf;
    if (!buf || !in.bg || !buf->pixels || buf->width == 0 || buf->height == 0)
        return fail(CGB_ERR_INVALID_ARG, "render: empty buffer");
    if (buf->flusher && buf->memory != CGB_MEMORY_HOST)
        return fail(CGB_ERR_INVALID_ARG, "render: a flusher needs a host buffer");
    const uint64_t stride = buf->width_stride ? buf->width_stride : buf->width;
    if (stride < buf->width || buf->width > (1u << 20) || buf->height > (1u << 20))
        return fail(CGB_ERR_INVALID_ARG, "render: bad width/stride/height");
    const uint32_t rows = (uint32_t)((buf->height + 7) / 8), row_len = (uint32_t)((buf->width + 7) / 8);
    const uint64_t n_tiles = (uint64_t)rows * row_len;
    in.cache = nullptr;
    if (buf->layer_cache >= 0) {
        auto it = c->caches.find(buf->layer_cache);
        if (it == c->caches.end()) return fail(CGB_ERR_NOT_FOUND, "render: unknown layer cache");
        in.cache = &it->second;
        if (in.cache->tiles != n_tiles) {  // composition.rs:218-225
            CK(c->s.ensure(in.cache->prev, n_tiles * 4));
            CK(cudaMemsetAsync(in.cache->prev.p, 0xFF, n_tiles * 4, c->stream));
            in.cache->tiles = n_tiles;
        }
    }
    if (!c->import_segs) {  // import mode: the props come from the stylings
        cgb_status s0 = remove_disabled(c);
        if (s0) return s0;
        if (c->props_dirty) rebuild_props(c);
    }
    cgb_status s1 = upload_layers(c);
    if (s1) return s1;
    if (c->props_uploaded != c->props_version) {
        CK(c->s.ensure(c->d_props, c->props_host.size() * sizeof(PaintProps)));
        CK(cudaMemcpyAsync(c->d_props.p, c->props_host.data(), c->props_host.size() * sizeof(PaintProps),
                           cudaMemcpyHostToDevice, c->stream));
        if (!c->grads_host.empty()) {
            CK(c->s.ensure(c->d_grads, c->grads_host.size() * sizeof(GradRec)));
            CK(c->s.ensure(c->d_stops, c->stops_host.size() * sizeof(GradStop)));
            CK(cudaMemcpyAsync(c->d_grads.p, c->grads_host.data(), c->grads_host.size() * sizeof(GradRec),
                               cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemcpyAsync(c->d_stops.p, c->stops_host.data(), c->stops_host.size() * sizeof(GradStop),
                               cudaMemcpyHostToDevice, c->stream));
        }
        c->props_uploaded = c->props_version;
    }
    if (in.cache) {
        std::vector<uint8_t> unchanged(c->n_orders, 0);
        for (uint32_t o = 0; o < c->n_orders; o++)
            if (c->order_layer[o] != UINT32_MAX)
                unchanged[o] = (c->layers[c->order_layer[o]].unchanged >> buf->layer_cache) & 1;
        CK(c->s.ensure(c->d_unchanged, unchanged.size()));
        CK(cudaMemcpyAsync(c->d_unchanged.p, unchanged.data(), unchanged.size(), cudaMemcpyHostToDevice, c->stream));
    }
    if (c->has_default_transform) {
        CK(c->s.ensure(c->dflt_t, 6 * 4));
        CK(cudaMemcpyAsync(c->dflt_t.p, c->default_transform, 24, cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    SceneDesc& d = in.d;
    d = SceneDesc{};
    d.p0x = c->p0x.as<float>();
    d.p0y = c->p0y.as<float>();
    d.p1x = c->p1x.as<float>();
    d.p1y = c->p1y.as<float>();
    d.lids = c->lids.as<uint32_t>();
    d.layers = c->d_layers.as<LayerRec>();
    d.props = c->d_props.as<PaintProps>();
    d.grads = c->grads_host.empty() ? nullptr : c->d_grads.as<GradRec>();
    d.stops = c->grads_host.empty() ? nullptr : c->d_stops.as<GradStop>();
    d.unchanged = in.cache ? c->d_unchanged.as<uint8_t>() : nullptr;
    d.prev_layers = in.cache ? in.cache->prev.as<int32_t>() : nullptr;
    d.default_t = c->has_default_transform ? c->dflt_t.as<float>() : nullptr;
    d.n_lines = (uint32_t)c->n_lines;
    d.n_layer_recs = c->n_layer_recs;
    d.n_orders = c->n_orders;
    d.wide = c->wide ? 1u : 0u;
    d.features = c->features;
    d.width = (uint32_t)buf->width;
    d.height = (uint32_t)buf->height;
    d.stride = (uint32_t)stride;
    d.rows = rows;
    d.row_len = row_len;
    d.crop_h0 = 0;
    d.crop_h1 = row_len;
    d.crop_v0 = 0;
    d.crop_v1 = rows;
    if (in.crop) {  // Rect::new (buffer_layout.rs:43-50)
        d.crop_h0 = (uint32_t)std::min<uint64_t>(in.crop->x0 / 8, row_len);
        d.crop_h1 = (uint32_t)std::min<uint64_t>((in.crop->x1 + 7) / 8, row_len);
        d.crop_v0 = (uint32_t)std::min<uint64_t>(in.crop->y0 / 8, rows);
        d.crop_v1 = (uint32_t)std::min<uint64_t>((in.crop->y1 + 7) / 8, rows);
    }
    std::memcpy(d.clear, in.bg, sizeof(d.clear));
    return prepare_incremental(c, in);
}

// Frame geometry shared by the staged and the graph form of a frame.
struct FrameSetup {
    BatchGeom bg{};
    uint64_t tiles = 0;
    uint32_t features = 0;
    bool flush = false;
    bool incremental = false;  // some scene is rendered incrementally (staged frames only)
};

// Incremental frames, after the sort of the new segments (*sorted, *P): the
// kept resident segments of the scenes rendered incrementally are merged
// in, then every incremental scene's range of the frame becomes its new
// resident segments (local key layout).
cgb_status incremental_merge(cgb_composition* c, const FrameSetup& f, std::vector<SceneInput>& scenes,
                             uint64_t** sorted, uint64_t* P) {
    cudaStream_t st = c->stream;
    const BatchGeom& bg = f.bg;
    // kept segments: resident segments of clean orders, scene after scene
    std::vector<KeepSource> src;
    uint64_t total = 0;
    for (const SceneInput& in : scenes) {
        if (in.incr != 2 || in.comp->resident_n == 0) continue;
        const cgb_composition* sc = in.comp;
        src.push_back(KeepSource{sc->resident.as<uint64_t>(), total, sc->resident_n, sc->d_rast_dirty.as<uint8_t>(),
                                 sc->max_ids, in.d.row_base, sc->resident_ob, sc->resident_cb});
        total += sc->resident_n;
    }
    if (src.size() > MAX_KEEP_SOURCES) return fail(CGB_ERR_INVALID_ARG, "incremental frame: too many scenes");
    uint64_t K = 0;
    if (total) {
        const uint32_t grid = keep_grid(total);
        CK(c->s.ensure(c->d_keep, src.size() * sizeof(KeepSource)));
        CK(cudaMemcpyAsync(c->d_keep.p, src.data(), src.size() * sizeof(KeepSource), cudaMemcpyHostToDevice, st));
        CK(c->s.ensure(c->bcounts, ((size_t)grid + 1) * 4));
        CK(c->s.ensure(c->boff, ((size_t)grid + 1) * 4));
        CK(launch_keep(0, c->d_keep.as<KeepSource>(), (uint32_t)src.size(), total, bg, c->bcounts.as<uint32_t>(),
                       nullptr, nullptr, 0, st));
        CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid, &c->s, st, &K));
        if (*P + K >= (1ull << 30) - 1) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^30 pixel segments");
        if (K) {
            CK(c->s.ensure(c->segs_k, K * 8));
            CK(launch_keep(1, c->d_keep.as<KeepSource>(), (uint32_t)src.size(), total, bg, nullptr,
                           c->boff.as<uint32_t>(), c->segs_k.as<uint64_t>(), K, st));
            CK(c->s.ensure(c->segs_m, (K + *P) * 8));
            CK(c->s.ensure(c->merge_split, ((size_t)merge_tiles(K + *P) + 1) * 4));
            CK(launch_merge(c->segs_k.as<uint64_t>(), (uint32_t)K, *sorted, (uint32_t)*P,
                            c->merge_split.as<uint32_t>(), c->segs_m.as<uint64_t>(), st));
            *sorted = c->segs_m.as<uint64_t>();
            *P += K;
        }
    }
    // A frame of one composition on its own handle: its sorted segments are
    // kept as they are, in this frame's key layout.
    if (scenes.size() == 1 && scenes[0].incr && scenes[0].comp == c) {
        if (*sorted == c->segs_m.as<uint64_t>()) {
            std::swap(c->resident, c->segs_m);
        } else {
            CK(c->s.ensure(c->resident, std::max<uint64_t>(*P, 1) * 8));
            if (*P) CK(cudaMemcpyAsync(c->resident.p, *sorted, *P * 8, cudaMemcpyDeviceToDevice, st));
        }
        c->resident_n = *P;
        c->resident_ob = bg.order_bits;
        c->resident_cb = bg.col_bits;
        c->resident_valid = true;
        c->resident_rows = scenes[0].d.rows;
        c->resident_row_len = scenes[0].d.row_len;
        return CGB_OK;
    }
    // the frame's segments of each incremental scene become its resident ones
    std::vector<uint32_t> ids;
    for (uint32_t k = 0; k < scenes.size(); k++)
        if (scenes[k].incr) ids.push_back(k);
    if (ids.size() > MAX_KEEP_SOURCES) return fail(CGB_ERR_INVALID_ARG, "incremental frame: too many scenes");
    CK(c->s.ensure(c->d_scene_ids, ids.size() * 4));
    CK(c->s.ensure(c->d_ranges, ids.size() * 8));
    CK(cudaMemcpyAsync(c->d_scene_ids.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, st));
    CK(launch_scene_ranges(*sorted, (uint32_t)*P, bg, c->d_scene_ids.as<uint32_t>(), (uint32_t)ids.size(),
                           c->d_ranges.as<uint32_t>(), st));
    std::vector<uint32_t> ranges(2 * ids.size());
    CK(cudaMemcpyAsync(ranges.data(), c->d_ranges.p, ranges.size() * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<ExtractTarget> tg;
    uint64_t n_all = 0;
    for (size_t q = 0; q < ids.size(); q++) {
        SceneInput& in = scenes[ids[q]];
        cgb_composition* sc = in.comp;
        const uint64_t n = ranges[2 * q + 1] >= ranges[2 * q] ? ranges[2 * q + 1] - ranges[2 * q] : 0;
        cudaError_t e = sc->s.ensure(sc->resident, std::max<uint64_t>(n, 1) * 8);
        if (e != cudaSuccess) {  // no room to keep them: the next frame rasterizes every line
            cudaGetLastError();
            sc->s.over_budget = false;
            sc->resident_valid = false;
            sc->resident_n = 0;
            continue;
        }
        tg.push_back(ExtractTarget{sc->resident.as<uint64_t>(), n_all, n, sc->resident.cap / 8, ranges[2 * q],
                                   in.d.row_base});
        n_all += n;
        sc->resident_n = n;
        sc->resident_ob = LOCAL_ORDER_BITS;
        sc->resident_cb = LOCAL_COL_BITS;
        sc->resident_valid = true;
        sc->resident_rows = in.d.rows;
        sc->resident_row_len = in.d.row_len;
    }
    if (!tg.empty()) {
        CK(c->s.ensure(c->d_extract, tg.size() * sizeof(ExtractTarget)));
        CK(cudaMemcpyAsync(c->d_extract.p, tg.data(), tg.size() * sizeof(ExtractTarget), cudaMemcpyHostToDevice, st));
        CK(launch_extract(*sorted, c->d_extract.as<ExtractTarget>(), (uint32_t)tg.size(), n_all, bg, st));
        CK(cudaStreamSynchronize(st));  // the host vectors above go out of scope
    }
    return CGB_OK;
}

// Build -> rasterize -> sort -> carries / items -> paint, stage by stage:
// the host reads S, P, G and W as they are produced and sizes each buffer
// to them.
cgb_status staged_frame(cgb_composition* c, const FrameSetup& f, std::vector<SceneInput>& scenes) {
    cudaStream_t st = c->stream;
    const BatchGeom& bg = f.bg;
    const uint64_t tiles = f.tiles;
    uint64_t P = 0, PT = 0;
    uint64_t* keys = nullptr;
    bool sparse = false;  // some scene rasterizes only its changed layers
    for (const SceneInput& in : scenes) sparse |= in.incr == 2;
    cgb_status s2 = c->import_segs ? import_segments(c, bg, 22, 22 + (int)bg.key_bits, &P, &PT, &keys)
                                   : build_and_rasterize(c, 1, bg, 22, 22 + (int)bg.key_bits, &P, &PT, &keys, sparse);
    if (s2) return s2;
    c->stats.painted_segments = P;
    // sort by (global row, order, tile column)
    uint64_t* sorted = keys;
    int passes = 0;
    CK(radix_sort_u64(keys, c->segs_a.as<uint64_t>(), (uint32_t)P, 22, 22 + (int)bg.key_bits,
                      (int)c->tuning.radix_bits, &c->s, c->err.as<uint32_t>(), st, &sorted, &passes, true));
    c->stats.sort_passes = passes;
    c->last_new_segs = P;
    if (f.incremental) {
        cgb_status si = incremental_merge(c, f, scenes, &sorted, &P);
        if (si) return si;
        c->stats.painted_segments = P;
    }
    CK(stage_mark(c, 3, st, "cgb:carry"));

    // tile-layer groups, carries, work items
    CarryBuffers cb{};
    const uint32_t hg = tl_scan_grid((uint32_t)P);
    CK(c->s.ensure(c->bcounts, ((size_t)hg + 1) * 4));
    CK(c->s.ensure(c->boff, ((size_t)hg + 1) * 4));
    CK(c->s.ensure(c->blk_cover, ((size_t)hg + 1) * 8));
    CK(c->s.ensure(c->blk_head, ((size_t)hg + 1) * 4));
    cb.blk_cover = c->blk_cover.as<uint64_t>();
    cb.blk_head = c->blk_head.as<uint32_t>();
    CK(launch_tl_scan(0, sorted, (uint32_t)P, bg.col_bits, c->bcounts.as<uint32_t>(), nullptr, cb, st));
    uint64_t G = 0;
    if (P) CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), hg, &c->s, st, &G));
    c->stats.tile_layers = G;
    CK(c->s.ensure(c->tl_start, (G + 1) * 4));
    CK(c->s.ensure(c->tl_key, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_cover, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_carry, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_flags, std::max<uint64_t>(G, 1) * 4));
    CK(c->s.ensure(c->item_count, std::max<uint64_t>(G, 1) * 4));
    CK(c->s.ensure(c->item_off, (G + 1) * 4));
    cb.tl_start = c->tl_start.as<uint32_t>();
    cb.tl_key = c->tl_key.as<uint64_t>();
    cb.tl_cover = c->tl_cover.as<uint64_t>();
    cb.tl_carry = c->tl_carry.as<uint64_t>();
    cb.tl_flags = c->tl_flags.as<uint32_t>();
    cb.item_count = c->item_count.as<uint32_t>();
    cb.item_off = c->item_off.as<uint32_t>();
    cb.order_bits = (int)bg.order_bits;
    CK(launch_tl_scan(1, sorted, (uint32_t)P, bg.col_bits, nullptr, c->boff.as<uint32_t>(), cb, st));
    CK(launch_tl_carry((uint32_t)G, (uint32_t)P, cb, st));
    CK(launch_items(0, (uint32_t)G, bg, cb, 0, st));
    uint64_t W = 0;
    if (G) CK(scan_u32(cb.item_count, cb.item_off, (uint32_t)G, &c->s, st, &W));
    c->stats.work_items = W;
    const int idx_bits = bits_for(std::max<uint64_t>(G, 1) - 1);
    const int tile_bits = bits_for(std::max<uint64_t>(tiles, 1) - 1);
    const int tile_shift = idx_bits + 3 + cb.order_bits;  // TL index, item flags, order, then the tile
    if (tile_shift + tile_bits > 64 || W >= (1ull << 30))
        return fail(CGB_ERR_LAYER_LIMIT, "render: too many tile x layer work items");
    CK(c->s.ensure(c->items_a, std::max<uint64_t>(W, 1) * 8));
    CK(c->s.ensure(c->items_b, std::max<uint64_t>(W, 1) * 8));
    CK(c->s.ensure(c->tile_start, (tiles + 1) * 4));
    cb.items = c->items_a.as<uint64_t>();
    cb.items_tmp = c->items_b.as<uint64_t>();
    cb.tile_start = c->tile_start.as<uint32_t>();
    CK(launch_items(1, (uint32_t)G, bg, cb, idx_bits, st));
    uint64_t* items_sorted = cb.items;
    int ipasses = 0;
    // stable sort on the tile field: each tile's items stay in order
    CK(radix_sort_u64(cb.items, cb.items_tmp, (uint32_t)W, tile_shift, tile_shift + tile_bits,
                      (int)c->tuning.radix_bits, &c->s, c->err.as<uint32_t>(), st, &items_sorted, &ipasses));
    c->stats.item_sort_passes = ipasses;
    CK(launch_tile_ranges(items_sorted, (uint32_t)W, (uint32_t)tiles, tile_shift, cb.tile_start, st));
    CK(stage_mark(c, 4, st, "cgb:paint"));
    uint8_t* item_state = nullptr;
    if (f.features & FEAT_CLIPS) {
        CK(c->s.ensure(c->item_state, std::max<uint64_t>(W, 1)));
        item_state = c->item_state.as<uint8_t>();
    }
    if (f.flush) CK(cudaMemsetAsync(c->written.p, 0, tiles, st));
    CK(launch_paint(bg, sorted, items_sorted, idx_bits, (uint32_t)G, cb.tile_start, cb, c->tuning.paint_warps,
                    f.features != 0, item_state, st));
    CK(stage_mark(c, 5, st, nullptr));
    return CGB_OK;
}

uint32_t with_headroom(uint64_t n, float headroom) {
    const uint64_t v = n + (uint64_t)((double)n * headroom) + 4096;
    return (uint32_t)std::min<uint64_t>(v, (1ull << 30) - 2);
}

// The frame-graph signature: what a captured frame bakes into its launches
// besides buffer pointers (those are compared separately).  Scene
// descriptors, layer tables, props and output pointers are read by the
// kernels from device memory, so they may change between replays.
std::string frame_signature(const cgb_composition* c, const FrameSetup& f) {
    const BatchGeom& bg = f.bg;
    const uint64_t v[] = {bg.n_scenes,        bg.total_rows,   bg.total_tiles,           bg.n_orders,
                          bg.row_len,         bg.order_bits,   bg.col_bits,              bg.key_bits,
                          bg.total_lines,     c->tuning.radix_bits, c->tuning.raster_block, c->tuning.steps_per_block,
                          c->tuning.paint_warps, f.features,   f.flush ? 1u : 0u};
    return std::string(reinterpret_cast<const char*>(v), sizeof(v));
}

// (pointer, size) of every buffer that a frame graph launches on.
std::vector<std::pair<const void*, size_t>> graph_buffers(cgb_composition* c) {
    const DevBuf* b[] = {&c->recs,       &c->lengths,   &c->step_off,  &c->bcounts,         &c->boff,
                         &c->segs_a,     &c->segs_b,    &c->blk_cover, &c->blk_head,        &c->tl_start,
                         &c->tl_key,     &c->tl_cover,  &c->tl_carry,  &c->tl_flags,        &c->item_count,
                         &c->item_off,   &c->items_a,   &c->items_b,   &c->tile_start,      &c->item_state,
                         &c->written,    &c->d_scenes,  &c->d_row_scene, &c->err,           &c->d_counts,
                         &c->s.scan_sums, &c->s.sort_hist, &c->s.sort_lookback, &c->s.sort_counter};
    std::vector<std::pair<const void*, size_t>> r;
    for (const DevBuf* x : b) r.emplace_back(x->p, x->cap);
    return r;
}

// Every buffer of a graph frame at its capacity (nothing may allocate while
// the stream captures).
cudaError_t ensure_graph_buffers(cgb_composition* c, const FrameSetup& f, const FrameCaps& k) {
    Scratch& s = c->s;
    const uint64_t L = f.bg.total_lines;
    const uint32_t block = c->tuning.raster_block, items = c->tuning.steps_per_block / block;
    const uint64_t grid = raster_grid(k.steps, block, items), slots = raster_run_slots(block, items);
    const uint64_t hg = tl_scan_grid(k.segs);
    cudaError_t e = cudaSuccess;
    auto need = [&](DevBuf& b, uint64_t bytes) {
        if (e == cudaSuccess) e = s.ensure(b, std::max<uint64_t>(bytes, 8));
    };
    need(c->recs, L * sizeof(LineRec));
    need(c->lengths, L * 4);
    need(c->step_off, (L + 1) * 4);
    need(c->segs_a, std::max<uint64_t>(grid * slots, k.segs) * 8);
    need(c->segs_b, (uint64_t)k.segs * 8);
    need(c->bcounts, (std::max(grid, hg) + 1) * 4);
    need(c->boff, (std::max(grid, hg) + 1) * 4);
    need(c->blk_cover, (hg + 1) * 8);
    need(c->blk_head, (hg + 1) * 4);
    need(c->tl_start, ((uint64_t)k.tls + 1) * 4);
    need(c->tl_key, (uint64_t)k.tls * 8);
    need(c->tl_cover, (uint64_t)k.tls * 8);
    need(c->tl_carry, (uint64_t)k.tls * 8);
    need(c->tl_flags, (uint64_t)k.tls * 4);
    need(c->item_count, (uint64_t)k.tls * 4);
    need(c->item_off, ((uint64_t)k.tls + 1) * 4);
    need(c->items_a, (uint64_t)k.items * 8);
    need(c->items_b, (uint64_t)k.items * 8);
    need(c->tile_start, (f.tiles + 1) * 4);
    if (f.features & FEAT_CLIPS) need(c->item_state, k.items);
    need(c->d_counts, sizeof(FrameCounts));
    if (e == cudaSuccess) {
        const uint64_t scan_n = std::max<uint64_t>(std::max<uint64_t>(L, grid), std::max<uint64_t>(hg, k.tls));
        e = reserve_frame_scratch(&s, (uint32_t)std::min<uint64_t>(scan_n, UINT32_MAX), std::max(k.segs, k.items));
    }
    return e;
}

cgb_status enqueue_counted_tail(cgb_composition* c, const FrameSetup& f, const FrameCaps& k, uint64_t* sorted,
                                FrameGraph* g);

// The body of a frame graph: the staged frame's launches with the counts
// kept on the device (no host synchronization) and every grid sized for
// the capacities.
cgb_status enqueue_counted_frame(cgb_composition* c, const FrameSetup& f, const FrameCaps& k, FrameGraph* g) {
    cudaStream_t st = c->stream;
    const BatchGeom& bg = f.bg;
    FrameCounts* fc = c->d_counts.as<FrameCounts>();
    uint32_t* err = c->err.as<uint32_t>();
    const uint32_t L = (uint32_t)bg.total_lines;
    const uint32_t block = c->tuning.raster_block, items = c->tuning.steps_per_block / block;
    const uint32_t grid = raster_grid(k.steps, block, items), slots = raster_run_slots(block, items);
    const int rbits = (int)c->tuning.radix_bits;
    CK(cudaMemsetAsync(fc, 0, sizeof(FrameCounts), st));
    CK(stage_mark(c, 0, st, nullptr));
    CK(launch_build_lines(bg, 1, c->recs.as<LineRec>(), c->lengths.as<uint32_t>(), st));
    CK(scan_u32(c->lengths.as<uint32_t>(), c->step_off.as<uint32_t>(), L, &c->s, st, nullptr, &fc->n[FC_STEPS]));
    CK(stage_mark(c, 1, st, nullptr));
    CK(launch_rasterize(1, bg, c->recs.as<LineRec>(), c->step_off.as<uint32_t>(), L, k.steps, block, items,
                        c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(), &fc->produced, st, fc));
    CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid, &c->s, st, nullptr, &fc->n[FC_SEGS]));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), slots, c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid,
                         c->segs_b.as<uint64_t>(), 22, 22 + (int)bg.key_bits, rbits, &c->s, st, k.segs));
    CK(stage_mark(c, 2, st, nullptr));
    uint64_t* sorted = nullptr;
    int passes = 0;
    CK(radix_sort_u64(c->segs_b.as<uint64_t>(), c->segs_a.as<uint64_t>(), k.segs, 22, 22 + (int)bg.key_bits, rbits,
                      &c->s, err, st, &sorted, &passes, true, fc, FC_SEGS));
    g->sort_passes = (uint32_t)passes;
    CK(stage_mark(c, 3, st, nullptr));
    return enqueue_counted_tail(c, f, k, sorted, g);
}

// The device-counted stages after the sort: tile-layer groups, carries,
// work items and their sort, the painter and the counts readback.  `sorted`
// holds the frame's sorted segments, at most k.segs of them
// (fc->n[FC_SEGS]).
cgb_status enqueue_counted_tail(cgb_composition* c, const FrameSetup& f, const FrameCaps& k, uint64_t* sorted,
                                FrameGraph* g) {
    cudaStream_t st = c->stream;
    const BatchGeom& bg = f.bg;
    FrameCounts* fc = c->d_counts.as<FrameCounts>();
    uint32_t* err = c->err.as<uint32_t>();
    const int rbits = (int)c->tuning.radix_bits;
    CarryBuffers cb{};
    const uint32_t hg = tl_scan_grid(k.segs);
    cb.blk_cover = c->blk_cover.as<uint64_t>();
    cb.blk_head = c->blk_head.as<uint32_t>();
    cb.tl_start = c->tl_start.as<uint32_t>();
    cb.tl_key = c->tl_key.as<uint64_t>();
    cb.tl_cover = c->tl_cover.as<uint64_t>();
    cb.tl_carry = c->tl_carry.as<uint64_t>();
    cb.tl_flags = c->tl_flags.as<uint32_t>();
    cb.item_count = c->item_count.as<uint32_t>();
    cb.item_off = c->item_off.as<uint32_t>();
    cb.items = c->items_a.as<uint64_t>();
    cb.items_tmp = c->items_b.as<uint64_t>();
    cb.tile_start = c->tile_start.as<uint32_t>();
    cb.order_bits = (int)bg.order_bits;
    cb.fc = fc;
    cb.tl_cap = k.tls;
    cb.items_cap = k.items;
    CK(launch_tl_scan(0, sorted, k.segs, bg.col_bits, c->bcounts.as<uint32_t>(), nullptr, cb, st));
    CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), hg, &c->s, st, nullptr, &fc->n[FC_TLS]));
    CK(launch_tl_scan(1, sorted, k.segs, bg.col_bits, nullptr, c->boff.as<uint32_t>(), cb, st));
    CK(launch_tl_carry(k.tls, k.segs, cb, st));
    CK(launch_items(0, k.tls, bg, cb, 0, st));
    CK(scan_u32(cb.item_count, cb.item_off, k.tls, &c->s, st, nullptr, &fc->n[FC_ITEMS]));
    const int idx_bits = bits_for((uint64_t)k.tls - 1);
    const int tile_bits = bits_for(std::max<uint64_t>(f.tiles, 1) - 1);
    const int tile_shift = idx_bits + 3 + cb.order_bits;
    if (tile_shift + tile_bits > 64) return fail(CGB_ERR_LAYER_LIMIT, "render: frame graph item key too wide");
    CK(launch_items(1, k.tls, bg, cb, idx_bits, st));
    uint64_t* items_sorted = nullptr;
    int ipasses = 0;
    CK(radix_sort_u64(cb.items, cb.items_tmp, k.items, tile_shift, tile_shift + tile_bits, rbits, &c->s, err, st,
                      &items_sorted, &ipasses, false, fc, FC_ITEMS));
    g->item_sort_passes = (uint32_t)ipasses;
    CK(launch_tile_ranges(items_sorted, k.items, (uint32_t)f.tiles, tile_shift, cb.tile_start, st, fc));
    CK(stage_mark(c, 4, st, nullptr));
    uint8_t* item_state = (f.features & FEAT_CLIPS) ? c->item_state.as<uint8_t>() : nullptr;
    if (f.flush) CK(cudaMemsetAsync(c->written.p, 0, f.tiles, st));
    CK(launch_paint(bg, sorted, items_sorted, idx_bits, k.tls, cb.tile_start, cb, c->tuning.paint_warps,
                    f.features != 0, item_state, st));
    CK(stage_mark(c, 5, st, nullptr));
    CK(cudaMemcpyAsync(c->h_counts, fc, sizeof(FrameCounts), cudaMemcpyDeviceToHost, st));
    return CGB_OK;
}

void destroy_graph(FrameGraph& g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
}

// Captures the frame graph of `f` with capacities from the counts of the
// frame just rendered.  A frame that cannot be captured (memory budget, an
// item key too wide) is simply rendered stage by stage next time.
void capture_frame_graph(cgb_composition* c, const FrameSetup& f, const std::string& sig) {
    FrameCaps k;
    k.steps = with_headroom(c->stats.steps, c->graph_headroom);
    k.segs = with_headroom(c->stats.painted_segments, c->graph_headroom);
    k.tls = with_headroom(c->stats.tile_layers, c->graph_headroom);
    k.items = with_headroom(c->stats.work_items, c->graph_headroom);
    if (!c->h_counts && cudaMallocHost(&c->h_counts, sizeof(FrameCounts)) != cudaSuccess) {
        cudaGetLastError();
        c->h_counts = nullptr;
        return;
    }
    if (ensure_graph_buffers(c, f, k) != cudaSuccess) {
        cudaGetLastError();
        c->s.over_budget = false;
        return;
    }
    FrameGraph g;
    g.caps = k;
    const uint64_t l0 = g_launches.load();
    cudaStream_t st = c->stream;
    c->capturing = true;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    cgb_status s1 = e == cudaSuccess ? enqueue_counted_frame(c, f, k, &g) : CGB_ERR_DEVICE;
    cudaGraph_t graph = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(st, &graph);
    c->capturing = false;
    g.launches = g_launches.load() - l0;
    g_launches.fetch_sub(g.launches);  // captured, not launched: counted at each replay
    if (s1 == CGB_OK && e == cudaSuccess && graph) e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (s1 != CGB_OK || e != cudaSuccess || !g.exec) {
        cudaGetLastError();
        destroy_graph(g);
        return;
    }
    g.bufs = graph_buffers(c);
    auto it = c->graphs.find(sig);
    if (it != c->graphs.end()) {
        destroy_graph(it->second);
        c->graphs.erase(it);
    }
    constexpr size_t MAX_GRAPHS = 32;  // frame geometries kept per handle
    if (c->graphs.size() >= MAX_GRAPHS) {
        destroy_graph(c->graphs.begin()->second);
        c->graphs.erase(c->graphs.begin());
    }
    c->graphs.emplace(sig, std::move(g));
}

// After the device frame: RGBA8 back into host buffers, the written-tile
// flags, the error flag and the stage times.
cgb_status finish_frame(cgb_composition* c, std::vector<SceneInput>& scenes, const FrameSetup& f,
                        std::vector<uint8_t>& written) {
    cudaStream_t st = c->stream;
    for (SceneInput& in : scenes)
        if (in.buf->memory == CGB_MEMORY_HOST)
            CK(cudaMemcpy2DAsync(in.buf->pixels, (size_t)in.d.stride * 4, in.d.out, (size_t)in.d.stride * 4,
                                 (size_t)in.d.width * 4, in.d.height, cudaMemcpyDeviceToHost, st));
    if (f.flush) {
        written.resize(f.tiles);
        CK(cudaMemcpyAsync(written.data(), c->written.p, f.tiles, cudaMemcpyDeviceToHost, st));
    }
    cgb_status s3 = check_device_error(c);
    if (s3) return s3;
    c->stats.build_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.rasterize_ms = elapsed(c->ev[1], c->ev[2]);
    c->stats.sort_ms = elapsed(c->ev[2], c->ev[3]);
    c->stats.carry_ms = elapsed(c->ev[3], c->ev[4]);
    c->stats.paint_ms = elapsed(c->ev[4], c->ev[5]);
    c->stats.total_ms = elapsed(c->ev[0], c->ev[5]);
    return CGB_OK;
}

// The host side of a finished frame: the flushers and the layer caches.
void post_frame(std::vector<SceneInput>& scenes, const std::vector<uint8_t>& written) {
    // Painter::write_to_tile's flush (painter/mod.rs:483-492): each written
    // tile's row slices, cut to the tile width
    for (const SceneInput& in : scenes) {
        if (!in.buf->flusher) continue;
        const SceneDesc& d = in.d;
        for (uint32_t j = 0; j < d.rows; j++)
            for (uint32_t i = 0; i < d.row_len; i++) {
                if (!written[d.tile_base + (uint64_t)j * d.row_len + i]) continue;
                const uint32_t x = i * 8, w = std::min<uint32_t>(8, d.width - x);
                for (uint32_t y = j * 8; y < std::min<uint32_t>(j * 8 + 8, d.height); y++)
                    in.buf->flusher(in.buf->flusher_user, in.buf->pixels + ((size_t)y * d.stride + x) * 4, w);
            }
    }
    for (SceneInput& in : scenes)
        if (in.cache)  // composition.rs:322-327
            for (HostLayer& l : in.comp->layers) {
                if (!l.present) continue;
                if (l.enabled) l.unchanged |= 1u << in.buf->layer_cache;
                else l.unchanged &= ~(1u << in.buf->layer_cache);
            }
}

// Capacities of the next sync-free incremental frame: the largest counts of
// the incremental frames so far, with headroom.
void note_incremental_counts(cgb_composition* c, uint64_t steps, uint64_t new_segs, uint64_t tls, uint64_t items) {
    FrameCaps& k = c->incr_caps;
    const float h = c->graph_headroom;
    k.steps = std::max(k.steps, with_headroom(steps, h));
    k.segs = std::max(k.segs, with_headroom(new_segs, h));
    k.tls = std::max(k.tls, with_headroom(tls, h));
    k.items = std::max(k.items, with_headroom(items, h));
    c->incr_caps_valid = true;
}

// An incremental frame of composition c on its own handle without host
// synchronization between stages: the changed layers' lines are rasterized
// and sorted, the resident segments of clean orders kept and merged in, and
// the device-counted stages of a frame graph finish it; every count stays on
// the device, grids are sized by the capacities of the earlier incremental
// frames.  *done is false when a count passed its capacity (nothing was
// painted; the caller renders the frame stage by stage).
cgb_status sync_free_incremental(cgb_composition* c, const FrameSetup& f, std::vector<SceneInput>& scenes,
                                 std::vector<uint8_t>& written, bool* done) {
    *done = false;
    const FrameCaps& ic = c->incr_caps;
    const uint64_t K = c->resident_n;
    if (K + ic.segs >= (1ull << 30) - 1) return CGB_OK;
    cudaStream_t st = c->stream;
    const BatchGeom& bg = f.bg;
    FrameCaps k;
    k.steps = ic.steps;
    k.segs = (uint32_t)(K + ic.segs);  // the merged frame
    k.tls = ic.tls;
    k.items = ic.items;
    const uint32_t L = (uint32_t)bg.total_lines;
    const uint32_t block = c->tuning.raster_block, items = c->tuning.steps_per_block / block;
    const uint64_t grid = raster_grid(k.steps, block, items), slots = raster_run_slots(block, items);
    const uint64_t hg = tl_scan_grid(k.segs), kg = keep_grid(std::max<uint64_t>(K, 1));
    const uint64_t nb = std::max(std::max(grid, hg), kg) + 1;
    if (!c->h_counts && cudaMallocHost(&c->h_counts, sizeof(FrameCounts)) != cudaSuccess) {
        cudaGetLastError();
        c->h_counts = nullptr;
        return CGB_OK;
    }
    Scratch& sc = c->s;
    CK(sc.ensure(c->recs, std::max<uint64_t>(L, 1) * sizeof(LineRec)));
    CK(sc.ensure(c->lengths, std::max<uint64_t>(L, 1) * 4));
    CK(sc.ensure(c->step_off, ((uint64_t)L + 1) * 4));
    CK(sc.ensure(c->segs_a, std::max<uint64_t>(grid * slots, ic.segs) * 8));
    CK(sc.ensure(c->segs_b, (uint64_t)ic.segs * 8));
    CK(sc.ensure(c->bcounts, nb * 4));
    CK(sc.ensure(c->boff, nb * 4));
    CK(sc.ensure(c->blk_cover, (hg + 1) * 8));
    CK(sc.ensure(c->blk_head, (hg + 1) * 4));
    CK(sc.ensure(c->segs_k, std::max<uint64_t>(K, 1) * 8));
    CK(sc.ensure(c->segs_m, (uint64_t)k.segs * 8));
    CK(sc.ensure(c->merge_split, ((uint64_t)merge_tiles(k.segs) + 1) * 4));
    CK(sc.ensure(c->tl_start, ((uint64_t)k.tls + 1) * 4));
    CK(sc.ensure(c->tl_key, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->tl_cover, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->tl_carry, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->tl_flags, (uint64_t)k.tls * 4));
    CK(sc.ensure(c->item_count, (uint64_t)k.tls * 4));
    CK(sc.ensure(c->item_off, ((uint64_t)k.tls + 1) * 4));
    CK(sc.ensure(c->items_a, (uint64_t)k.items * 8));
    CK(sc.ensure(c->items_b, (uint64_t)k.items * 8));
    CK(sc.ensure(c->tile_start, (f.tiles + 1) * 4));
    if (f.features & FEAT_CLIPS) CK(sc.ensure(c->item_state, k.items));
    CK(sc.ensure(c->d_counts, sizeof(FrameCounts)));
    CK(sc.ensure(c->d_keep, sizeof(KeepSource)));
    const uint64_t scan_n = std::max(std::max<uint64_t>(L, grid), std::max<uint64_t>(std::max(hg, kg), k.tls));
    CK(reserve_frame_scratch(&sc, (uint32_t)std::min<uint64_t>(scan_n, UINT32_MAX), std::max(ic.segs, k.items)));

    FrameCounts* fc = c->d_counts.as<FrameCounts>();
    uint32_t* err = c->err.as<uint32_t>();
    const int rbits = (int)c->tuning.radix_bits;
    const KeepSource src{c->resident.as<uint64_t>(), 0, K, c->d_rast_dirty.as<uint8_t>(), c->max_ids, 0,
                         c->resident_ob, c->resident_cb};
    CK(cudaMemsetAsync(fc, 0, sizeof(FrameCounts), st));
    CK(cudaMemcpyAsync(c->d_keep.p, &src, sizeof(src), cudaMemcpyHostToDevice, st));
    CK(stage_mark(c, 0, st, "cgb:build_lines"));
    CK(launch_build_lines(bg, 1, c->recs.as<LineRec>(), c->lengths.as<uint32_t>(), st));
    CK(scan_u32(c->lengths.as<uint32_t>(), c->step_off.as<uint32_t>(), L, &sc, st, nullptr, &fc->n[FC_STEPS]));
    CK(stage_mark(c, 1, st, "cgb:rasterize"));
    CK(launch_rasterize(1, bg, c->recs.as<LineRec>(), c->step_off.as<uint32_t>(), L, k.steps, block, items,
                        c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(), &fc->produced, st, fc, true));
    CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), (uint32_t)grid, &sc, st, nullptr,
                &fc->n[FC_NEW]));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), (uint32_t)slots, c->bcounts.as<uint32_t>(),
                         c->boff.as<uint32_t>(), (uint32_t)grid, c->segs_b.as<uint64_t>(), 22, 22 + (int)bg.key_bits,
                         rbits, &sc, st, ic.segs));
    CK(stage_mark(c, 2, st, "cgb:sort"));
    uint64_t* sorted_new = nullptr;
    int passes = 0;
    CK(radix_sort_u64(c->segs_b.as<uint64_t>(), c->segs_a.as<uint64_t>(), ic.segs, 22, 22 + (int)bg.key_bits, rbits,
                      &sc, err, st, &sorted_new, &passes, true, fc, FC_NEW));
    if (K) {
        CK(launch_keep(0, c->d_keep.as<KeepSource>(), 1, K, bg, c->bcounts.as<uint32_t>(), nullptr, nullptr, 0, st));
        CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), (uint32_t)kg, &sc, st, nullptr,
                    &fc->n[FC_KEPT]));
        CK(launch_keep(1, c->d_keep.as<KeepSource>(), 1, K, bg, nullptr, c->boff.as<uint32_t>(),
                       c->segs_k.as<uint64_t>(), K, st));
    }
    CK(launch_merge(c->segs_k.as<uint64_t>(), (uint32_t)K, sorted_new, ic.segs, c->merge_split.as<uint32_t>(),
                    c->segs_m.as<uint64_t>(), st, fc));
    CK(stage_mark(c, 3, st, "cgb:carry"));
    FrameGraph g;
    cgb_status s1 = enqueue_counted_tail(c, f, k, c->segs_m.as<uint64_t>(), &g);
    if (s1) return s1;
    cgb_status s3 = finish_frame(c, scenes, f, written);
    if (s3) return s3;
    const FrameCounts& h = *c->h_counts;
    if (h.overflow) return CGB_OK;
    // the merged frame is the resident segments of the next one
    std::swap(c->resident, c->segs_m);
    c->resident_n = h.n[FC_SEGS];
    c->resident_ob = bg.order_bits;
    c->resident_cb = bg.col_bits;
    c->resident_valid = true;
    c->resident_rows = scenes[0].d.rows;
    c->resident_row_len = scenes[0].d.row_len;
    c->stats.lines = bg.total_lines;
    c->stats.steps = h.n[FC_STEPS];
    c->stats.segments = h.produced;
    c->stats.painted_segments = h.n[FC_SEGS];
    c->stats.tile_layers = h.n[FC_TLS];
    c->stats.work_items = h.n[FC_ITEMS];
    c->stats.sort_passes = (uint32_t)passes;
    c->stats.item_sort_passes = g.item_sort_passes;
    note_incremental_counts(c, h.n[FC_STEPS], h.n[FC_NEW], h.n[FC_TLS], h.n[FC_ITEMS]);
    *done = true;
    return CGB_OK;
}

// Renders every scene of `scenes` in one pipeline on `c`'s stream and
// buffers: build, rasterize, sort, carries / items, paint.  In graph mode a
// frame whose signature and buffers match a captured one is replayed from
// its graph; a replay whose counts passed the graph's capacities paints
// nothing and the frame is rendered again stage by stage.
cgb_status render_frame(cgb_composition* c, std::vector<SceneInput>& scenes) {
    cudaStream_t st = c->stream;
    for (SceneInput& in : scenes) {
        cgb_status s0 = prepare_scene(in.comp, in);
        if (s0) return s0;
    }
    // frame geometry: global rows / tiles, key factors, host-output staging
    uint64_t lines = 0, rows = 0, tiles = 0, staging = 0;
    uint32_t n_orders = 1, row_len = 1;
    FrameSetup f;
    for (SceneInput& in : scenes) {
        in.d.line_base = lines;
        in.d.row_base = (uint32_t)rows;
        in.d.tile_base = (uint32_t)tiles;
        lines += in.d.n_lines;
        rows += in.d.rows;
        tiles += (uint64_t)in.d.rows * in.d.row_len;
        n_orders = std::max(n_orders, in.d.n_orders);
        row_len = std::max(row_len, in.d.row_len);
        in.staging_off = staging;
        if (in.buf->memory == CGB_MEMORY_HOST) staging += ((size_t)in.d.height * in.d.stride * 4 + 255) & ~(size_t)255;
        f.features |= in.d.features;
        f.flush |= in.buf->flusher != nullptr;
        f.incremental |= in.incr != 0;
    }
    if (tiles >= (1ull << 31)) return fail(CGB_ERR_LAYER_LIMIT, "render: too many tiles in a frame");
    BatchGeom& bg = f.bg;
    f.tiles = tiles;
    bg.n_scenes = (uint32_t)scenes.size();
    bg.total_rows = (uint32_t)rows;
    bg.total_tiles = (uint32_t)tiles;
    bg.n_orders = n_orders;
    bg.row_len = row_len;
    bg.total_lines = lines;
    bg.order_bits = bits_for(std::max<uint32_t>(n_orders, 1) - 1);
    bg.col_bits = bits_for(row_len);
    bg.key_bits = bits_for(std::max<uint64_t>(rows, 1) - 1) + bg.order_bits + bg.col_bits;
    if (bg.key_bits > 42) return fail(CGB_ERR_LAYER_LIMIT, "render: rows x orders x tiles too large for the segment key");
    if (staging) CK(c->s.ensure(c->out_rgba, staging));
    if (f.flush) CK(c->s.ensure(c->written, std::max<uint64_t>(tiles, 1)));  // per-tile written flags
    std::vector<SceneDesc> descs;
    std::vector<uint32_t> row_scene(std::max<uint64_t>(rows, 1), 0);
    for (size_t k = 0; k < scenes.size(); k++) {
        SceneInput& in = scenes[k];
        if (in.buf->memory == CGB_MEMORY_HOST) {
            in.d.out = c->out_rgba.as<uint8_t>() + in.staging_off;
            if (in.cache || in.crop)  // tiles that are not repainted keep the caller's pixels
                CK(cudaMemcpy2DAsync(in.d.out, (size_t)in.d.stride * 4, in.buf->pixels, (size_t)in.d.stride * 4,
                                     (size_t)in.d.width * 4, in.d.height, cudaMemcpyHostToDevice, st));
        } else {
            in.d.out = in.buf->pixels;
        }
        if (in.buf->flusher) in.d.written = c->written.as<uint8_t>() + in.d.tile_base;
        for (uint32_t r = 0; r < in.d.rows; r++) row_scene[in.d.row_base + r] = (uint32_t)k;
        descs.push_back(in.d);
    }
    CK(c->s.ensure(c->d_scenes, descs.size() * sizeof(SceneDesc)));
    CK(c->s.ensure(c->d_row_scene, row_scene.size() * 4));
    CK(cudaMemcpyAsync(c->d_scenes.p, descs.data(), descs.size() * sizeof(SceneDesc), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_row_scene.p, row_scene.data(), row_scene.size() * 4, cudaMemcpyHostToDevice, st));
    bg.scenes = c->d_scenes.as<SceneDesc>();
    bg.row_scene = c->d_row_scene.as<uint32_t>();

    c->last_replayed = false;
    std::vector<uint8_t> written;
    const bool graphable = c->graph_mode && !c->import_segs && lines > 0 && !f.incremental;
    std::string sig;
    if (graphable) {
        sig = frame_signature(c, f);
        auto it = c->graphs.find(sig);
        if (it != c->graphs.end() && it->second.bufs == graph_buffers(c)) {
            FrameGraph& g = it->second;
            CK(cudaGraphLaunch(g.exec, st));
            count_launches(g.launches);
            cgb_status s3 = finish_frame(c, scenes, f, written);
            if (s3) return s3;
            const FrameCounts& k = *c->h_counts;
            if (!k.overflow) {
                c->stats.lines = lines;
                c->stats.steps = k.n[FC_STEPS];
                c->stats.segments = k.produced;
                c->stats.painted_segments = k.n[FC_SEGS];
                c->stats.tile_layers = k.n[FC_TLS];
                c->stats.work_items = k.n[FC_ITEMS];
                c->stats.sort_passes = g.sort_passes;
                c->stats.item_sort_passes = g.item_sort_passes;
                c->last_replayed = true;
                post_frame(scenes, written);
                return CGB_OK;
            }
            // a count passed its capacity: nothing was painted; render the
            // frame stage by stage and capture again with the new counts
            destroy_graph(g);
            c->graphs.erase(it);
        }
    }
    // an incremental frame of a composition on its own handle, once earlier
    // incremental frames have sized its buffers: no synchronization between stages
    const bool own_incremental = f.incremental && scenes.size() == 1 && scenes[0].incr == 2 && scenes[0].comp == c;
    c->incr_form = f.incremental ? 1 : 0;
    if (own_incremental && c->incr_caps_valid && lines > 0) {
        bool done = false;
        cgb_status si = sync_free_incremental(c, f, scenes, written, &done);
        if (si) {
            c->resident_valid = false;
            return si;
        }
        if (done) {
            c->incr_form = 2;
            post_frame(scenes, written);
            return CGB_OK;
        }
        written.clear();  // a count passed its capacity: nothing was painted
    }
    cgb_status s2 = staged_frame(c, f, scenes);
    cgb_status s3 = s2 ? s2 : finish_frame(c, scenes, f, written);
    if (s3) {
        // the changed layers of this frame were taken off the dirty lists:
        // the next frame of an incremental scene rasterizes every line
        for (SceneInput& in : scenes)
            if (in.incr) in.comp->resident_valid = false;
        return s3;
    }
    post_frame(scenes, written);
    if (own_incremental)  // sizes for the sync-free form of the next frames
        note_incremental_counts(c, c->stats.steps, c->last_new_segs, c->stats.tile_layers, c->stats.work_items);
    if (graphable) capture_frame_graph(c, f, sig);
    return CGB_OK;
}

cgb_status render(cgb_composition* c, const cgb_buffer* buf, const float bg[4], const cgb_rect* crop) {
    std::vector<SceneInput> scenes(1);
    scenes[0].comp = c;
    scenes[0].buf = buf;
    scenes[0].bg = bg;
    scenes[0].crop = crop;
    return render_frame(c, scenes);
}

}  // namespace

#define HANDLE_CHECK()                                                      \
    if (!c) return fail(CGB_ERR_INVALID_ARG, "null composition handle");   \
    DeviceGuard _guard(c->device)

extern "C" {

CGB_EXPORT const char* cgb_version(void) { return "cassia_gb300 0.1.0 (sm_103a)"; }
CGB_EXPORT const char* cgb_last_error(void) { return g_last_error.c_str(); }

CGB_EXPORT cgb_status cgb_composition_new(uint32_t flags, uint64_t hbm_budget_bytes, cgb_composition** out) {
    if (!out) return fail(CGB_ERR_INVALID_ARG, "null out");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(CGB_ERR_NO_DEVICE, "no CUDA device");
    }
    cgb_composition* c = new cgb_composition();
    cudaGetDevice(&c->device);
    c->wide = (flags & CGB_COMPOSITION_WIDE_LAYERS) != 0;
    c->max_ids = c->wide ? (1u << 17) : (1u << 16);
    c->s.budget = hbm_budget_bytes;
    int prio_least = 0, prio_greatest = 0;  // numerically: least = lowest priority
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    const int prio = (flags & CGB_COMPOSITION_PRIORITY_HIGH)  ? prio_greatest
                     : (flags & CGB_COMPOSITION_PRIORITY_LOW) ? prio_least
                                                              : 0;
    cudaError_t e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio);
    if (e == cudaSuccess) e = cudaMallocHost(&c->s.pinned, 64);
    for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
    if (e == cudaSuccess) e = c->s.ensure(c->err, 256);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->err.p, 0, 4, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cgb_status st = c->cuda_fail(e, "cgb_composition_new");
        cgb_composition_free(c);
        return st;
    }
    *out = c;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_composition_free(cgb_composition* c) {
    if (!c) return CGB_OK;
    DeviceGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    DevBuf* bufs[] = {&c->p0x, &c->p0y, &c->p1x, &c->p1y, &c->lids, &c->d_layers, &c->recs, &c->lengths,
                      &c->step_off, &c->bcounts, &c->boff, &c->segs_a, &c->segs_b,
                      &c->tl_start, &c->tl_key, &c->blk_cover, &c->blk_head, &c->rlb, &c->item_state, &c->d_import, &c->written, &c->tl_cover, &c->tl_carry, &c->tl_flags, &c->item_count, &c->item_off,
                      &c->items_a, &c->items_b, &c->tile_start, &c->d_props, &c->d_grads, &c->d_stops, &c->d_unchanged, &c->out_rgba, &c->err,
                      &c->dflt_t, &c->f_kinds, &c->f_points, &c->f_cmd_off, &c->f_pt_off, &c->f_t9, &c->f_has_t,
                      &c->f_path_layer, &c->f_counts, &c->f_off, &c->g_flags, &c->g_off, &c->s.scan_sums,
                      &c->s.sort_hist, &c->s.sort_lookback, &c->s.sort_counter, &c->d_scenes, &c->d_row_scene,
                      &c->d_counts, &c->d_rast_dirty, &c->resident, &c->segs_k, &c->segs_m, &c->d_keep,
                      &c->d_scene_ids, &c->d_ranges, &c->d_extract, &c->merge_split};
    for (auto& kv : c->graphs) destroy_graph(kv.second);
    c->graphs.clear();
    if (c->h_counts) cudaFreeHost(c->h_counts);
    for (DevBuf* b : bufs) c->s.release(*b);
    for (auto& b : c->g_tmp) c->s.release(b);
    for (auto& kv : c->caches) c->s.release(kv.second.prev);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->s.pinned) cudaFreeHost(c->s.pinned);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_create_layer(cgb_composition* c, uint32_t* out_layer_id) {
    if (!c || !out_layer_id) return fail(CGB_ERR_INVALID_ARG, "null argument");
    // IdSet::acquire (mold/src/layer.rs:61-72), lowest free id first
    uint32_t id;
    if (!c->released.empty()) {
        id = *c->released.begin();
    } else {
        while (c->next_fresh < c->used.size() && c->used[c->next_fresh]) c->next_fresh++;
        id = c->next_fresh;
        if (id >= c->max_ids) return fail(CGB_ERR_LAYER_LIMIT, "create_layer: no free layer id");
        c->next_fresh++;
    }
    mark_used(c, id);
    *out_layer_id = id;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_create_layers(cgb_composition* c, size_t n, uint32_t* out_layer_ids) {
    if (!c || (n && !out_layer_ids)) return fail(CGB_ERR_INVALID_ARG, "null argument");
    for (size_t i = 0; i < n; i++) {
        cgb_status st = cgb_create_layer(c, out_layer_ids + i);
        if (st) return st;
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_insert_in_layer(cgb_composition* c, uint32_t layer_id, const uint32_t* kinds,
                                          size_t n_cmds, const float* points, size_t n_point_floats,
                                          const float* transform9) {
    HANDLE_CHECK();
    uint64_t co[2] = {0, n_cmds}, po[2] = {0, n_point_floats};
    uint8_t has = transform9 ? 1 : 0;
    float zero = 0.0f;
    return insert_paths(c, 1, &layer_id, co, kinds, po, points ? points : &zero, transform9, transform9 ? &has : nullptr);
}

CGB_EXPORT cgb_status cgb_insert_paths(cgb_composition* c, size_t n_paths, const uint32_t* layer_ids,
                                       const uint64_t* cmd_offsets, const uint32_t* kinds,
                                       const uint64_t* point_offsets, const float* points, const float* transforms9,
                                       const uint8_t* has_transform) {
    HANDLE_CHECK();
    return insert_paths(c, n_paths, layer_ids, cmd_offsets, kinds, point_offsets, points, transforms9, has_transform);
}

CGB_EXPORT cgb_status cgb_insert_lines(cgb_composition* c, uint32_t layer_id, const float* segments, size_t n_lines) {
    HANDLE_CHECK();
    if (layer_id >= c->max_ids) return fail(CGB_ERR_LAYER_LIMIT, "insert_lines: layer id out of range");
    if (n_lines && !segments) return fail(CGB_ERR_INVALID_ARG, "insert_lines: null segments");
    if (c->n_lines + n_lines >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "insert_lines: too many lines");
    CK(ensure_lines(c, c->n_lines + n_lines));
    if (n_lines) {
        std::vector<float> soa(4 * n_lines);
        std::vector<uint32_t> ids(n_lines, layer_id);
        for (size_t i = 0; i < n_lines; i++)
            for (int k = 0; k < 4; k++) soa[k * n_lines + i] = segments[4 * i + k];
        DevBuf* arrs[4] = {&c->p0x, &c->p0y, &c->p1x, &c->p1y};
        for (int k = 0; k < 4; k++)
            CK(cudaMemcpyAsync(arrs[k]->as<float>() + c->n_lines, soa.data() + k * n_lines, n_lines * 4,
                               cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->lids.as<uint32_t>() + c->n_lines, ids.data(), n_lines * 4, cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->n_lines += n_lines;
    insert_bookkeeping(c, layer_id, n_lines);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_layer_set_enabled(cgb_composition* c, uint32_t layer_id, int enabled) {
    if (!c) return fail(CGB_ERR_INVALID_ARG, "null composition handle");
    HostLayer* l = find_layer(c, layer_id);
    if (!l) return fail(CGB_ERR_NOT_FOUND, "set_enabled: unknown layer");
    const bool e = enabled != 0;
    if (l->enabled != e) {
        if (e) c->enabled_len += l->len;
        else c->enabled_len -= l->len;
        l->enabled = e;
        touch(c, layer_id);
        c->props_dirty = true;
    }
    return CGB_OK;
}

static cgb_status set_transform(cgb_composition* c, uint32_t layer_id, const float* t, uint32_t flags) {
    HostLayer* l = find_layer(c, layer_id);
    if (!l) return fail(CGB_ERR_NOT_FOUND, "set_transform: unknown layer");
    // Layer::set_transform (mold/src/layer.rs:182-201)
    static const float I[6] = {1, 0, 0, 1, 0, 0};
    const bool identity = !t || std::memcmp(t, I, sizeof(I)) == 0 ||
                          (t[0] == 1 && t[1] == 0 && t[2] == 0 && t[3] == 1 && t[4] == 0 && t[5] == 0);
    const bool has = !identity;
    if (has && !(flags & CGB_TRANSFORM_UNCHECKED) &&
        (t[0] * t[0] + t[2] * t[2] > 1.001f || t[1] * t[1] + t[3] * t[3] > 1.001f))
        return fail(CGB_ERR_SCALE, "set_transform: Layer's scaling on each axis must be between -1.0 and 1.0");
    bool changed = has != l->has_transform;
    if (!changed && has)
        for (int i = 0; i < 6; i++) changed |= l->t[i] != t[i];
    if (changed) {
        l->unchanged = 0;
        l->has_transform = has;
        if (has) std::memcpy(l->t, t, sizeof(l->t));
        touch(c, layer_id);
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_layer_set_transform(cgb_composition* c, uint32_t layer_id, const float* affine6,
                                              uint32_t flags) {
    if (!c) return fail(CGB_ERR_INVALID_ARG, "null composition handle");
    return set_transform(c, layer_id, affine6, flags);
}

CGB_EXPORT cgb_status cgb_layers_set_transforms(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                                const float* affine6, uint32_t flags) {
    if (!c || (n && (!layer_ids || !affine6))) return fail(CGB_ERR_INVALID_ARG, "null argument");
    const bool check = !(flags & CGB_TRANSFORM_UNCHECKED);
    const bool incremental = c->incremental;
    for (size_t i = 0; i < n; i++) {
        const uint32_t id = layer_ids[i];
        const float* t = affine6 + 6 * i;
        // the common case inline: an existing layer whose transform stays a
        // non-identity one; everything else through set_transform
        HostLayer* l = find_layer(c, id);
        const bool identity = t[0] == 1 && t[1] == 0 && t[2] == 0 && t[3] == 1 && t[4] == 0 && t[5] == 0;
        if (!l || identity || !l->has_transform || id >= c->layer_recs.size()) {
            cgb_status st = set_transform(c, id, t, flags);
            if (st) return st;
            continue;
        }
        if (check && (t[0] * t[0] + t[2] * t[2] > 1.001f || t[1] * t[1] + t[3] * t[3] > 1.001f))
            return fail(CGB_ERR_SCALE, "set_transform: Layer's scaling on each axis must be between -1.0 and 1.0");
        if (l->t[0] == t[0] && l->t[1] == t[1] && l->t[2] == t[2] && l->t[3] == t[3] && l->t[4] == t[4] &&
            l->t[5] == t[5])
            continue;  // equal as f32 (Layer::set_transform compares with ==)
        l->unchanged = 0;
        std::memcpy(l->t, t, sizeof(l->t));
        std::memcpy(c->layer_recs[id].t, t, sizeof(l->t));
        if (incremental) mark_raster(c, id);
        c->dirty_lo = std::min(c->dirty_lo, id);
        c->dirty_hi = std::max(c->dirty_hi, id + 1);
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_layer_set_order(cgb_composition* c, uint32_t layer_id, uint32_t order) {
    if (!c) return fail(CGB_ERR_INVALID_ARG, "null composition handle");
    HostLayer* l = find_layer(c, layer_id);
    if (!l) return fail(CGB_ERR_NOT_FOUND, "set_order: unknown layer");
    if (order >= c->max_ids) return fail(CGB_ERR_LAYER_LIMIT, "set_order: order out of range");
    if (!(l->has_order && l->order == order)) {
        l->unchanged = 0;
        l->has_order = true;
        l->order = order;
        touch(c, layer_id);
        c->props_dirty = true;
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_layer_set_props(cgb_composition* c, uint32_t layer_id, const cgb_props* props) {
    if (!c || !props) return fail(CGB_ERR_INVALID_ARG, "null argument");
    HostLayer* l = find_layer(c, layer_id);
    if (!l) return fail(CGB_ERR_NOT_FOUND, "set_props: unknown layer");
    if (props->fill_rule > 1 || props->func > 1 || props->blend_mode > 11 || props->fill_kind > 1)
        return fail(CGB_ERR_INVALID_ARG, "set_props: enum out of range");
    HostProps hp;
    hp.c = *props;
    hp.c.stops = nullptr;
    if (props->fill_kind == CGB_FILL_GRADIENT) {
        // GradientBuilder::build (style.rs:66-84): at least two stops, each in
        // [0, 1] (color_with_stop panics otherwise), linear or radial
        if (props->n_stops < 2 || !props->stops) return fail(CGB_ERR_INVALID_ARG, "set_props: gradient needs 2 stops");
        if (props->gradient_type > CGB_GRADIENT_RADIAL) return fail(CGB_ERR_INVALID_ARG, "set_props: gradient type");
        for (uint32_t i = 0; i < props->n_stops; i++) {
            const float st = props->stops[5 * (size_t)i + 4];
            if (st < 0.0f || st > 1.0f) return fail(CGB_ERR_INVALID_ARG, "set_props: gradient stop outside [0, 1]");
        }
        hp.stops.assign(props->stops, props->stops + 5 * (size_t)props->n_stops);
    }
    if (!(l->props == hp)) {
        l->unchanged = 0;
        l->props = hp;
        c->props_dirty = true;
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_layers_set_enabled(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                             const uint8_t* enabled) {
    if (!c || (n && (!layer_ids || !enabled))) return fail(CGB_ERR_INVALID_ARG, "null argument");
    for (size_t i = 0; i < n; i++) {
        cgb_status st = cgb_layer_set_enabled(c, layer_ids[i], enabled[i]);
        if (st) return st;
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_layers_set_props(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                           const cgb_props* props) {
    if (!c || (n && (!layer_ids || !props))) return fail(CGB_ERR_INVALID_ARG, "null argument");
    for (size_t i = 0; i < n; i++) {
        cgb_status st = cgb_layer_set_props(c, layer_ids[i], props + i);
        if (st) return st;
    }
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_remove_disabled(cgb_composition* c) {
    HANDLE_CHECK();
    return remove_disabled(c);
}

CGB_EXPORT cgb_status cgb_lines_len(cgb_composition* c, uint64_t* builder_len, uint64_t* actual) {
    if (!c || !builder_len || !actual) return fail(CGB_ERR_INVALID_ARG, "null argument");
    *builder_len = c->n_lines;
    *actual = actual_len(c);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_create_buffer_layer_cache(cgb_composition* c, int32_t* out_cache_id) {
    if (!c || !out_cache_id) return fail(CGB_ERR_INVALID_ARG, "null argument");
    int slot = 0;  // SmallBitSet::first_empty_slot (mold/src/layer.rs:137-141)
    while (slot < 32 && ((c->caches_used >> slot) & 1)) slot++;
    if (slot >= 32) return fail(CGB_ERR_LAYER_LIMIT, "create_buffer_layer_cache: 32 caches in use");
    c->caches_used |= 1u << slot;
    c->caches[slot] = CacheState{};
    *out_cache_id = slot;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_release_buffer_layer_cache(cgb_composition* c, int32_t cache_id) {
    HANDLE_CHECK();
    auto it = c->caches.find(cache_id);
    if (it == c->caches.end()) return fail(CGB_ERR_NOT_FOUND, "release_buffer_layer_cache: unknown cache");
    c->s.release(it->second.prev);
    c->caches.erase(it);
    c->caches_used &= ~(1u << cache_id);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_render(cgb_composition* c, const cgb_buffer* buffer, const float background[4],
                                 const cgb_rect* crop) {
    HANDLE_CHECK();
    return render(c, buffer, background, crop);
}

CGB_EXPORT cgb_status cgb_render_batch(cgb_composition* ctx, size_t n, cgb_composition* const* comps,
                                       const cgb_buffer* buffers, const float* backgrounds, const cgb_rect* crops) {
    if (!ctx || (n && (!comps || !buffers || !backgrounds))) return fail(CGB_ERR_INVALID_ARG, "null argument");
    if (n > 4096) return fail(CGB_ERR_INVALID_ARG, "render_batch: at most 4096 scenes per frame");
    DeviceGuard _guard(ctx->device);
    std::vector<SceneInput> scenes(n);
    for (size_t k = 0; k < n; k++) {
        if (!comps[k] || comps[k]->device != ctx->device)
            return fail(CGB_ERR_INVALID_ARG, "render_batch: scene on another device or null");
        scenes[k].comp = comps[k];
        scenes[k].buf = &buffers[k];
        scenes[k].bg = backgrounds + 4 * k;
        scenes[k].crop = crops ? &crops[k] : nullptr;
    }
    if (n == 0) return CGB_OK;
    return render_frame(ctx, scenes);
}

CGB_EXPORT cgb_status cgb_cassia_render(cgb_composition* c, const uint64_t* segments, size_t n,
                                        const cgb_cassia_styling* stylings, size_t m, const cgb_buffer* buffer,
                                        const float background[4]) {
    HANDLE_CHECK();
    if ((n && !segments) || (m && !stylings) || !buffer || !background)
        return fail(CGB_ERR_INVALID_ARG, "cassia_render: null argument");
    if (m > c->max_ids) return fail(CGB_ERR_LAYER_LIMIT, "cassia_render: more stylings than layer orders");
    // each styling is Props { fill_rule, Func::Draw(Style { Fill::Solid(fill), blend_mode }) }
    // (demo/src/cassia.rs:7-13, demo/src/circles.rs:117-131)
    std::vector<PaintProps> props(std::max<size_t>(m, 1),
                                  PaintProps{CGB_FILL_NONZERO, CGB_BLEND_OVER, PROPS_SOLID | PROPS_DRAW, 0, {0, 0, 0, 1}});
    for (size_t o = 0; o < m; o++) {
        const cgb_cassia_styling& sy = stylings[o];
        if (sy.fill_rule > 1 || sy.blend_mode > 11) return fail(CGB_ERR_INVALID_ARG, "cassia_render: bad styling");
        PaintProps& pp = props[o];
        pp.fill_rule = sy.fill_rule;
        pp.blend_mode = sy.blend_mode;
        pp.flags = PROPS_SOLID | PROPS_DRAW | PROPS_PRESENT;
        if (sy.blend_mode == CGB_BLEND_OVER && sy.fill[3] == 1.0f) pp.flags |= PROPS_OPAQUE_OVER;
        std::memcpy(pp.color, sy.fill, sizeof(pp.color));
    }
    c->props_host.swap(props);
    c->grads_host.clear();
    c->stops_host.clear();
    c->n_orders = (uint32_t)std::max<size_t>(m, 1);
    c->features = 0;
    c->props_dirty = false;
    c->props_version++;
    c->import_segs = segments;
    c->import_n = n;
    cgb_status s = render(c, buffer, background, nullptr);
    c->import_segs = nullptr;
    c->import_n = 0;
    c->props_dirty = true;  // a later render rebuilds the props from the layers
    return s;
}

CGB_EXPORT cgb_status cgb_pixel_segments(cgb_composition* c, uint64_t* out, size_t cap, uint64_t* out_len,
                                         uint64_t* out_none, uint32_t order) {
    HANDLE_CHECK();
    if (!out_len || !out_none || order > 1) return fail(CGB_ERR_INVALID_ARG, "pixel_segments: bad argument");
    cgb_status s0 = remove_disabled(c);
    if (s0) return s0;
    cgb_status s1 = upload_layers(c);
    if (s1) return s1;
    uint64_t P = 0, PT = 0;
    if (c->has_default_transform) {
        CK(c->s.ensure(c->dflt_t, 6 * 4));
        CK(cudaMemcpyAsync(c->dflt_t.p, c->default_transform, 24, cudaMemcpyHostToDevice, c->stream));
    }
    SceneDesc d{};
    d.p0x = c->p0x.as<float>();
    d.p0y = c->p0y.as<float>();
    d.p1x = c->p1x.as<float>();
    d.p1y = c->p1y.as<float>();
    d.lids = c->lids.as<uint32_t>();
    d.layers = c->d_layers.as<LayerRec>();
    d.default_t = c->has_default_transform ? c->dflt_t.as<float>() : nullptr;
    d.n_lines = (uint32_t)c->n_lines;
    d.n_layer_recs = c->n_layer_recs;
    d.wide = c->wide ? 1u : 0u;
    CK(c->s.ensure(c->d_scenes, sizeof(SceneDesc)));
    CK(cudaMemcpyAsync(c->d_scenes.p, &d, sizeof(SceneDesc), cudaMemcpyHostToDevice, c->stream));
    BatchGeom bg{};
    bg.scenes = c->d_scenes.as<SceneDesc>();
    bg.n_scenes = 1;
    bg.total_lines = c->n_lines;
    const int lo = order == CGB_SORT_CANONICAL ? 0 : 22;
    uint64_t* keys = nullptr;
    cgb_status s2 = build_and_rasterize(c, 0, bg, lo, 64, &P, &PT, &keys);
    if (s2) return s2;
    uint64_t* sorted = keys;
    int passes = 0;
    CK(radix_sort_u64(keys, c->segs_a.as<uint64_t>(), (uint32_t)P, lo, 64, (int)c->tuning.radix_bits, &c->s,
                      c->err.as<uint32_t>(), c->stream, &sorted, &passes, true));
    c->stats.sort_passes = passes;
    CK(stage_mark(c, 3, c->stream, nullptr));
    *out_len = P;
    *out_none = 2 * c->stats.steps - P;
    if (cap < P) {
        cgb_status s3 = check_device_error(c);
        return s3 ? s3 : fail(CGB_ERR_CAPACITY, "pixel_segments: output array too small");
    }
    if (P) CK(cudaMemcpyAsync(out, sorted, P * 8, cudaMemcpyDeviceToHost, c->stream));
    cgb_status s3 = check_device_error(c);
    if (s3) return s3;
    c->stats.build_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.rasterize_ms = elapsed(c->ev[1], c->ev[2]);
    c->stats.sort_ms = elapsed(c->ev[2], c->ev[3]);
    c->stats.total_ms = elapsed(c->ev[0], c->ev[3]);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_get_stats(cgb_composition* c, cgb_stats* out) {
    if (!c || !out) return fail(CGB_ERR_INVALID_ARG, "null argument");
    *out = c->stats;
    out->graph_replayed = c->last_replayed ? 1u : 0u;
    out->graphs_cached = (uint32_t)c->graphs.size();
    out->incremental_form = c->incr_form;
    out->reserved = 0;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_set_incremental(cgb_composition* c, int enabled) {
    HANDLE_CHECK();
    CK(cudaStreamSynchronize(c->stream));
    c->incremental = enabled != 0;
    c->resident_valid = false;
    c->resident_n = 0;
    c->incr_caps = FrameCaps{};
    c->incr_caps_valid = false;
    c->rast_ids.clear();
    c->rast_flag.clear();
    c->rast_order.clear();
    if (!c->incremental) c->s.release(c->resident);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_set_graph_mode(cgb_composition* c, int enabled, float headroom) {
    HANDLE_CHECK();
    if (!(headroom >= 0.0f && headroom <= 4.0f)) return fail(CGB_ERR_INVALID_ARG, "graph headroom must be in [0, 4]");
    CK(cudaStreamSynchronize(c->stream));
    c->graph_mode = enabled != 0;
    if (headroom != c->graph_headroom || !c->graph_mode) {
        for (auto& kv : c->graphs) destroy_graph(kv.second);
        c->graphs.clear();
    }
    c->graph_headroom = headroom;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_set_tuning(cgb_composition* c, const cgb_tuning* t) {
    if (!c || !t) return fail(CGB_ERR_INVALID_ARG, "null argument");
    if (t->radix_bits) {
        if (t->radix_bits < 4 || t->radix_bits > 9) return fail(CGB_ERR_INVALID_ARG, "radix_bits must be 4..9");
        c->tuning.radix_bits = t->radix_bits;
    }
    const uint32_t block = t->raster_block ? t->raster_block : c->tuning.raster_block;
    if (block % 32 || block < 32 || block > 256)
        return fail(CGB_ERR_INVALID_ARG, "raster_block must be a multiple of 32 in 32..256");
    // steps per block: 4 or 8 steps per thread (the current count per thread when not given)
    const uint32_t steps = t->steps_per_block ? t->steps_per_block
                                              : block * (c->tuning.steps_per_block / c->tuning.raster_block);
    if (steps != 4 * block && steps != 8 * block)
        return fail(CGB_ERR_INVALID_ARG, "steps_per_block must be 4 or 8 x raster_block");
    if (t->paint_warps && t->paint_warps != 2 && t->paint_warps != 4 && t->paint_warps != 8)
        return fail(CGB_ERR_INVALID_ARG, "paint_warps must be 2, 4 or 8");
    c->tuning.raster_block = block;
    c->tuning.steps_per_block = steps;
    if (t->paint_warps) c->tuning.paint_warps = t->paint_warps;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_get_tuning(cgb_composition* c, cgb_tuning* out) {
    if (!c || !out) return fail(CGB_ERR_INVALID_ARG, "null argument");
    *out = c->tuning;
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_get_stream(cgb_composition* c, void** out_stream) {
    if (!c || !out_stream) return fail(CGB_ERR_INVALID_ARG, "null argument");
    *out_stream = (void*)c->stream;
    return CGB_OK;
}

CGB_EXPORT uint64_t cgb_kernel_launches(void) { return g_launches.load(); }

CGB_EXPORT cgb_status cgb_selftest_bounded_wait(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(CGB_ERR_NO_DEVICE, "no CUDA device");
    }
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return fail(CGB_ERR_DEVICE, "selftest: stream");
    uint32_t flag = 0;
    cudaError_t e = selftest_bounded_wait(st, &flag);
    // the context must still work: sort a few keys the normal way
    bool sorted_ok = false;
    if (e == cudaSuccess) {
        const uint32_t n_keys = 10000;
        std::vector<uint64_t> host(n_keys);
        uint64_t x = 88172645463325252ull;
        for (auto& v : host) {
            x ^= x << 13, x ^= x >> 7, x ^= x << 17;
            v = x;
        }
        uint64_t* d = nullptr;
        if (cudaMalloc(&d, 2 * n_keys * 8) == cudaSuccess) {
            cudaMemcpyAsync(d, host.data(), n_keys * 8, cudaMemcpyHostToDevice, st);
            cgb_status s = cgb_sort_keys_noalloc(d, d + n_keys, n_keys, 0, 64, st);
            std::vector<uint64_t> back(n_keys);
            cudaMemcpyAsync(back.data(), d + n_keys, n_keys * 8, cudaMemcpyDeviceToHost, st);
            e = cudaStreamSynchronize(st);
            std::sort(host.begin(), host.end());
            sorted_ok = s == CGB_OK && e == cudaSuccess && back == host;
            cudaFree(d);
        }
    }
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(CGB_ERR_DEVICE, std::string("selftest: ") + cudaGetErrorString(e));
    if (flag != 1) return fail(CGB_ERR_DEVICE, "selftest: the bounded wait did not report its expiry");
    if (!sorted_ok) return fail(CGB_ERR_DEVICE, "selftest: the device did not sort correctly afterwards");
    return fail(CGB_ERR_DEVICE_TIMEOUT, "selftest: the bounded wait expired as designed");
}

CGB_EXPORT cgb_status cgb_composition_clear(cgb_composition* c) {
    if (!c) return fail(CGB_ERR_INVALID_ARG, "null composition handle");
    c->n_lines = 0;
    c->layers.clear();
    c->used.clear();
    c->released.clear();
    c->next_fresh = 0;
    c->enabled_len = 0;
    c->layer_recs.clear();
    c->layers_grew = true;
    c->dirty_lo = UINT32_MAX;
    c->dirty_hi = 0;
    c->props_dirty = true;
    for (auto& kv : c->caches) kv.second.tiles = 0;
    c->resident_valid = false;
    c->rast_ids.clear();
    c->rast_flag.clear();
    c->rast_order.clear();
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_synchronize(cgb_composition* c) {
    HANDLE_CHECK();
    CK(cudaStreamSynchronize(c->stream));
    return CGB_OK;
}

}  // extern "C"
