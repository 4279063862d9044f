// Host state of a composition handle -- mold's Composition, Layer and Props
// (mold/src/composition.rs, mold/src/layer.rs) -- shared by the library's two
// host translation units: composition.cu (the C ABI and the layer state) and
// frame.cu (the frame pipeline: staged frames, frame graphs, incremental
// frames).  Internal to the library.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include <nvtx3/nvToolsExt.h>

#include "cgb_internal.cuh"

namespace cgb_host {
using namespace cgb;

// The last error message of this thread (cgb_last_error) and the status it goes with.
extern thread_local std::string g_last_error;
cgb_status fail(cgb_status st, const std::string& msg);
cgb_status from_cuda(cudaError_t e, const char* where);

inline int bits_for(uint64_t max_value) {  // bits to hold values in [0, max_value]
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

inline HostProps default_props() {
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
    // Where the layer's lines sit in the builder: one run [first_line,
    // first_line + len) while `contiguous` (cgb_insert_layer_copies reads it).
    uint64_t first_line = 0;
    bool contiguous = true;
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

}  // namespace cgb_host

using namespace cgb;
using namespace cgb_host;

struct cgb_composition {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool wide = false;
    uint32_t max_ids = 1u << 16;
    Scratch s;
    cgb_tuning tuning{9, 256, 2048, 2};  // radix bits, raster block, steps per block, painter warps
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
    DevBuf raster_lines;  // [2 * (raster grid + 1)] first and last line of each rasterizer block
    DevBuf tl_start, tl_key, tl_cover, tl_carry, tl_rec_a, tl_rec_b, tl_skey, tl_sout, item_count, item_off, items_a,
        items_b, tile_start;
    DevBuf order_flag;  // u32: 1 = some scene's lines are not in non-decreasing layer order
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

#define CK(expr)                                                  \
    do {                                                          \
        cudaError_t _e = (expr);                                  \
        if (_e != cudaSuccess) return c->cuda_fail(_e, #expr);   \
    } while (0)

namespace cgb_host {

// One scene of a frame as the host prepares it.
struct SceneInput {
    cgb_composition* comp;
    const cgb_buffer* buf;
    const float* bg;
    const cgb_rect* crop;
    CacheState* cache;
    SceneDesc d;
    size_t staging_off;  // offset in the frame's host-output staging buffer
    uint8_t* mapped = nullptr;  // CGB_MEMORY_HOST_MAPPED: the buffer's device address
    // incremental frames: 0 no; 1 all lines rasterized, the resident
    // segments rebuilt; 2 only changed layers rasterized, the resident ones kept
    int incr = 0;
};

// composition.cu: the process-wide host thread pool (the caller works too;
// returns when every part is done; one run at a time)
void host_parallel(int parts, const std::function<void(int)>& f);
int host_threads();

// composition.cu: mold's per-frame host work
cgb_status upload_layers(cgb_composition* c);
void rebuild_props(cgb_composition* c);
cgb_status remove_disabled(cgb_composition* c);

// frame.cu: the frame pipeline
cudaError_t stage_mark(cgb_composition* c, int k, cudaStream_t st, const char* next);
// sb: the sort the gathered keys get (its digit counts are taken on the way);
// order_flag: render mode's order check of the lines (see launch_build_lines), or null.
cgb_status build_and_rasterize(cgb_composition* c, int render, const BatchGeom& bg, SortBits sb, uint32_t* order_flag,
                               uint64_t* n_segs, uint64_t* n_total, uint64_t** keys, bool sparse = false);
cgb_status check_device_error(cgb_composition* c);
float elapsed(cudaEvent_t a, cudaEvent_t b);
cgb_status render_frame(cgb_composition* c, std::vector<SceneInput>& scenes);
cgb_status render(cgb_composition* c, const cgb_buffer* buf, const float bg[4], const cgb_rect* crop);
void destroy_graph(FrameGraph& g);

}  // namespace cgb_host
