// C ABI of cassia_gb300: mold's Composition / Layer / Props API
// (mold/src/composition.rs, mold/src/layer.rs) over the GPU pipeline
//   build lines -> rasterize -> radix sort -> carries / work items -> paint
// (the frame pipeline is in frame.cu).
//
// Host state mirrors mold: layers by id (FxHashMap<u16, Layer> in the
// reference), an IdSet of free ids, orders_to_layers, per-cache layer counts.
// Lines live on the device (the LinesBuilder SoA, surpass/src/segment.rs:30-89)
// and are garbage-collected by the reference's rule (composition.rs:124-142).
#include "host_state.cuh"

namespace cgb_host {

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

}  // namespace cgb_host

namespace cgb {

static std::atomic<uint64_t> g_launches{0};
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launches_total() { return g_launches.load(std::memory_order_relaxed); }
void uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

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

namespace cgb_host {

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
// n lines were appended to layer `id` at builder position `first`.
void insert_bookkeeping(cgb_composition* c, uint32_t id, uint64_t n, uint64_t first) {
    if (id >= c->layers.size()) c->layers.resize((size_t)id + 1);
    HostLayer& l = c->layers[id];
    if (!l.present) {
        l = HostLayer();
        l.present = true;
    }
    if (n > 0) {
        if (l.len == 0) {
            l.first_line = first;
            l.contiguous = true;
        } else if (l.first_line + l.len != first) {
            l.contiguous = false;
        }
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
        for (HostLayer& l : c->layers) l.contiguous = false;  // the kept lines moved
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
    uint64_t at = base;
    for (size_t k = 0; k < n_paths; k++) {
        insert_bookkeeping(c, layer_ids[k], counts[k], at);
        at += counts[k];
    }
    return CGB_OK;
}

}  // namespace cgb_host

namespace cgb_host {

// A few persistent host threads for per-layer updates of long id lists (a
// frame that moves every layer of a large scene).  The calling thread works
// too; run() returns when every part is done.  After a fork the child has no
// workers, so run() then does all parts itself.
class HostPool {
public:
    static HostPool& get() {
        static HostPool* pool = new HostPool();  // never destroyed: its threads wait for work until exit
        return *pool;
    }
    int threads() const { return (int)workers_.size() + 1; }
    void run(int parts, const std::function<void(int)>& f) {
        std::lock_guard<std::mutex> one(run_mu_);
        if (workers_.empty() || getpid() != owner_) {
            for (int p = 0; p < parts; p++) f(p);
            return;
        }
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &f;
            parts_ = parts;
            next_.store(0);
            pending_ = (int)workers_.size();
            gen_++;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> g(m_);
        done_cv_.wait(g, [&] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    HostPool() : owner_(getpid()) {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned n = std::min(7u, hw - 1);
        for (unsigned i = 0; i < n; i++) workers_.emplace_back([this] { loop(); });
    }
    void work() {
        for (int p; (p = next_.fetch_add(1)) < parts_;) (*job_)(p);
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return gen_ != seen; });
                seen = gen_;
            }
            work();
            std::lock_guard<std::mutex> g(m_);
            if (--pending_ == 0) done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    pid_t owner_;
    std::mutex m_, run_mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)>* job_ = nullptr;
    int parts_ = 0;
    std::atomic<int> next_{0};
    int pending_ = 0;
    uint64_t gen_ = 0;
};

// cgb_layers_set_transforms over many layers at once: when every item takes
// the common path (an existing layer whose transform stays a non-identity
// one, within the scale limit) and the ids strictly increase, the items are
// checked, then applied, by the host pool; the result equals the sequential
// loop's.  Returns false, having changed nothing, when that does not hold.
void host_parallel(int parts, const std::function<void(int)>& f) { HostPool::get().run(parts, f); }

int host_threads() { return HostPool::get().threads(); }

bool set_transforms_parallel(cgb_composition* c, size_t n, const uint32_t* ids, const float* affine6, bool check) {
    HostPool& pool = HostPool::get();
    if (pool.threads() < 2) return false;
    const int parts = pool.threads() * 4;
    const size_t chunk = (n + parts - 1) / parts;
    std::vector<uint8_t> ok(parts, 1);
    pool.run(parts, [&](int p) {
        const size_t a = (size_t)p * chunk, b = std::min(n, a + chunk);
        bool good = true;
        for (size_t i = a; i < b && good; i++) {
            const uint32_t id = ids[i];
            const float* t = affine6 + 6 * i;
            const HostLayer* l = find_layer(c, id);
            const bool identity = t[0] == 1 && t[1] == 0 && t[2] == 0 && t[3] == 1 && t[4] == 0 && t[5] == 0;
            good = (i == 0 || id > ids[i - 1]) && l && !identity && l->has_transform && id < c->layer_recs.size() &&
                   !(check && (t[0] * t[0] + t[2] * t[2] > 1.001f || t[1] * t[1] + t[3] * t[3] > 1.001f));
        }
        ok[p] = good;
    });
    for (uint8_t g : ok)
        if (!g) return false;
    std::vector<uint32_t> lo(parts, UINT32_MAX), hi(parts, 0);
    pool.run(parts, [&](int p) {
        const size_t a = (size_t)p * chunk, b = std::min(n, a + chunk);
        uint32_t plo = UINT32_MAX, phi = 0;
        for (size_t i = a; i < b; i++) {
            const uint32_t id = ids[i];
            const float* t = affine6 + 6 * i;
            HostLayer& l = c->layers[id];
            if (l.t[0] == t[0] && l.t[1] == t[1] && l.t[2] == t[2] && l.t[3] == t[3] && l.t[4] == t[4] &&
                l.t[5] == t[5])
                continue;  // equal as f32 (Layer::set_transform compares with ==)
            l.unchanged = 0;
            std::memcpy(l.t, t, sizeof(l.t));
            std::memcpy(c->layer_recs[id].t, t, sizeof(l.t));
            plo = std::min(plo, id);
            phi = std::max(phi, id + 1);
        }
        lo[p] = plo;  // once per part: the parts' slots share cache lines
        hi[p] = phi;
    });
    for (int p = 0; p < parts; p++) {
        c->dirty_lo = std::min(c->dirty_lo, lo[p]);
        c->dirty_hi = std::max(c->dirty_hi, hi[p]);
    }
    return true;
}

}  // namespace cgb_host

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
                      &c->step_off, &c->bcounts, &c->boff, &c->segs_a, &c->segs_b, &c->raster_lines,
                      &c->tl_start, &c->tl_key, &c->blk_cover, &c->blk_head, &c->rlb, &c->item_state, &c->d_import, &c->written, &c->tl_cover, &c->tl_carry, &c->tl_rec_a, &c->tl_rec_b, &c->tl_skey, &c->tl_sout, &c->order_flag, &c->item_count, &c->item_off,
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
    insert_bookkeeping(c, layer_id, n_lines, c->n_lines - n_lines);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_insert_layer_copies(cgb_composition* c, size_t n, const uint32_t* layer_ids,
                                              cgb_composition* src, const uint32_t* src_layer_ids) {
    HANDLE_CHECK();
    if (n == 0) return CGB_OK;
    if (!src || !layer_ids || !src_layer_ids) return fail(CGB_ERR_INVALID_ARG, "insert_layer_copies: null argument");
    if (src->device != c->device) return fail(CGB_ERR_INVALID_ARG, "insert_layer_copies: handles on two devices");
    if (n >= (1u << 31)) return fail(CGB_ERR_INVALID_ARG, "insert_layer_copies: too many layers");
    // runs: the source's first line of each copy, then each copy's offset in the appended lines
    std::vector<uint64_t> runs(2 * n + 1);
    uint64_t total = 0;
    for (size_t k = 0; k < n; k++) {
        if (layer_ids[k] >= c->max_ids) return fail(CGB_ERR_LAYER_LIMIT, "insert_layer_copies: layer id out of range");
        const HostLayer* l = find_layer(src, src_layer_ids[k]);
        if (!l) return fail(CGB_ERR_NOT_FOUND, "insert_layer_copies: unknown source layer");
        if (l->len > 0 && !l->contiguous)
            return fail(CGB_ERR_INVALID_ARG, "insert_layer_copies: the source layer's lines are not one run");
        runs[k] = l->first_line;
        runs[n + k] = total;
        total += l->len;
    }
    runs[2 * n] = total;
    if (c->n_lines + total >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "insert_layer_copies: too many lines");
    // (when src == c, growing the arrays keeps the old lines in place)
    CK(ensure_lines(c, c->n_lines + total));
    const float* src4[4] = {src->p0x.as<float>(), src->p0y.as<float>(), src->p1x.as<float>(), src->p1y.as<float>()};
    const uint64_t base = c->n_lines;
    float* dst4[4] = {c->p0x.as<float>() + base, c->p0y.as<float>() + base, c->p1x.as<float>() + base,
                      c->p1y.as<float>() + base};
    CK(c->s.ensure(c->f_cmd_off, runs.size() * 8));
    CK(c->s.ensure(c->f_path_layer, n * 4));
    uint64_t* d_runs = c->f_cmd_off.as<uint64_t>();
    CK(cudaMemcpyAsync(d_runs, runs.data(), runs.size() * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f_path_layer.p, layer_ids, n * 4, cudaMemcpyHostToDevice, c->stream));
    if (src != c) {  // the source's lines are complete before they are copied
        CK(cudaEventRecord(c->ev[7], src->stream));
        CK(cudaStreamWaitEvent(c->stream, c->ev[7], 0));
    }
    CK(launch_copy_lines(src4, d_runs, d_runs + n, c->f_path_layer.as<uint32_t>(), (uint32_t)n, total, dst4,
                         c->lids.as<uint32_t>() + base, c->stream));
    c->n_lines += total;
    for (size_t k = 0; k < n; k++) insert_bookkeeping(c, layer_ids[k], runs[n + k + 1] - runs[n + k], base + runs[n + k]);
    return CGB_OK;
}

CGB_EXPORT cgb_status cgb_get_memory(cgb_composition* c, uint64_t* device_bytes) {
    if (!c || !device_bytes) return fail(CGB_ERR_INVALID_ARG, "null argument");
    *device_bytes = c->s.used;
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
    // long lists (a frame that moves every layer) on the host pool; the
    // incremental bookkeeping of changed layers stays sequential
    if (n >= (1u << 14) && !incremental && set_transforms_parallel(c, n, layer_ids, affine6, check)) return CGB_OK;
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
    cgb_status s2 = build_and_rasterize(c, 0, bg, sort_bits(lo, 64), nullptr, &P, &PT, &keys);
    if (s2) return s2;
    uint64_t* sorted = keys;
    int passes = 0;
    CK(radix_sort_u64(keys, c->segs_a.as<uint64_t>(), (uint32_t)P, sort_bits(lo, 64), (int)c->tuning.radix_bits,
                      &c->s, c->err.as<uint32_t>(), c->stream, &sorted, &passes, true));
    c->stats.sort_passes = passes;
    c->stats.sort_passes_skipped = 0;
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
    // the context must still work: sort a few keys with the pipeline's sort,
    // on scratch of its own (not the allocation-free entry point's shared
    // array, which a caller's call on another stream may be using)
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
        if (cudaMalloc(&d, 2 * n_keys * 8 + 64) == cudaSuccess) {
            uint32_t* err = reinterpret_cast<uint32_t*>(d + 2 * n_keys);
            Scratch scratch;
            uint64_t* result = nullptr;
            uint32_t err_host = 0;
            cudaError_t es = cudaMemsetAsync(err, 0, 4, st);
            if (es == cudaSuccess) es = cudaMemcpyAsync(d, host.data(), n_keys * 8, cudaMemcpyHostToDevice, st);
            if (es == cudaSuccess)
                es = radix_sort_u64(d, d + n_keys, n_keys, sort_bits(0, 64), 8, &scratch, err, st, &result, nullptr,
                                    false, nullptr, 0, 0);
            std::vector<uint64_t> back(n_keys);
            if (es == cudaSuccess)
                es = cudaMemcpyAsync(back.data(), result, n_keys * 8, cudaMemcpyDeviceToHost, st);
            if (es == cudaSuccess) es = cudaMemcpyAsync(&err_host, err, 4, cudaMemcpyDeviceToHost, st);
            e = cudaStreamSynchronize(st);
            std::sort(host.begin(), host.end());
            sorted_ok = es == cudaSuccess && e == cudaSuccess && err_host == 0 && back == host;
            scratch.release(scratch.sort_hist);
            scratch.release(scratch.sort_lookback);
            scratch.release(scratch.sort_counter);
            scratch.release(scratch.scan_sums);
            cudaFree(d);
        }
    }
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(CGB_ERR_DEVICE, std::string("selftest: ") + cudaGetErrorString(e));
    if (flag != 1) return fail(CGB_ERR_DEVICE, "selftest: the bounded wait did not report its expiry");
    if (!sorted_ok) return fail(CGB_ERR_DEVICE, "selftest: the device did not sort correctly afterwards");
    return fail(CGB_ERR_DEVICE_TIMEOUT, "selftest: the bounded wait expired as designed");
}

CGB_EXPORT cgb_status cgb_update_layers(size_t n, const cgb_layer_update* updates) {
    if (n && !updates) return fail(CGB_ERR_INVALID_ARG, "update_layers: null updates");
    std::vector<uint8_t> off;
    for (size_t k = 0; k < n; k++) {
        const cgb_layer_update& u = updates[k];
        cgb_composition* c = u.comp;
        if (!c) return fail(CGB_ERR_INVALID_ARG, "update_layers: null composition");
        cgb_status st = CGB_OK;
        if (u.n_transforms)
            st = cgb_layers_set_transforms(c, u.n_transforms, u.transform_ids, u.transforms, u.transform_flags);
        if (!st && u.n_removed) {
            off.assign(u.n_removed, 0);
            st = cgb_layers_set_enabled(c, u.n_removed, u.removed_ids, off.data());
            if (!st) st = cgb_remove_disabled(c);
        }
        if (!st && u.n_added) {
            if (!u.added_ids || !u.added_from || !u.added_from_ids)
                return fail(CGB_ERR_INVALID_ARG, "update_layers: added layers need ids and sources");
            st = cgb_create_layers(c, u.n_added, u.added_ids);
            if (!st) st = cgb_insert_layer_copies(c, u.n_added, u.added_ids, u.added_from, u.added_from_ids);
            if (!st && u.added_props) st = cgb_layers_set_props(c, u.n_added, u.added_ids, u.added_props);
            if (!st && u.added_transforms)
                st = cgb_layers_set_transforms(c, u.n_added, u.added_ids, u.added_transforms, u.transform_flags);
        }
        if (st) return fail(st, "update_layers: update " + std::to_string(k) + ": " + g_last_error);
    }
    return CGB_OK;
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
