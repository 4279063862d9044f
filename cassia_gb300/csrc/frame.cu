// The frame pipeline of cassia_gb300: mold's Composition::render
// (mold/src/composition.rs:212-329) over the GPU stages
//   build lines -> rasterize -> radix sort -> carries / work items -> paint,
// as a staged frame (counts read back between stages), a frame replayed from
// a captured CUDA graph (counts kept on the device), or an incremental frame
// (only changed layers rasterized, staged or sync-free).
#include "host_state.cuh"

namespace cgb_host {

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
cgb_status build_and_rasterize(cgb_composition* c, int render, const BatchGeom& bg, SortBits sb, uint32_t* order_flag,
                               uint64_t* n_segs, uint64_t* n_total, uint64_t** keys, bool sparse) {
    cudaStream_t st = c->stream;
    if (bg.total_lines >= (1ull << 32)) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^32 lines in a frame");
    const uint32_t L = (uint32_t)bg.total_lines;
    c->stats.lines = L;
    CK(c->s.ensure(c->recs, std::max<size_t>(L, 1) * sizeof(LineRec)));
    CK(c->s.ensure(c->lengths, std::max<size_t>(L, 1) * 4));
    CK(c->s.ensure(c->step_off, ((size_t)L + 1) * 4));
    CK(stage_mark(c, 0, st, "cgb:build_lines"));
    if (order_flag) CK(cudaMemsetAsync(order_flag, 0, 4, st));
    CK(launch_build_lines(bg, render, c->recs.as<LineRec>(), c->lengths.as<uint32_t>(), st, order_flag));
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
    CK(c->s.ensure(c->raster_lines, ((size_t)grid + 1) * 8));
    CK(c->s.ensure(c->rlb, 8));
    CK(cudaMemsetAsync(c->rlb.p, 0, 8, st));
    unsigned long long* produced = c->rlb.as<unsigned long long>();
    CK(launch_rasterize(render, bg, c->recs.as<LineRec>(), c->step_off.as<uint32_t>(), L, S, block, items,
                        c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(), produced, st, nullptr, sparse,
                        c->raster_lines.as<uint32_t>()));
    CK(cudaMemcpyAsync(&c->s.pinned[3], produced, 8, cudaMemcpyDeviceToHost, st));
    uint64_t P = 0;
    if (grid) CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid, &c->s, st, &P));
    const uint64_t PT = S ? c->s.pinned[3] : 0;
    if (P >= (1ull << 30) - 1) return fail(CGB_ERR_LAYER_LIMIT, "more than 2^30 pixel segments");
    CK(c->s.ensure(c->segs_b, std::max<size_t>(P, 1) * 8));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), slots, c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid,
                         c->segs_b.as<uint64_t>(), sb, (int)c->tuning.radix_bits, &c->s, st));
    CK(stage_mark(c, 2, st, "cgb:sort"));
    *n_segs = P;
    *n_total = PT;
    *keys = c->segs_b.as<uint64_t>();
    c->stats.segments = PT;
    return CGB_OK;
}

// cassia_render's segments (host memory) into packed keys of scene 0, with
// the sort's digit histogram counted, like build_and_rasterize.
cgb_status import_segments(cgb_composition* c, const BatchGeom& bg, SortBits sb, uint64_t* n_segs,
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
                         c->segs_b.as<uint64_t>(), sb, (int)c->tuning.radix_bits, &c->s, st));
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
    c->h_rast_dirty.resize(c->max_ids);
    uint8_t* dirty = c->h_rast_dirty.data();
    const uint32_t held = std::min(c->n_orders, c->max_ids);
    std::memset(dirty, 0, held);
    std::memset(dirty + held, 1, c->max_ids - held);  // orders no layer holds
    size_t need = c->layers.size();
    for (uint32_t id : c->rast_ids) need = std::max<size_t>(need, (size_t)id + 1);
    if (c->rast_order.size() < need) c->rast_order.resize(need, -1);
    // every listed layer marks its old and its new order (marks are idempotent
    // byte stores, so parts of a long list run on the host pool)
    int32_t* rorder = c->rast_order.data();
    uint8_t* rflag = c->rast_flag.data();
    const uint32_t* list = c->rast_ids.data();
    const size_t n_ids = c->rast_ids.size();
    auto mark = [&](size_t lo, size_t hi) {
        for (size_t k = lo; k < hi; k++) {
            const uint32_t id = list[k];
            const int32_t old = rorder[id];
            if (old >= 0 && (uint32_t)old < c->max_ids) __atomic_store_n(&dirty[(uint32_t)old], (uint8_t)1, __ATOMIC_RELAXED);
            const int32_t cur = current_order(id);
            if (cur >= 0 && (uint32_t)cur < c->max_ids) __atomic_store_n(&dirty[(uint32_t)cur], (uint8_t)1, __ATOMIC_RELAXED);
            rorder[id] = cur;
            rflag[id] = 0;
        }
    };
    // (each id costs a few host cache misses: 5,000 ids on one thread took 0.38 ms)
    if (n_ids >= 1024 && host_threads() > 1) {
        const int parts = host_threads() * 2;
        const size_t chunk = (n_ids + parts - 1) / parts;
        host_parallel(parts, [&](int p) { mark(std::min(n_ids, p * chunk), std::min(n_ids, (p + 1) * chunk)); });
    } else {
        mark(0, n_ids);
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
    if (buf->memory > CGB_MEMORY_HOST_MAPPED) return fail(CGB_ERR_INVALID_ARG, "render: unknown buffer memory kind");
    if (buf->flusher && buf->memory == CGB_MEMORY_DEVICE)
        return fail(CGB_ERR_INVALID_ARG, "render: a flusher needs a host buffer");
    const uint64_t stride = buf->width_stride ? buf->width_stride : buf->width;
    if (stride < buf->width || buf->width > (1u << 20) || buf->height > (1u << 20))
        return fail(CGB_ERR_INVALID_ARG, "render: bad width/stride/height");
    in.mapped = nullptr;
    if (buf->memory == CGB_MEMORY_HOST_MAPPED) {
        // page-locked host memory the device reaches directly (its first and
        // last byte checked; the caller vouches for the range between)
        const size_t last = ((size_t)(buf->height - 1) * stride + buf->width) * 4 - 1;
        cudaPointerAttributes a0{}, a1{};
        // the device addresses are those of the current context: make the
        // device's primary context current on this thread first
        const bool ok = cudaSetDevice(c->device) == cudaSuccess &&
                        cudaPointerGetAttributes(&a0, buf->pixels) == cudaSuccess &&
                        cudaPointerGetAttributes(&a1, buf->pixels + last) == cudaSuccess &&
                        a0.type == cudaMemoryTypeHost && a1.type == cudaMemoryTypeHost && a0.devicePointer &&
                        a1.devicePointer &&
                        (uint8_t*)a1.devicePointer - (uint8_t*)a0.devicePointer == (ptrdiff_t)last;
        if (!ok) {
            cudaGetLastError();
            return fail(CGB_ERR_INVALID_ARG, "render: a mapped buffer must be page-locked host memory");
        }
        in.mapped = (uint8_t*)a0.devicePointer;
    }
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
    CK(c->s.ensure(c->order_flag, 4));
    uint32_t* order_flag = c->order_flag.as<uint32_t>();
    // imported segments come in any order: every pass runs
    const SortBits sb = render_sort_bits(bg, c->import_segs ? nullptr : order_flag);
    cgb_status s2 = c->import_segs ? import_segments(c, bg, sb, &P, &PT, &keys)
                                   : build_and_rasterize(c, 1, bg, sb, order_flag, &P, &PT, &keys, sparse);
    if (s2) return s2;
    c->stats.painted_segments = P;
    // sort tile-major: by (global row, tile column, order)
    uint64_t* sorted = keys;
    int passes = 0;
    CK(radix_sort_u64(keys, c->segs_a.as<uint64_t>(), (uint32_t)P, sb, (int)c->tuning.radix_bits, &c->s,
                      c->err.as<uint32_t>(), st, &sorted, &passes, true));
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
    cb.order_bits = (int)bg.order_bits;
    cb.col_bits = (int)bg.col_bits;
    CK(launch_tl_scan(0, sorted, (uint32_t)P, c->bcounts.as<uint32_t>(), nullptr, cb, st));
    uint64_t G = 0;
    if (P) CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), hg, &c->s, st, &G));
    c->stats.tile_layers = G;
    const int idx_bits = bits_for(std::max<uint64_t>(G, 1) - 1);
    const int run_bits = (int)(bg.key_bits - bg.col_bits);
    if (idx_bits + run_bits > 64) return fail(CGB_ERR_LAYER_LIMIT, "render: too many tile-layer groups");
    CK(c->s.ensure(c->tl_start, (G + 1) * 4));
    CK(c->s.ensure(c->tl_key, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_cover, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_carry, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_rec_a, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_rec_b, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_skey, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->tl_sout, std::max<uint64_t>(G, 1) * 8));
    CK(c->s.ensure(c->item_count, std::max<uint64_t>(G, 1) * 4));
    CK(c->s.ensure(c->item_off, (G + 1) * 4));
    cb.tl_start = c->tl_start.as<uint32_t>();
    cb.tl_key = c->tl_key.as<uint64_t>();
    cb.tl_cover = c->tl_cover.as<uint64_t>();
    cb.tl_carry = c->tl_carry.as<uint64_t>();
    cb.tl_rec = c->tl_rec_a.as<uint64_t>();
    cb.tl_skey = c->tl_skey.as<uint64_t>();
    cb.tl_sout = c->tl_sout.as<uint64_t>();
    cb.item_count = c->item_count.as<uint32_t>();
    cb.item_off = c->item_off.as<uint32_t>();
    cb.idx_bits = idx_bits;
    CK(launch_tl_scan(1, sorted, (uint32_t)P, nullptr, c->boff.as<uint32_t>(), cb, st));
    // the (row, order) runs: the TLs' run records sorted by run
    CK(radix_sort_u64(cb.tl_rec, c->tl_rec_b.as<uint64_t>(), (uint32_t)G, sort_bits(idx_bits, idx_bits + run_bits),
                      (int)c->tuning.radix_bits, &c->s, c->err.as<uint32_t>(), st, &cb.tl_rec, nullptr, false, nullptr,
                      0, TL_SORT_BALLOT_PASSES));
    CK(launch_tl_carry((uint32_t)G, (uint32_t)P, cb, bg, st));
    uint64_t W = 0;
    if (G) CK(scan_u32(cb.item_count, cb.item_off, (uint32_t)G, &c->s, st, &W));
    c->stats.work_items = W;
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
    CK(launch_items((uint32_t)G, bg, cb, idx_bits, st));
    uint64_t* items_sorted = cb.items;
    int ipasses = 0;
    // stable sort on the tile field: each tile's items stay in order
    CK(radix_sort_u64(cb.items, cb.items_tmp, (uint32_t)W, sort_bits(tile_shift, tile_shift + tile_bits),
                      (int)c->tuning.radix_bits, &c->s, c->err.as<uint32_t>(), st, &items_sorted, &ipasses, false,
                      nullptr, 0, 1u));
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
    const DevBuf* b[] = {&c->recs,       &c->lengths,   &c->step_off,  &c->bcounts,         &c->boff, &c->raster_lines,
                         &c->segs_a,     &c->segs_b,    &c->blk_cover, &c->blk_head,        &c->tl_start,
                         &c->tl_key,     &c->tl_cover,  &c->tl_carry,  &c->tl_rec_a,        &c->tl_rec_b,
                         &c->tl_skey,    &c->tl_sout,   &c->order_flag, &c->item_count,
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
    need(c->raster_lines, (grid + 1) * 8);
    need(c->boff, (std::max(grid, hg) + 1) * 4);
    need(c->blk_cover, (hg + 1) * 8);
    need(c->blk_head, (hg + 1) * 4);
    need(c->tl_start, ((uint64_t)k.tls + 1) * 4);
    need(c->tl_key, (uint64_t)k.tls * 8);
    need(c->tl_cover, (uint64_t)k.tls * 8);
    need(c->tl_carry, (uint64_t)k.tls * 8);
    need(c->tl_rec_a, (uint64_t)k.tls * 8);
    need(c->tl_rec_b, (uint64_t)k.tls * 8);
    need(c->tl_skey, (uint64_t)k.tls * 8);
    need(c->tl_sout, (uint64_t)k.tls * 8);
    need(c->order_flag, 4);
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
    uint32_t* order_flag = c->order_flag.as<uint32_t>();
    const SortBits sb = render_sort_bits(bg, order_flag);
    CK(cudaMemsetAsync(fc, 0, sizeof(FrameCounts), st));
    CK(cudaMemsetAsync(order_flag, 0, 4, st));
    CK(stage_mark(c, 0, st, nullptr));
    CK(launch_build_lines(bg, 1, c->recs.as<LineRec>(), c->lengths.as<uint32_t>(), st, order_flag));
    CK(scan_u32(c->lengths.as<uint32_t>(), c->step_off.as<uint32_t>(), L, &c->s, st, nullptr, &fc->n[FC_STEPS]));
    CK(stage_mark(c, 1, st, nullptr));
    CK(launch_rasterize(1, bg, c->recs.as<LineRec>(), c->step_off.as<uint32_t>(), L, k.steps, block, items,
                        c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(), &fc->produced, st, fc, false,
                        c->raster_lines.as<uint32_t>()));
    CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid, &c->s, st, nullptr, &fc->n[FC_SEGS]));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), slots, c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), grid,
                         c->segs_b.as<uint64_t>(), sb, rbits, &c->s, st, k.segs));
    CK(stage_mark(c, 2, st, nullptr));
    uint64_t* sorted = nullptr;
    int passes = 0;
    CK(radix_sort_u64(c->segs_b.as<uint64_t>(), c->segs_a.as<uint64_t>(), k.segs, sb, rbits, &c->s, err, st, &sorted,
                      &passes, true, fc, FC_SEGS));
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
    cb.tl_rec = c->tl_rec_a.as<uint64_t>();
    cb.tl_skey = c->tl_skey.as<uint64_t>();
    cb.tl_sout = c->tl_sout.as<uint64_t>();
    cb.item_count = c->item_count.as<uint32_t>();
    cb.item_off = c->item_off.as<uint32_t>();
    cb.items = c->items_a.as<uint64_t>();
    cb.items_tmp = c->items_b.as<uint64_t>();
    cb.tile_start = c->tile_start.as<uint32_t>();
    cb.order_bits = (int)bg.order_bits;
    cb.col_bits = (int)bg.col_bits;
    cb.fc = fc;
    cb.tl_cap = k.tls;
    cb.items_cap = k.items;
    const int idx_bits = bits_for((uint64_t)k.tls - 1);
    const int run_bits = (int)(bg.key_bits - bg.col_bits);
    if (idx_bits + run_bits > 64) return fail(CGB_ERR_LAYER_LIMIT, "render: frame graph run record too wide");
    cb.idx_bits = idx_bits;
    CK(launch_tl_scan(0, sorted, k.segs, c->bcounts.as<uint32_t>(), nullptr, cb, st));
    CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), hg, &c->s, st, nullptr, &fc->n[FC_TLS]));
    CK(launch_tl_scan(1, sorted, k.segs, nullptr, c->boff.as<uint32_t>(), cb, st));
    CK(radix_sort_u64(cb.tl_rec, c->tl_rec_b.as<uint64_t>(), k.tls, sort_bits(idx_bits, idx_bits + run_bits), rbits,
                      &c->s, err, st, &cb.tl_rec, nullptr, false, fc, FC_TLS, TL_SORT_BALLOT_PASSES));
    CK(launch_tl_carry(k.tls, k.segs, cb, bg, st));
    CK(scan_u32(cb.item_count, cb.item_off, k.tls, &c->s, st, nullptr, &fc->n[FC_ITEMS]));
    const int tile_bits = bits_for(std::max<uint64_t>(f.tiles, 1) - 1);
    const int tile_shift = idx_bits + 3 + cb.order_bits;
    if (tile_shift + tile_bits > 64) return fail(CGB_ERR_LAYER_LIMIT, "render: frame graph item key too wide");
    CK(launch_items(k.tls, bg, cb, idx_bits, st));
    uint64_t* items_sorted = nullptr;
    int ipasses = 0;
    CK(radix_sort_u64(cb.items, cb.items_tmp, k.items, sort_bits(tile_shift, tile_shift + tile_bits), rbits, &c->s,
                      err, st, &items_sorted, &ipasses, false, fc, FC_ITEMS, 1u));
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
    const uint64_t l0 = launches_total();
    cudaStream_t st = c->stream;
    c->capturing = true;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    cgb_status s1 = e == cudaSuccess ? enqueue_counted_frame(c, f, k, &g) : CGB_ERR_DEVICE;
    cudaGraph_t graph = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(st, &graph);
    c->capturing = false;
    g.launches = launches_total() - l0;
    uncount_launches(g.launches);  // captured, not launched: counted at each replay
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
    uint32_t* flag_host = reinterpret_cast<uint32_t*>(&c->s.pinned[5]);
    *flag_host = 1;
    if (!c->import_segs && c->order_flag.p) CK(cudaMemcpyAsync(flag_host, c->order_flag.p, 4, cudaMemcpyDeviceToHost, st));
    cgb_status s3 = check_device_error(c);
    if (s3) return s3;
    // the passes of the order digits (SortBits [22, 22 + order_bits)) the sort skipped
    const uint32_t d = std::min(9u, std::max(1u, c->tuning.radix_bits));
    c->stats.sort_passes_skipped = *flag_host == 0 ? (f.bg.order_bits + d - 1) / d : 0u;
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
    CK(sc.ensure(c->raster_lines, ((uint64_t)grid + 1) * 8));
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
    CK(sc.ensure(c->tl_rec_a, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->tl_rec_b, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->tl_skey, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->tl_sout, (uint64_t)k.tls * 8));
    CK(sc.ensure(c->order_flag, 4));
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
    uint32_t* order_flag = c->order_flag.as<uint32_t>();
    const SortBits sb = render_sort_bits(bg, order_flag);
    CK(cudaMemsetAsync(fc, 0, sizeof(FrameCounts), st));
    CK(cudaMemsetAsync(order_flag, 0, 4, st));
    CK(cudaMemcpyAsync(c->d_keep.p, &src, sizeof(src), cudaMemcpyHostToDevice, st));
    CK(stage_mark(c, 0, st, "cgb:build_lines"));
    CK(launch_build_lines(bg, 1, c->recs.as<LineRec>(), c->lengths.as<uint32_t>(), st, order_flag));
    CK(scan_u32(c->lengths.as<uint32_t>(), c->step_off.as<uint32_t>(), L, &sc, st, nullptr, &fc->n[FC_STEPS]));
    CK(stage_mark(c, 1, st, "cgb:rasterize"));
    CK(launch_rasterize(1, bg, c->recs.as<LineRec>(), c->step_off.as<uint32_t>(), L, k.steps, block, items,
                        c->segs_a.as<uint64_t>(), c->bcounts.as<uint32_t>(), &fc->produced, st, fc, true,
                        c->raster_lines.as<uint32_t>()));
    CK(scan_u32(c->bcounts.as<uint32_t>(), c->boff.as<uint32_t>(), (uint32_t)grid, &sc, st, nullptr,
                &fc->n[FC_NEW]));
    CK(radix_gather_hist(c->segs_a.as<uint64_t>(), (uint32_t)slots, c->bcounts.as<uint32_t>(),
                         c->boff.as<uint32_t>(), (uint32_t)grid, c->segs_b.as<uint64_t>(), sb, rbits, &sc, st, ic.segs));
    CK(stage_mark(c, 2, st, "cgb:sort"));
    uint64_t* sorted_new = nullptr;
    int passes = 0;
    CK(radix_sort_u64(c->segs_b.as<uint64_t>(), c->segs_a.as<uint64_t>(), ic.segs, sb, rbits, &sc, err, st,
                      &sorted_new, &passes, true, fc, FC_NEW));
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
        } else if (in.buf->memory == CGB_MEMORY_HOST_MAPPED) {
            in.d.out = in.mapped;  // the painter writes the caller's pages directly
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
                c->incr_form = 0;
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

}  // namespace cgb_host
