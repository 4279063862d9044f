// Line expansion and rasterization kernels.
//
//   k_flatten      mold PathSegments (mold/src/path/segments.rs:97-263) with
//                  Transform (mold/src/path/transform.rs:56-94): one thread per
//                  path; a count pass, a scan of the counts, a write pass.
//   k_build_lines  LinesBuilder::build (surpass/src/segment.rs:91-237): one
//                  thread per line; writes a packed 32-byte LineRec + length,
//                  and flags a scene whose lines are not in non-decreasing
//                  layer order (the sort may skip its order passes otherwise).
//   k_block_lines  the first and last line of each rasterizer block.
//   k_rasterize    Rasterizer::rasterize (surpass/src/rasterizer/mod.rs:214-285):
//                  each thread walks 4 or 8 consecutive pixel steps; each block
//                  block-scans the per-thread counts, stages its segments in
//                  shared memory and stores them coalesced into its own run
//                  of slots; k_gather_hist (k_sort.cu) packs the runs.  No
//                  NONE slots are materialized.
#include "cgb_internal.cuh"

namespace cgb {

namespace {

// ---------------------------------------------------------------------------
// path flattening
// ---------------------------------------------------------------------------

struct Pt {
    float x, y;
};
__device__ __forceinline__ Pt pmul(Pt p, float s) { return {p.x * s, p.y * s}; }
__device__ __forceinline__ Pt padd(Pt a, Pt b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ Pt plerp(float t, Pt p0, Pt p1) { return padd(pmul(p0, 1.0f - t), pmul(p1, t)); }
__device__ __forceinline__ float lerp1(float t, float a, float b) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ Pt from_weighted(float x, float y, float w) {
    float r = 1.0f / w;
    return {x * r, y * r};
}
__device__ __forceinline__ bool approx_eq(Pt a, Pt b) {
    const float eps = 1.1920929e-7f;
    return fabsf(a.x - b.x) < eps && fabsf(a.y - b.y) < eps;
}

struct Cmd {
    uint32_t kind;
    Pt p[4];
    float w[4];
};

__device__ __forceinline__ int cmd_floats(uint32_t kind) {
    switch (kind) {
        case CGB_CMD_LINE: return 4;
        case CGB_CMD_QUAD: return 6;
        case CGB_CMD_RAT_QUAD: return 9;
        case CGB_CMD_CUBIC: return 8;
        case CGB_CMD_RAT_CUBIC: return 12;
        default: return 0;
    }
}

// Path::line/quad/rat_quad/cubic/rat_cubic storage (mold/src/path/mod.rs:53-143).
__device__ Cmd load_cmd(uint32_t kind, const float* f) {
    Cmd c;
    c.kind = kind;
    switch (kind) {
        case CGB_CMD_LINE:
        case CGB_CMD_QUAD:
        case CGB_CMD_CUBIC: {
            int np = kind == CGB_CMD_LINE ? 2 : kind == CGB_CMD_QUAD ? 3 : 4;
            for (int k = 0; k < np; k++) c.p[k] = {f[2 * k], f[2 * k + 1]};
            break;
        }
        case CGB_CMD_RAT_QUAD:
        case CGB_CMD_RAT_CUBIC: {
            int np = kind == CGB_CMD_RAT_QUAD ? 3 : 4;
            for (int k = 0; k < np; k++) {
                float w = f[3 * k + 2];
                c.p[k] = pmul(Pt{f[3 * k], f[3 * k + 1]}, w);
                c.w[k] = w;
            }
            break;
        }
        default: break;
    }
    return c;
}

struct DTransform {
    float t[9];
    bool persp;
};

__device__ DTransform make_transform(const float* t9) {
    DTransform r;
    float rc = 1.0f / t9[8];
    for (int i = 0; i < 9; i++) r.t[i] = t9[i] * rc;
    const float eps = 1.1920929e-7f;
    r.persp = fabsf(r.t[6]) > eps || fabsf(r.t[7]) > eps;
    return r;
}

// Transform::transform (transform.rs:71-93)
__device__ Cmd apply_transform(const DTransform& T, const Cmd& c) {
    Cmd r = c;
    const float* t = T.t;
    int np = c.kind == CGB_CMD_LINE ? 2 : (c.kind == CGB_CMD_QUAD || c.kind == CGB_CMD_RAT_QUAD) ? 3 : 4;
    if (c.kind == CGB_CMD_CLOSE) return r;
    bool rational = c.kind == CGB_CMD_RAT_QUAD || c.kind == CGB_CMD_RAT_CUBIC;
    if (c.kind == CGB_CMD_LINE || (!rational && !T.persp)) {
        for (int k = 0; k < np; k++) {
            float x = c.p[k].x, y = c.p[k].y;
            if (!T.persp) {
                r.p[k] = {t[0] * x + t[1] * y + t[2], t[3] * x + t[4] * y + t[5]};
            } else {
                float o0 = t[0] * x + t[1] * y + t[2] * 1.0f;
                float o1 = t[3] * x + t[4] * y + t[5] * 1.0f;
                float o2 = t[6] * x + t[7] * y + t[8] * 1.0f;
                r.p[k] = from_weighted(o0, o1, o2);
            }
        }
        return r;
    }
    for (int k = 0; k < np; k++) {
        float w = rational ? c.w[k] : 1.0f;
        float x = c.p[k].x, y = c.p[k].y;
        r.p[k] = {t[0] * x + t[1] * y + t[2] * w, t[3] * x + t[4] * y + t[5] * w};
        r.w[k] = t[6] * x + t[7] * y + t[8] * w;
    }
    if (c.kind == CGB_CMD_QUAD) r.kind = CGB_CMD_RAT_QUAD;
    if (c.kind == CGB_CMD_CUBIC) r.kind = CGB_CMD_RAT_CUBIC;
    return r;
}

__device__ Pt eval_curve(const Cmd& c, float tt) {
    switch (c.kind) {
        case CGB_CMD_QUAD: return plerp(tt, plerp(tt, c.p[0], c.p[1]), plerp(tt, c.p[1], c.p[2]));
        case CGB_CMD_CUBIC: {
            Pt a = plerp(tt, plerp(tt, c.p[0], c.p[1]), plerp(tt, c.p[1], c.p[2]));
            Pt b = plerp(tt, plerp(tt, c.p[1], c.p[2]), plerp(tt, c.p[2], c.p[3]));
            return plerp(tt, a, b);
        }
        case CGB_CMD_RAT_QUAD: {
            Pt b = plerp(tt, plerp(tt, c.p[0], c.p[1]), plerp(tt, c.p[1], c.p[2]));
            float w = lerp1(tt, lerp1(tt, c.w[0], c.w[1]), lerp1(tt, c.w[1], c.w[2]));
            return pmul(b, 1.0f / w);
        }
        default: {  // RAT_CUBIC
            Pt a = plerp(tt, plerp(tt, c.p[0], c.p[1]), plerp(tt, c.p[1], c.p[2]));
            Pt b = plerp(tt, plerp(tt, c.p[1], c.p[2]), plerp(tt, c.p[2], c.p[3]));
            Pt bz = plerp(tt, a, b);
            float wa = lerp1(tt, lerp1(tt, c.w[0], c.w[1]), lerp1(tt, c.w[1], c.w[2]));
            float wb = lerp1(tt, lerp1(tt, c.w[1], c.w[2]), lerp1(tt, c.w[2], c.w[3]));
            return pmul(bz, 1.0f / lerp1(tt, wa, wb));
        }
    }
}

__device__ __forceinline__ float dev3(float a, float b, float c) { return a + c - 2.0f * b; }
__device__ __forceinline__ float dev4(float a, float b, float c, float d) {
    return fmaxf(fabsf(a + c - 2.0f * b), fabsf(b + d - 2.0f * c));
}

// Output side of PathSegments::line (segments.rs:106-114): tracks the
// closing and last points and counts or stores each emitted segment.
struct LineSink {
    bool has_last = false, has_closing = false;
    Pt last_point{0, 0}, closing_point{0, 0};
    uint32_t n = 0;
    bool write = false;
    uint32_t o = 0, lid = 0;
    float *p0x = nullptr, *p0y = nullptr, *p1x = nullptr, *p1y = nullptr;
    uint32_t* lids = nullptr;

    __device__ void line(Pt a, Pt b) {
        if (!has_closing) {
            has_closing = true;
            closing_point = a;
        }
        has_last = true;
        last_point = b;
        if (write) {
            p0x[o] = a.x;
            p0y[o] = a.y;
            p1x[o] = b.x;
            p1y[o] = b.y;
            lids[o] = lid;
            o++;
        }
        n++;
    }
};

// Flattens one path (PathSegments as an iterator, segments.rs:233-262), each
// curve run to completion with the incremental-t sampler of next_segment.
__device__ void flatten_path(const uint32_t* kinds, uint32_t n_cmds, const float* pts, const float* t9,
                             LineSink& sink) {
    DTransform T;
    const bool has_t = t9 != nullptr;
    if (has_t) T = make_transform(t9);
    const float PIXEL_ACCURACY = 0.5f / (float)PIXEL_WIDTH;
    uint64_t po = 0;
    for (uint32_t ci = 0; ci < n_cmds; ci++) {
        const uint32_t kind = kinds[ci];
        if (kind == CGB_CMD_CLOSE) {
            // close (segments.rs:208-223)
            if (sink.has_closing && sink.has_last) {
                if (!approx_eq(sink.closing_point, sink.last_point)) sink.line(sink.last_point, sink.closing_point);
                sink.has_closing = false;
            }
            continue;
        }
        Cmd c = load_cmd(kind, pts + po);
        po += cmd_floats(kind);
        if (has_t) c = apply_transform(T, c);
        if (c.kind == CGB_CMD_LINE) {
            sink.line(c.p[0], c.p[1]);
            continue;
        }
        Pt first, last;
        float dx, dy;
        if (c.kind == CGB_CMD_QUAD) {
            first = c.p[0];
            last = c.p[2];
            dx = dev3(c.p[0].x, c.p[1].x, c.p[2].x);
            dy = dev3(c.p[0].y, c.p[1].y, c.p[2].y);
        } else if (c.kind == CGB_CMD_CUBIC) {
            first = c.p[0];
            last = c.p[3];
            dx = dev4(c.p[0].x, c.p[1].x, c.p[2].x, c.p[3].x);
            dy = dev4(c.p[0].y, c.p[1].y, c.p[2].y, c.p[3].y);
        } else if (c.kind == CGB_CMD_RAT_QUAD) {
            Pt p0 = from_weighted(c.p[0].x, c.p[0].y, c.w[0]);
            Pt p1 = from_weighted(c.p[1].x, c.p[1].y, c.w[1]);
            Pt p2 = from_weighted(c.p[2].x, c.p[2].y, c.w[2]);
            first = p0;
            last = p2;
            dx = dev3(p0.x, p1.x, p2.x);
            dy = dev3(p0.y, p1.y, p2.y);
        } else {
            Pt p0 = from_weighted(c.p[0].x, c.p[0].y, c.w[0]);
            Pt p1 = from_weighted(c.p[1].x, c.p[1].y, c.w[1]);
            Pt p2 = from_weighted(c.p[2].x, c.p[2].y, c.w[2]);
            Pt p3 = from_weighted(c.p[3].x, c.p[3].y, c.w[3]);
            first = p0;
            last = p3;
            dx = dev4(p0.x, p1.x, p2.x, p3.x);
            dy = dev4(p0.y, p1.y, p2.y, p3.y);
        }
        // subdivisions (segments.rs:51-72) then next_segment (:116-157)
        const float dev2 = dx * dx + dy * dy;
        uint64_t subs = 0;
        if (!(dev2 < PIXEL_ACCURACY)) {
            uint64_t count = f2usize(ceilf(sqrtf(sqrtf(dev2) * 2.0f / (8.0f * PIXEL_ACCURACY))));
            subs = (count > 1 ? count : 1) - 1;
        }
        if (subs == 0) {
            sink.line(first, last);
            continue;
        }
        const float increment = 1.0f / (float)subs;
        float t = 0.0f;
        Pt point = first;
        for (uint64_t left = subs; left > 1; left--) {
            t += increment;
            Pt np = eval_curve(c, t);
            sink.line(point, np);
            point = np;
        }
        sink.line(point, last);
    }
}

__global__ void k_flatten(int write, const uint32_t* __restrict__ kinds, const float* __restrict__ points,
                          const uint64_t* __restrict__ cmd_off, const uint64_t* __restrict__ pt_off,
                          const float* __restrict__ transforms9, const uint8_t* __restrict__ has_t,
                          const uint32_t* __restrict__ path_layer, uint32_t n_paths, uint32_t* __restrict__ counts,
                          const uint32_t* __restrict__ out_off, float* __restrict__ p0x, float* __restrict__ p0y,
                          float* __restrict__ p1x, float* __restrict__ p1y, uint32_t* __restrict__ lids) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_paths) return;
    const float* t9 = (transforms9 && has_t && has_t[k]) ? transforms9 + 9 * (uint64_t)k : nullptr;
    const uint64_t c0 = cmd_off[k], c1 = cmd_off[k + 1];
    LineSink sink;
    if (write) {
        sink.write = true;
        sink.o = out_off[k];
        sink.lid = path_layer[k];
        sink.p0x = p0x;
        sink.p0y = p0y;
        sink.p1x = p1x;
        sink.p1y = p1y;
        sink.lids = lids;
    }
    flatten_path(kinds + c0, (uint32_t)(c1 - c0), points + pt_off[k], t9, sink);
    if (!write) counts[k] = sink.n;
}

// ---------------------------------------------------------------------------
// LinesBuilder::build
// ---------------------------------------------------------------------------

constexpr int MAX_SMEM_SCENES = 1024;

// Scene of global line g: the last scene whose line_base <= g.
__device__ __forceinline__ uint32_t scene_of_line(const uint64_t* base, uint32_t n_scenes, uint64_t g) {
    uint32_t lo = 0, hi = n_scenes;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_build_lines(BatchGeom bg, int cull, LineRec* __restrict__ recs, uint32_t* __restrict__ lengths,
                              uint32_t* __restrict__ order_flag) {
    __shared__ uint64_t s_base[MAX_SMEM_SCENES];
    const uint32_t ns = min(bg.n_scenes, (uint32_t)MAX_SMEM_SCENES);
    for (uint32_t k = threadIdx.x; k < ns; k += blockDim.x) s_base[k] = bg.scenes[k].line_base;
    __syncthreads();
    const uint64_t gi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= bg.total_lines) return;
    const uint32_t sc = scene_of_line(s_base, ns, gi);
    const SceneDesc& S = bg.scenes[sc];
    const uint32_t i = (uint32_t)(gi - S.line_base);
    float p0x = S.p0x[i], p0y = S.p0y[i], p1x = S.p1x[i], p1y = S.p1y[i];
    const uint32_t lid = S.lids[i];
    const LayerRec* __restrict__ layers = S.layers;
    const uint32_t n_layer_recs = S.n_layer_recs;
    const float* __restrict__ default_t = S.default_t;
    LineRec r{0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0u};
    uint32_t length = 0;
    LayerRec lrec{};
    if (lid < n_layer_recs) lrec = layers[lid];
    const uint32_t flags = lrec.flags, lorder = lrec.order;
    const bool present = (flags & LAYER_PRESENT) != 0;
    const uint32_t order = (present && (flags & LAYER_HAS_ORDER)) ? lorder : lid;
    if (order_flag && i > 0) {
        // the scene's lines in non-decreasing order?  (The line before is
        // mostly of the same layer, whose record is already cached.)
        const uint32_t plid = S.lids[i - 1];
        uint32_t porder = plid;
        if (plid < n_layer_recs) {
            const uint2 h = *reinterpret_cast<const uint2*>(&layers[plid]);
            if ((h.x & LAYER_PRESENT) && (h.x & LAYER_HAS_ORDER)) porder = h.y;
        }
        if (order < porder) *order_flag = 1u;
    }
    if (!(present && !(flags & LAYER_ENABLED))) {
        // the layer's affine, else the builder's default (segment.rs:130-142)
        bool has_t = false;
        float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f, t4 = 0.f, t5 = 0.f;
        if (present && (flags & LAYER_HAS_TRANSFORM)) {
            const float* tr = lrec.t;
            t0 = tr[0], t1 = tr[1], t2 = tr[2], t3 = tr[3], t4 = tr[4], t5 = tr[5];
            has_t = true;
        } else if (default_t) {
            t0 = default_t[0], t1 = default_t[1], t2 = default_t[2], t3 = default_t[3], t4 = default_t[4],
            t5 = default_t[5];
            has_t = true;
        }
        if (has_t) {
            float a = __fmaf_rn(t0, p0x, __fmaf_rn(t1, p0y, t4));
            float b = __fmaf_rn(t2, p0x, __fmaf_rn(t3, p0y, t5));
            float c = __fmaf_rn(t0, p1x, __fmaf_rn(t1, p1y, t4));
            float d = __fmaf_rn(t2, p1x, __fmaf_rn(t3, p1y, t5));
            p0x = a;
            p0y = b;
            p1x = c;
            p1y = d;
        }
        int32_t p0x_sub = to_sub_pixel(p0x), p0y_sub = to_sub_pixel(p0y);
        int32_t p1x_sub = to_sub_pixel(p1x), p1y_sub = to_sub_pixel(p1y);
        // Render mode: a line wholly above, below or right of the canvas (with
        // a pixel of margin for rounding) yields only segments the painter
        // never reads, unless the 12-bit tile_j / 13-bit tile_i fields could
        // wrap back into the canvas (|y| >= 16,384 px, x >= 30,720 px).
        // incremental frames: only the lines of changed layers (by order)
        bool off_canvas = cull && S.rast_dirty && !S.rast_dirty[order];
        if (cull && !off_canvas) {
            const int32_t ymin = min(p0y_sub, p1y_sub), ymax = max(p0y_sub, p1y_sub);
            const int32_t xmin = min(p0x_sub, p1x_sub), xmax = max(p0x_sub, p1x_sub);
            const int32_t lim_y = 16384 * PIXEL_WIDTH, lim_x = 30720 * PIXEL_WIDTH;
            off_canvas = off_canvas || (ymax < -PIXEL_WIDTH && ymin > -lim_y) ||
                         (ymin >= (int32_t)(S.rows * 8 + 1) * PIXEL_WIDTH && ymax < lim_y) ||
                         (xmin >= (int32_t)(S.row_len * 8 + 1) * PIXEL_WIDTH && xmax < lim_x);
        }
        if (p0y_sub != p1y_sub && !off_canvas) {
            int32_t dx = wsub(p1x_sub, p0x_sub), dy = wsub(p1y_sub, p0y_sub);
            bool dx_dy = wabs(dx) > wabs(dy);
            bool sum_0 = wadd(dx, dy) > 0 || (dx == wsub(0, dy) && dx < dy);
            int32_t start_sub = dx_dy ? (sum_0 ? p0x_sub : p1x_sub) : (sum_0 ? p0y_sub : p1y_sub);
            int32_t end_sub = dx_dy ? (sum_0 ? p1x_sub : p0x_sub) : (sum_0 ? p1y_sub : p0y_sub);
            int32_t start = start_sub >> PIXEL_SHIFT;
            int32_t end = (end_sub & PIXEL_MASK) == 0 ? end_sub >> PIXEL_SHIFT : (end_sub >> PIXEL_SHIFT) + 1;
            length = (uint32_t)wsub(end, start);
            const float rcp = 1.0f / (float)PIXEL_WIDTH;
            float fp0x = (float)p0x_sub * rcp, fp0y = (float)p0y_sub * rcp;
            float px = dx_dy ? fp0x : fp0y, py = dx_dy ? fp0y : fp0x;
            float slope = dx_dy ? (float)dy / (float)dx : (float)dx / (float)dy;
            float slope_recip = 1.0f / slope;
            bool xp = dx > 0, yp = dy > 0;
            uint32_t oct = dx_dy ? (xp ? (yp ? 0u : 7u) : (yp ? 3u : 4u)) : (xp ? (yp ? 1u : 6u) : (yp ? 2u : 5u));
            r.start = start;
            r.start_f32 = (float)start_sub * rcp;
            r.end_f32 = (float)end_sub * rcp;
            r.slope = slope;
            r.slope_recip = slope_recip;
            r.py_slope_px = __fmaf_rn(slope, -px, py);
            r.px_slope_recip_py = __fmaf_rn(slope_recip, -py, px);
            r.order_octant = (sc << LINE_SCENE_SHIFT) | (order << 3) | oct;
        }
    }
    recs[gi] = r;
    lengths[gi] = length;
}

// ---------------------------------------------------------------------------
// rasterization
// ---------------------------------------------------------------------------

// The fields of one CompactSegment: tile_j, the stored tile_i (+256) and the
// low 22 bits (tile_y | tile_x | area | cover).
struct SegFields {
    int32_t tj, tis;
    uint32_t low;
};

// tiles + area_cover + CompactSegment::new (rasterizer/mod.rs:134-189).  The
// octant's coordinate swaps are selects, so lanes on lines of different
// octants do not diverge.
__device__ __forceinline__ SegFields seg_fields(int32_t x0, int32_t x1, int32_t y0, int32_t y1, int32_t bx,
                                                int32_t by, uint32_t oct) {
    const bool swap = (0x66u >> oct) & 1u;    // octants 1, 2, 5, 6: x and y exchanged
    const bool flip_a = (0x44u >> oct) & 1u;  // 2, 6: the first coordinate's ends exchanged
    const bool flip_b = (0x78u >> oct) & 1u;  // 3, 4, 5, 6: the second coordinate's ends exchanged
    const int32_t cx = swap ? by : bx, cy = swap ? bx : by;
    const int32_t p0 = swap ? y0 : x0, p1 = swap ? y1 : x1;
    const int32_t q0 = swap ? x0 : y0, q1 = swap ? x1 : y1;
    const int32_t a0 = flip_a ? p1 : p0, a1 = flip_a ? p0 : p1;
    const int32_t b0 = flip_b ? q1 : q0, b1 = flip_b ? q0 : q1;
    const int32_t ti = (int16_t)(cx >> TILE_SHIFT);
    const int32_t tj = (int16_t)(cy >> TILE_SHIFT);
    const uint32_t tx = (uint32_t)(cx & TILE_MASK), ty = (uint32_t)(cy & TILE_MASK);
    const int32_t border = wadd(a0 & ~PIXEL_MASK, PIXEL_WIDTH);
    const int32_t height = wsub(b1, b0);
    const int32_t triangle = (int16_t)(wmul(height, wsub(a1, a0)) / 2);
    const int32_t rectangle = (int16_t)wmul(height, wsub(border, a1));
    const int32_t area = (int16_t)(uint16_t)((uint32_t)triangle + (uint32_t)rectangle);
    const int32_t cover = (int8_t)height;
    const int32_t tis = (int16_t)(uint16_t)((uint32_t)(ti > -1 ? ti : -1) + 256u);
    return SegFields{tj, tis, (ty << 19) | (tx << 16) | (((uint32_t)area & 0x3FFu) << 6) | ((uint32_t)cover & 0x3Fu)};
}

// The packed CompactSegment (raster_segment.rs:142-154; with `wide`, the
// 17-bit layer field of the widened format in place of is_none).
__device__ __forceinline__ uint64_t pack_fields(uint32_t wide, uint32_t layer, const SegFields& f) {
    const uint64_t hi = ((uint64_t)((uint32_t)f.tj & 0xFFFu) << 13) | ((uint32_t)f.tis & 0x1FFFu);
    const uint64_t mid = wide ? ((hi << 17) | (layer & 0x1FFFFu)) : ((hi << 16) | (layer & 0xFFFFu));
    return (mid << 22) | f.low;
}

__device__ __forceinline__ bool intersects_y_border(int32_t y0, int32_t y1) {
    return (y0 & PIXEL_MASK) != 0 && (y1 & PIXEL_MASK) != 0 && (y0 >> PIXEL_SHIFT) != (y1 >> PIXEL_SHIFT);
}

// Render format: culls segments the painter never reads (rows outside the
// canvas, tiles right of it, 13-bit tile_i wrap) and re-keys the rest by
// (global tile row, order, tile column + 1) above the reference's low 22 bits.
// The tile fields are read as the packed segment stores them (12-bit
// tile_j, 13-bit tile_i), so wrapped values land where the reference's do.
struct SceneRaster {
    uint32_t wide, rows, row_len, row_base;
};

__device__ __forceinline__ bool render_key(const SceneRaster& sr, const BatchGeom& bg, uint32_t layer,
                                           const SegFields& f, uint64_t& out) {
    const int32_t tj = (int32_t)((uint32_t)f.tj << 20) >> 20;
    const int32_t ti = ((int32_t)((uint32_t)f.tis << 19) >> 19) - 256;
    if (tj < 0 || tj >= (int32_t)sr.rows || ti < -1 || ti >= (int32_t)sr.row_len) return false;
    const uint32_t lmask = sr.wide ? 0x1FFFFu : 0xFFFFu;
    out = (make_render_key(bg, sr.row_base + (uint32_t)tj, layer & lmask, (uint32_t)(ti + 1)) << 22) | f.low;
    return true;
}

// One pixel step (rasterizer/mod.rs:233-281): one or two segments, at out[0]
// and out[1]; returns the mask of those kept (all of them outside render
// mode); `produced` counts both.
template <int RENDER>
__device__ __forceinline__ uint32_t raster_step(const SceneRaster& sr, const BatchGeom& bg, const LineRec& l,
                                                int32_t pi, uint64_t out[2], int& produced) {
    const uint32_t oct = l.order_octant & 7, layer = (l.order_octant >> 3) & ((1u << (LINE_SCENE_SHIFT - 3)) - 1);
    const int32_t x0i = wadd(l.start, pi);
    const int32_t x1i = wadd(x0i, 1);
    const int32_t border_x = x0i;
    const float x0 = fmaxf((float)x0i, l.start_f32);
    const float x1 = fminf((float)x1i, l.end_f32);
    const float y0 = __fmaf_rn(l.slope, x0, l.py_slope_px);
    const float y1 = __fmaf_rn(l.slope, x1, l.py_slope_px);
    const int32_t x0s = to_sub_pixel(x0), x1s = to_sub_pixel(x1), y0s = to_sub_pixel(y0), y1s = to_sub_pixel(y1);
    const bool inter = intersects_y_border(y0s, y1s);
    // the crossing of the pixel row border (used only when the step crosses it)
    const int32_t ys = (int32_t)((uint32_t)(max(y0s, y1s) >> PIXEL_SHIFT) << PIXEL_SHIFT);
    const int32_t xs = to_sub_pixel(__fmaf_rn(l.slope_recip, (float)(max(y0s, y1s) >> PIXEL_SHIFT), l.px_slope_recip_py));
    const int32_t ex = inter ? xs : x1s, ey = inter ? ys : y1s;
    uint32_t mask = 0;
    {
        const SegFields f = seg_fields(x0s, ex, y0s, ey, border_x, min(ey, y0s) >> PIXEL_SHIFT, oct);
        if (RENDER) {
            if (render_key(sr, bg, layer, f, out[0])) mask |= 1u;
        } else {
            out[0] = pack_fields(sr.wide, layer, f);
            mask |= 1u;
        }
    }
    produced += 1;
    if (inter) {
        const SegFields f = seg_fields(xs, x1s, ys, y1s, border_x, min(ys, y1s) >> PIXEL_SHIFT, oct);
        if (RENDER) {
            if (render_key(sr, bg, layer, f, out[1])) mask |= 2u;
        } else {
            out[1] = pack_fields(sr.wide, layer, f);
            mask |= 2u;
        }
        produced += 1;
    }
    return mask;
}


constexpr uint32_t RASTER_LINE_STAGE = 1024;  // line offsets staged per rasterizer block

__device__ __forceinline__ uint32_t find_line(const uint32_t* __restrict__ off, uint32_t n_lines, uint64_t s) {
    // largest l with off[l] <= s (off has n_lines + 1 entries, off[0] = 0)
    uint32_t lo = 0, hi = n_lines;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if ((uint64_t)off[mid] <= s) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The first and the last line of each rasterizer block's steps (per_block
// steps per block): each line with steps [a, e) records itself for the blocks
// whose first or last step lies in it.  block_lines[b] = first line of block
// b, block_lines[nb + 1 + b] = its last line, for the nb blocks of the count.
constexpr int BL_LINES = 4;  // lines per thread of k_block_lines (one 16-byte load of their offsets)
__global__ void k_block_lines(const uint32_t* __restrict__ off, uint32_t n_lines, uint64_t n_steps,
                              uint32_t per_block, uint32_t* __restrict__ block_lines, uint32_t cap_blocks,
                              FrameCounts* fc) {
    if (fc) n_steps = fc_count(fc, FC_STEPS, (uint32_t)n_steps, false);
    const uint32_t nb = (uint32_t)((n_steps + per_block - 1) / per_block);
    const uint64_t l0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * BL_LINES;
    if (l0 >= n_lines) return;
    uint32_t o[BL_LINES + 1];
    if (l0 + BL_LINES <= n_lines) {
        const uint4 v = *reinterpret_cast<const uint4*>(off + l0);
        o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
        o[BL_LINES] = off[l0 + BL_LINES];
    } else {
#pragma unroll
        for (int j = 0; j <= BL_LINES; j++) o[j] = l0 + j <= n_lines ? off[l0 + j] : 0u;
    }
#pragma unroll
    for (int j = 0; j < BL_LINES; j++) {
        const uint32_t l = (uint32_t)l0 + j;
        if (l >= n_lines) break;
        const uint32_t a = o[j], e = o[j + 1];
        if (a >= e) continue;
        for (uint32_t b = a / per_block; b < nb && (uint64_t)b * per_block < e; b++) {
            if ((uint64_t)b * per_block >= a) block_lines[b] = l;
            const uint64_t last = min((uint64_t)(b + 1) * per_block, n_steps) - 1;
            if (last >= a && last < e) block_lines[cap_blocks + 1 + b] = l;
        }
    }
}

// Every block rasterizes RASTER_ITEMS pixel steps per thread and stores its
// kept segments, in step order, at the start of its own run of
// 2 * RASTER_ITEMS * blockDim.x slots (a step yields at most two segments);
// run_count[block] receives how many.  No block waits on another: a later
// gather (fused with the sort's digit histogram) packs the runs.
template <int RENDER, int RASTER_ITEMS, bool SPARSE>
__global__ void __launch_bounds__(256) k_rasterize(const LineRec* __restrict__ recs, const uint32_t* __restrict__ off,
                                                   uint32_t n_lines, uint64_t n_steps, BatchGeom bg,
                                                   uint64_t* __restrict__ runs, uint32_t* __restrict__ run_count,
                                                   unsigned long long* __restrict__ produced, FrameCounts* fc,
                                                   const uint32_t* __restrict__ block_lines) {
    extern __shared__ __align__(16) uint64_t s_out[];  // 2 * RASTER_ITEMS * blockDim.x
    // The line offsets of the block's step range, staged once: two searches
    // over the whole offset array per block instead of one per thread.
    __shared__ uint32_t s_off[RASTER_LINE_STAGE + 1];
    if (fc) n_steps = fc_count(fc, FC_STEPS, (uint32_t)n_steps, blockIdx.x == 0 && threadIdx.x == 0);
    const uint64_t bs0 = (uint64_t)blockIdx.x * blockDim.x * RASTER_ITEMS;
    const uint64_t bs1 = min(bs0 + (uint64_t)blockDim.x * RASTER_ITEMS, n_steps);  // exclusive
    // lines l0..l1 hold the block's steps (from k_block_lines); off[l0 .. l1 + 1] go to s_off
    const uint32_t l0 = bs0 < n_steps ? block_lines[blockIdx.x] : 0u;
    const uint32_t nl = bs0 < n_steps ? block_lines[gridDim.x + 1 + blockIdx.x] - l0 + 1 : 0u;
    const bool staged = nl > 0 && nl <= RASTER_LINE_STAGE;
    if (staged)
        for (uint32_t q = threadIdx.x; q <= nl; q += blockDim.x) s_off[q] = off[l0 + q];
    // Full frames: the block's line records too, loaded together, into the
    // output stage (free until the steps are walked); the walk then reads
    // them from shared memory.  Incremental frames skip it: most of their
    // lines are empty.
    LineRec* s_recs = reinterpret_cast<LineRec*>(s_out);
    const bool recs_staged =
        !SPARSE && staged && nl * sizeof(LineRec) <= 2 * RASTER_ITEMS * blockDim.x * sizeof(uint64_t);
    if (recs_staged)
        for (uint32_t q = threadIdx.x; q < nl; q += blockDim.x) s_recs[q] = recs[l0 + q];
    __syncthreads();
    const uint64_t s0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * RASTER_ITEMS;
    // step k's segments at fixed positions 2k, 2k + 1 (constant indices keep
    // the array in registers); `kept` marks the positions that hold one
    uint64_t segs[2 * RASTER_ITEMS];
    uint32_t kept = 0;
    int n = 0, total = 0;
    if (s0 < n_steps) {
        uint32_t l;
        if (staged) {  // largest q with s_off[q] <= s0 (s_off[0] <= s0 < s_off[nl])
            uint32_t lo = 0, hi = nl;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if ((uint64_t)s_off[mid] <= s0) lo = mid;
                else hi = mid;
            }
            l = l0 + lo;
        } else if (SPARSE) {  // the block's lines l0..l1 do not fit the stage: search them in place
            uint32_t lo = l0, hi = l0 + nl;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if ((uint64_t)off[mid] <= s0) lo = mid;
                else hi = mid;
            }
            l = lo;
        } else {
            l = find_line(off, n_lines, s0);
        }
        uint32_t cur = staged ? s_off[l - l0] : off[l];
        uint32_t next = staged ? s_off[l - l0 + 1] : off[l + 1];
        LineRec rec = recs_staged ? s_recs[l - l0] : recs[l];
        uint32_t sc = rec.order_octant >> LINE_SCENE_SHIFT;
        SceneRaster sr{bg.scenes[sc].wide, bg.scenes[sc].rows, bg.scenes[sc].row_len, bg.scenes[sc].row_base};
#pragma unroll
        for (int k = 0; k < RASTER_ITEMS; k++) {
            uint64_t s = s0 + k;
            if (s < n_steps) {
                if (s >= next) {
                    // the next line with steps: usually the next line; lines of
                    // length 0 (culled) are passed over one by one, except in
                    // incremental frames (SPARSE: most lines belong to unchanged
                    // layers and have length 0), which search the block's range,
                    // off[l] <= s < off[l0 + nl]
                    l++;
                    cur = next;
                    next = staged ? s_off[l - l0 + 1] : off[l + 1];
                    while (!SPARSE && s >= next) {
                        l++;
                        cur = next;
                        next = staged ? s_off[l - l0 + 1] : off[l + 1];
                    }
                    if (SPARSE && s >= next) {
                        uint32_t lo = l + 1, hi = l0 + nl;
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if ((uint64_t)(staged ? s_off[mid - l0] : off[mid]) <= s) lo = mid;
                            else hi = mid;
                        }
                        l = lo;
                        cur = staged ? s_off[l - l0] : off[l];
                        next = staged ? s_off[l - l0 + 1] : off[l + 1];
                    }
                    rec = recs_staged ? s_recs[l - l0] : recs[l];
                    if ((rec.order_octant >> LINE_SCENE_SHIFT) != sc) {
                        sc = rec.order_octant >> LINE_SCENE_SHIFT;
                        sr = SceneRaster{bg.scenes[sc].wide, bg.scenes[sc].rows, bg.scenes[sc].row_len,
                                         bg.scenes[sc].row_base};
                    }
                }
                const uint32_t m = raster_step<RENDER>(sr, bg, rec, (int32_t)(s - cur), &segs[2 * k], total);
                kept |= m << (2 * k);
                n += __popc(m);
            }
        }
    }
    // block-wide exclusive scan of the per-thread counts
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t warp_tot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = n;
    uint32_t tinc = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t a = __shfl_up_sync(0xffffffffu, inc, o);
        uint32_t b = __shfl_up_sync(0xffffffffu, tinc, o);
        if (lane >= o) {
            inc += a;
            tinc += b;
        }
    }
    if (lane == 31) {
        warp_sums[warp] = inc;
        warp_tot[warp] = tinc;
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? warp_sums[lane] : 0, wt = lane < nw ? warp_tot[lane] : 0;
        uint32_t wi = w, wti = wt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t a = __shfl_up_sync(0xffffffffu, wi, o);
            uint32_t b = __shfl_up_sync(0xffffffffu, wti, o);
            if (lane >= o) {
                wi += a;
                wti += b;
            }
        }
        if (lane < nw) warp_sums[lane] = wi - w;
        if (lane == 31) {
            warp_tot[0] = wi;
            run_count[blockIdx.x] = wi;
            if (wti) atomicAdd(produced, (unsigned long long)wti);
        }
    }
    __syncthreads();
    const uint32_t local = warp_sums[warp] + inc - n;
    const uint32_t btotal = warp_tot[0];
#pragma unroll
    for (int q = 0; q < 2 * RASTER_ITEMS; q++)
        if ((kept >> q) & 1u) s_out[local + __popc(kept & ((1u << q) - 1u))] = segs[q];
    __syncthreads();
    uint64_t* dst = runs + (uint64_t)blockIdx.x * (2 * RASTER_ITEMS * blockDim.x);
    for (uint32_t i = threadIdx.x; i < btotal; i += blockDim.x) dst[i] = s_out[i];
}

// cassia_render's input (cassia/src/Cassia.h:25-41): reference CompactSegments
// in any order, NONE slots allowed.  Every thread takes IMPORT_ITEMS
// consecutive segments, drops NONE slots, segments of orders without a styling
// and segments outside the canvas, keys the rest as the rasterizer does, and
// the block stores them as one run (gathered with the sort's histogram).
constexpr int IMPORT_ITEMS = 8;

__global__ void __launch_bounds__(256) k_import_segments(const uint64_t* __restrict__ in, uint64_t n, BatchGeom bg,
                                                         uint64_t* __restrict__ runs, uint32_t* __restrict__ run_count,
                                                         unsigned long long* __restrict__ produced) {
    extern __shared__ __align__(16) uint64_t s_out[];  // IMPORT_ITEMS * blockDim.x
    const SceneDesc& sc = bg.scenes[0];
    const SceneRaster sr{sc.wide, sc.rows, sc.row_len, sc.row_base};
    const uint64_t s0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * IMPORT_ITEMS;
    uint64_t keys[IMPORT_ITEMS];  // segment k's key at slot k (constant indices: registers)
    uint32_t mask = 0;
    int kept = 0, real = 0;
#pragma unroll
    for (int k = 0; k < IMPORT_ITEMS; k++) {
        const uint64_t i = s0 + k;
        if (i >= n) break;
        const uint64_t v = in[i];
        SegFields f;
        uint32_t layer;
        if (sc.wide) {  // tile_j:12 tile_i:13 layer:17 (no NONE slots)
            f.tj = (int32_t)((v >> 52) & 0xFFFu);
            f.tis = (int32_t)((v >> 39) & 0x1FFFu);
            layer = (uint32_t)((v >> 22) & 0x1FFFFu);
        } else {  // is_none:1 tile_j:12 tile_i:13 layer:16
            if (v >> 63) continue;
            f.tj = (int32_t)((v >> 51) & 0xFFFu);
            f.tis = (int32_t)((v >> 38) & 0x1FFFu);
            layer = (uint32_t)((v >> 22) & 0xFFFFu);
        }
        f.low = (uint32_t)(v & 0x3FFFFFu);
        real++;
        uint64_t key;
        if (layer < sc.n_orders && render_key(sr, bg, layer, f, key)) {
            keys[k] = key;
            mask |= 1u << k;
            kept++;
        }
    }
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t warp_tot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = kept, tinc = real;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, inc, o);
        const uint32_t b = __shfl_up_sync(0xffffffffu, tinc, o);
        if (lane >= o) {
            inc += a;
            tinc += b;
        }
    }
    if (lane == 31) {
        warp_sums[warp] = inc;
        warp_tot[warp] = tinc;
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < nw ? warp_sums[lane] : 0, wt = lane < nw ? warp_tot[lane] : 0;
        uint32_t wi = w, wti = wt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t a = __shfl_up_sync(0xffffffffu, wi, o);
            const uint32_t b = __shfl_up_sync(0xffffffffu, wti, o);
            if (lane >= o) {
                wi += a;
                wti += b;
            }
        }
        if (lane < nw) warp_sums[lane] = wi - w;
        if (lane == 31) {
            warp_tot[0] = wi;
            run_count[blockIdx.x] = wi;
            if (wti) atomicAdd(produced, (unsigned long long)wti);
        }
    }
    __syncthreads();
    const uint32_t local = warp_sums[warp] + inc - kept;
    const uint32_t btotal = warp_tot[0];
#pragma unroll
    for (int q = 0; q < IMPORT_ITEMS; q++)
        if ((mask >> q) & 1u) s_out[local + __popc(mask & ((1u << q) - 1u))] = keys[q];
    __syncthreads();
    uint64_t* dst = runs + (uint64_t)blockIdx.x * (IMPORT_ITEMS * blockDim.x);
    for (uint32_t i = threadIdx.x; i < btotal; i += blockDim.x) dst[i] = s_out[i];
}

__global__ void k_keep_flags(const uint32_t* __restrict__ lids, uint32_t n, const LayerRec* __restrict__ layers,
                             uint32_t n_layer_recs, uint32_t* __restrict__ flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t lid = lids[i];
    uint32_t f = lid < n_layer_recs ? layers[lid].flags : 0u;
    flags[i] = ((f & LAYER_PRESENT) && (f & LAYER_ENABLED)) ? 1u : 0u;
}

__global__ void k_scatter_lines(const float* __restrict__ a, const float* __restrict__ b, const float* __restrict__ c,
                                const float* __restrict__ d, const uint32_t* __restrict__ lid_in, uint32_t n,
                                const uint32_t* __restrict__ flags, const uint32_t* __restrict__ off,
                                float* __restrict__ oa, float* __restrict__ ob, float* __restrict__ oc,
                                float* __restrict__ od, uint32_t* __restrict__ lid_out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flags[i]) return;
    uint32_t o = off[i];
    oa[o] = a[i];
    ob[o] = b[i];
    oc[o] = c[i];
    od[o] = d[i];
    lid_out[o] = lid_in[i];
}

}  // namespace

cudaError_t launch_flatten(int write, const uint32_t* kinds, const float* points, const uint64_t* cmd_off,
                           const uint64_t* pt_off, const float* transforms9, const uint8_t* has_t,
                           const uint32_t* path_layer, uint32_t n_paths, uint32_t* counts, const uint32_t* out_off,
                           float* p0x, float* p0y, float* p1x, float* p1y, uint32_t* lids, cudaStream_t st) {
    if (n_paths == 0) return cudaSuccess;
    count_launches(1);
    k_flatten<<<(n_paths + 127) / 128, 128, 0, st>>>(write, kinds, points, cmd_off, pt_off, transforms9, has_t,
                                                     path_layer, n_paths, counts, out_off, p0x, p0y, p1x, p1y, lids);
    return cudaGetLastError();
}

cudaError_t launch_build_lines(const BatchGeom& bg, int cull, LineRec* recs, uint32_t* lengths, cudaStream_t st,
                               uint32_t* order_flag) {
    if (bg.total_lines == 0) return cudaSuccess;
    if (bg.n_scenes > MAX_SMEM_SCENES) return cudaErrorInvalidValue;
    count_launches(1);
    k_build_lines<<<(uint32_t)((bg.total_lines + 255) / 256), 256, 0, st>>>(bg, cull, recs, lengths, order_flag);
    return cudaGetLastError();
}

cudaError_t launch_rasterize(int render, const BatchGeom& bg, const LineRec* recs, const uint32_t* step_off,
                             uint32_t n_lines, uint64_t n_steps, uint32_t block, uint32_t items, uint64_t* runs,
                             uint32_t* run_count, unsigned long long* produced, cudaStream_t st,
                             FrameCounts* fc, bool sparse, uint32_t* block_lines) {
    if (n_steps == 0) return cudaSuccess;
    if (fc && n_steps >= (1ull << 32)) return cudaErrorInvalidValue;
    if (block == 0 || block % 32 || block > 256 || (items != 4 && items != 8)) return cudaErrorInvalidValue;
    const uint32_t grid = raster_grid(n_steps, block, items);
    const size_t smem = (size_t)raster_run_slots(block, items) * sizeof(uint64_t);
    count_launches(2);
    if (n_lines > 0)
        k_block_lines<<<(n_lines + 256 * BL_LINES - 1) / (256 * BL_LINES), 256, 0, st>>>(
            step_off, n_lines, n_steps, block * items, block_lines, grid, fc);
#define CGB_RASTER(R, I, S)                                                                                   \
    k_rasterize<R, I, S><<<grid, block, smem, st>>>(recs, step_off, n_lines, n_steps, bg, runs, run_count, produced, \
                                                    fc, block_lines)
    if (render && sparse) {
        if (items == 4) CGB_RASTER(1, 4, true);
        else CGB_RASTER(1, 8, true);
    } else if (render) {
        if (items == 4) CGB_RASTER(1, 4, false);
        else CGB_RASTER(1, 8, false);
    } else {
        if (items == 4) CGB_RASTER(0, 4, false);
        else CGB_RASTER(0, 8, false);
    }
#undef CGB_RASTER
    return cudaGetLastError();
}

uint32_t raster_run_slots(uint32_t block, uint32_t items) { return 2 * items * block; }

uint32_t raster_grid(uint64_t n_steps, uint32_t block, uint32_t items) {
    const uint64_t per_block = (uint64_t)block * items;
    return (uint32_t)((n_steps + per_block - 1) / per_block);
}

cudaError_t launch_import_segments(const uint64_t* segs, uint64_t n, const BatchGeom& bg, uint64_t* runs,
                                   uint32_t* run_count, unsigned long long* produced, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t block = 256;
    const uint32_t grid = import_grid(n);
    count_launches(1);
    k_import_segments<<<grid, block, (size_t)IMPORT_ITEMS * block * sizeof(uint64_t), st>>>(segs, n, bg, runs,
                                                                                         run_count, produced);
    return cudaGetLastError();
}

uint32_t import_grid(uint64_t n) { return (uint32_t)((n + 256 * IMPORT_ITEMS - 1) / (256 * IMPORT_ITEMS)); }
uint32_t import_run_slots() { return 256 * IMPORT_ITEMS; }

// Line copies for cgb_insert_layer_copies: one thread per copied line finds
// its run by a binary search over the run offsets.
__global__ void k_copy_lines(const float* __restrict__ sx0, const float* __restrict__ sy0,
                             const float* __restrict__ sx1, const float* __restrict__ sy1,
                             const uint64_t* __restrict__ src_first, const uint64_t* __restrict__ dst_off,
                             const uint32_t* __restrict__ dst_ids, uint32_t n, uint64_t total, float* __restrict__ dx0,
                             float* __restrict__ dy0, float* __restrict__ dx1, float* __restrict__ dy1,
                             uint32_t* __restrict__ dlid) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < total;
         j += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n;  // the last run k with dst_off[k] <= j
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (dst_off[mid] <= j) lo = mid;
            else hi = mid;
        }
        const uint64_t s = src_first[lo] + (j - dst_off[lo]);
        dx0[j] = sx0[s];
        dy0[j] = sy0[s];
        dx1[j] = sx1[s];
        dy1[j] = sy1[s];
        dlid[j] = dst_ids[lo];
    }
}

cudaError_t launch_copy_lines(const float* const src4[4], const uint64_t* src_first, const uint64_t* dst_off,
                              const uint32_t* dst_ids, uint32_t n, uint64_t total, float* const dst4[4],
                              uint32_t* dst_lids, cudaStream_t st) {
    if (total == 0 || n == 0) return cudaSuccess;
    const uint64_t blocks = std::min<uint64_t>((total + 255) / 256, 4096);
    count_launches(1);
    k_copy_lines<<<(uint32_t)blocks, 256, 0, st>>>(src4[0], src4[1], src4[2], src4[3], src_first, dst_off, dst_ids,
                                                   n, total, dst4[0], dst4[1], dst4[2], dst4[3], dst_lids);
    return cudaGetLastError();
}

cudaError_t launch_compact_lines(const float* in4[4], const uint32_t* lid_in, uint32_t n, const LayerRec* layers,
                                 uint32_t n_layer_recs, float* out4[4], uint32_t* lid_out, uint32_t* flags,
                                 uint32_t* offsets, Scratch* s, cudaStream_t st, uint32_t* n_out_host) {
    if (n == 0) {
        *n_out_host = 0;
        return cudaSuccess;
    }
    count_launches(2);
    k_keep_flags<<<(n + 255) / 256, 256, 0, st>>>(lid_in, n, layers, n_layer_recs, flags);
    uint64_t total = 0;
    cudaError_t e = scan_u32(flags, offsets, n, s, st, &total);
    if (e != cudaSuccess) return e;
    k_scatter_lines<<<(n + 255) / 256, 256, 0, st>>>(in4[0], in4[1], in4[2], in4[3], lid_in, n, flags, offsets,
                                                     out4[0], out4[1], out4[2], out4[3], lid_out);
    *n_out_host = (uint32_t)total;
    return cudaGetLastError();
}

}  // namespace cgb
