// CPU restatement of Kangz/cassia's surpass + mold rasterization path.
//
// TEST INFRASTRUCTURE ONLY: the correctness oracle and the timed CPU baseline
// for the GPU implementation.  Never linked into the product.
//
// Parity status: the reference is Rust and cannot be built where this file is
// compiled (no cargo/rustc, no vendored crates), so this restatement is pinned
// to the reference's own known-answer tests (segment.rs, style.rs, path/mod.rs,
// composition.rs render tests, the commented rasterizer area/cover tables) in
// tests/test_oracle_kats.py.
//
// Compile with -ffp-contract=off and without -ffast-math: Rust never contracts
// a*b+c, and every `mul_add` of the reference is an explicit std::fma here.
// Float -> integer conversions follow Rust's saturating `as` (NaN -> 0), and
// f32::round is round-half-away-from-zero (std::round).  Integer arithmetic
// wraps as Rust release builds do.
//
// Deviations (the reference painter cannot run at HEAD with 8x8 tiles):
//   D1  The painter decodes tile_i as (stored - 256).  The rasterizer stores
//       max(ti, -1) + 256 (surpass/src/rasterizer/mod.rs:188) for cassia's WGSL
//       (cassia/src/CommonWGSL.cpp:35,52), but the CPU painter never removes
//       the offset (surpass/src/painter/mod.rs:517-566).  The left-of-canvas
//       run (decoded -1) is at the head of each row in sort order and is
//       accumulated as the row's initial cover carry.  Stored values that
//       wrapped the 13-bit field (x >= 30,712 px) decode below -1 and, like
//       tiles right of the canvas, are never painted.
//   D2  Cover is 8 x i8 (one lane per tile row); Painter covers are 9x8 i8
//       and areas 8x8 i16 (fixes painter/mod.rs:150, 209-210, 269 which size
//       them for 16-row tiles and evaluate to zero-length arrays).  Cover is
//       a single 8-lane vector, so is_full's any-over-vectors
//       (painter/mod.rs:183-187) reduces to "every row", which is also what
//       the reference computes at its working 16-row tile size.
//   D3  compute_areas and the running column cover take all 8 rows of a pixel
//       column (fixes the 16-lane cols! slicing, painter/mod.rs:29-51, 310-313,
//       347-362).
//   D4  Per-layer affine transforms may scale beyond 1 when requested: they are
//       stored in surpass::Layer::affine_transform (surpass/src/layer.rs:8),
//       bypassing mold's check (mold/src/layer.rs:186-190).
//   D5  Widened segment format for more than 65,536 layer orders: the is_none
//       bit becomes layer bit 16 (tile_j:12 tile_i:13 layer:17 then the
//       reference's low 22 bits); NONE slots are never materialized.
// Other restatement choices:
//   - IdSet hands out the lowest free id (the reference's first pick depends on
//     FxHashMap iteration order, mold/src/layer.rs:45-47).
//   - orders_to_layers is filled in ascending layer-id order, so with duplicate
//     orders the highest layer id wins (the reference iterates an FxHashMap).
//   - Style::fill_rule is unused by the reference painter; props carry only
//     Props::fill_rule.

#include "surpass_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace orc {

// surpass/src/lib.rs:18-33
constexpr int32_t PIXEL_WIDTH = 16;
constexpr int32_t PIXEL_SHIFT = 4;
constexpr int32_t PIXEL_MASK = 15;
constexpr int32_t TILE_WIDTH = 8;
constexpr int32_t TILE_HEIGHT = 8;
constexpr int32_t TILE_SHIFT = 3;
constexpr int32_t TILE_MASK = 7;
constexpr uint64_t NONE = 1ull << 63;  // raster_segment.rs:11

// ---------------------------------------------------------------------------
// numerics (Rust semantics)
// ---------------------------------------------------------------------------

static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
static inline int32_t wshl(int32_t a, int s) { return (int32_t)((uint32_t)a << s); }
static inline int32_t wabs(int32_t a) { return a < 0 ? wsub(0, a) : a; }
static inline int8_t abs8(int8_t v) { return v < 0 ? (int8_t)(uint8_t)(0u - (uint8_t)v) : v; }

// Rust `f as i32`: toward zero, saturating, NaN -> 0.
static inline int32_t f2i32(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v < -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
// Rust `f as u8`.
static inline uint8_t f2u8(float v) {
    if (std::isnan(v) || v <= 0.0f) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}
// Rust `f as usize`.
static inline uint64_t f2usize(float v) {
    if (std::isnan(v) || v <= 0.0f) return 0;
    if (v >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)v;
}
// Rust f32::min / f32::max: a NaN operand yields the other operand.
static inline float fmin_r(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return a < b ? a : b;
}
static inline float fmax_r(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return a > b ? a : b;
}
static inline float clamp_r(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}
static inline float fbits_or(float a, float b) {
    uint32_t x, y;
    std::memcpy(&x, &a, 4);
    std::memcpy(&y, &b, 4);
    x |= y;
    float r;
    std::memcpy(&r, &x, 4);
    return r;
}

// surpass/src/segment.rs:13-16
static inline int32_t to_sub_pixel(float v) {
    return f2i32(std::fma(v, (float)PIXEL_WIDTH, std::copysign(0.5f, v)));
}

// ---------------------------------------------------------------------------
// mold path flattening (mold/src/path/segments.rs, transform.rs, point.rs)
// ---------------------------------------------------------------------------

struct Pt {
    float x, y;
};
static inline Pt pmul(Pt p, float s) { return {p.x * s, p.y * s}; }
static inline Pt padd(Pt a, Pt b) { return {a.x + b.x, a.y + b.y}; }
// Point::lerp (mold/src/point.rs:30-32)
static inline Pt plerp(float t, Pt p0, Pt p1) { return padd(pmul(p0, 1.0f - t), pmul(p1, t)); }
// Point::approx_eq (point.rs:34-36)
static inline bool approx_eq(Pt a, Pt b) {
    const float eps = 1.1920929e-7f;
    return std::fabs(a.x - b.x) < eps && std::fabs(a.y - b.y) < eps;
}
// Point::from_weighted (point.rs:38-40)
static inline Pt from_weighted(float x, float y, float w) {
    float r = 1.0f / w;
    return {x * r, y * r};
}
// segments.rs:15-17
static inline float lerp1(float t, float a, float b) { return a * (1.0f - t) + b * t; }

// PathCommand (mold/src/path/mod.rs:13-21) in the stored form: rational points
// are pre-weighted (p * w, w) as Path::rat_quad / rat_cubic store them.
struct Cmd {
    uint32_t kind;
    Pt p[4];
    float w[4];
};

static int cmd_floats(uint32_t kind) {
    switch (kind) {
        case CGB_CMD_LINE: return 4;
        case CGB_CMD_QUAD: return 6;
        case CGB_CMD_RAT_QUAD: return 9;
        case CGB_CMD_CUBIC: return 8;
        case CGB_CMD_RAT_CUBIC: return 12;
        case CGB_CMD_CLOSE: return 0;
        default: return -1;
    }
}

// Decodes the ABI float layout into stored commands (Path methods,
// mold/src/path/mod.rs:53-170).  Returns false on an unknown kind.
static bool decode_cmds(const uint32_t* kinds, size_t n, const float* pts, std::vector<Cmd>& out) {
    out.clear();
    size_t o = 0;
    for (size_t i = 0; i < n; i++) {
        Cmd c{};
        c.kind = kinds[i];
        switch (c.kind) {
            case CGB_CMD_LINE:
                for (int k = 0; k < 2; k++) c.p[k] = {pts[o + 2 * k], pts[o + 2 * k + 1]};
                o += 4;
                break;
            case CGB_CMD_QUAD:
                for (int k = 0; k < 3; k++) c.p[k] = {pts[o + 2 * k], pts[o + 2 * k + 1]};
                o += 6;
                break;
            case CGB_CMD_CUBIC:
                for (int k = 0; k < 4; k++) c.p[k] = {pts[o + 2 * k], pts[o + 2 * k + 1]};
                o += 8;
                break;
            case CGB_CMD_RAT_QUAD:
            case CGB_CMD_RAT_CUBIC: {
                int np = c.kind == CGB_CMD_RAT_QUAD ? 3 : 4;
                for (int k = 0; k < np; k++) {
                    float x = pts[o + 3 * k], y = pts[o + 3 * k + 1], w = pts[o + 3 * k + 2];
                    c.p[k] = pmul(Pt{x, y}, w);  // (p0.0 * p0.1, p0.1)
                    c.w[k] = w;
                }
                o += 3 * np;
                break;
            }
            case CGB_CMD_CLOSE: break;
            default: return false;
        }
        out.push_back(c);
    }
    return true;
}

// Transform (mold/src/path/transform.rs:24-94)
struct Transform {
    float t[9];
    bool is_perspective;
    explicit Transform(const float* t9) {
        float r = 1.0f / t9[8];
        for (int i = 0; i < 9; i++) t[i] = t9[i] * r;
        const float eps = 1.1920929e-7f;
        is_perspective = std::fabs(t[6]) > eps || std::fabs(t[7]) > eps;
    }
    void full(float x, float y, float w, float o[3]) const {
        o[0] = t[0] * x + t[1] * y + t[2] * w;
        o[1] = t[3] * x + t[4] * y + t[5] * w;
        o[2] = t[6] * x + t[7] * y + t[8] * w;
    }
    Pt simple(Pt p) const { return {t[0] * p.x + t[1] * p.y + t[2], t[3] * p.x + t[4] * p.y + t[5]}; }
    Cmd apply(const Cmd& c) const {
        Cmd r = c;
        int np = 0;
        switch (c.kind) {
            case CGB_CMD_LINE: np = 2; break;
            case CGB_CMD_QUAD: np = 3; break;
            case CGB_CMD_CUBIC: np = 4; break;
            case CGB_CMD_RAT_QUAD: np = 3; break;
            case CGB_CMD_RAT_CUBIC: np = 4; break;
            default: return r;
        }
        if (c.kind == CGB_CMD_LINE) {
            for (int k = 0; k < 2; k++) {
                if (!is_perspective) {
                    r.p[k] = simple(c.p[k]);
                } else {
                    float o[3];
                    full(c.p[k].x, c.p[k].y, 1.0f, o);
                    r.p[k] = from_weighted(o[0], o[1], o[2]);
                }
            }
            return r;
        }
        bool rational = c.kind == CGB_CMD_RAT_QUAD || c.kind == CGB_CMD_RAT_CUBIC;
        if (!rational && !is_perspective) {
            for (int k = 0; k < np; k++) r.p[k] = simple(c.p[k]);
            return r;
        }
        // full!: Quad/Cubic become RatQuad/RatCubic with unit weights.
        for (int k = 0; k < np; k++) {
            float w = rational ? c.w[k] : 1.0f;
            float o[3];
            full(c.p[k].x, c.p[k].y, w, o);
            r.p[k] = {o[0], o[1]};
            r.w[k] = o[2];
        }
        if (c.kind == CGB_CMD_QUAD) r.kind = CGB_CMD_RAT_QUAD;
        if (c.kind == CGB_CMD_CUBIC) r.kind = CGB_CMD_RAT_CUBIC;
        return r;
    }
};

struct Seg4 {
    float x0, y0, x1, y1;
};

// PathSegments (mold/src/path/segments.rs:39-263)
struct PathSegments {
    const Cmd* cmds;
    size_t n;
    const Transform* transform;
    bool has_state = false;
    uint64_t subdivisions = 0;
    float t = 0, increment = 0;
    Pt point{};
    bool has_last = false, has_closing = false;
    Pt last_point{}, closing_point{};

    static constexpr float PIXEL_ACCURACY = 0.5f / (float)PIXEL_WIDTH;  // segments.rs:13

    Cmd first() const { return transform ? transform->apply(cmds[0]) : cmds[0]; }

    Seg4 line(Pt a, Pt b) {  // segments.rs:106-114
        if (!has_closing) {
            has_closing = true;
            closing_point = a;
        }
        has_last = true;
        last_point = b;
        return {a.x, a.y, b.x, b.y};
    }

    static Pt eval(const Cmd& c, float tt) {
        switch (c.kind) {
            case CGB_CMD_QUAD:
                return plerp(tt, plerp(tt, c.p[0], c.p[1]), plerp(tt, c.p[1], c.p[2]));
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
            case CGB_CMD_RAT_CUBIC: {
                Pt a = plerp(tt, plerp(tt, c.p[0], c.p[1]), plerp(tt, c.p[1], c.p[2]));
                Pt b = plerp(tt, plerp(tt, c.p[1], c.p[2]), plerp(tt, c.p[2], c.p[3]));
                Pt bz = plerp(tt, a, b);
                float wa = lerp1(tt, lerp1(tt, c.w[0], c.w[1]), lerp1(tt, c.w[1], c.w[2]));
                float wb = lerp1(tt, lerp1(tt, c.w[1], c.w[2]), lerp1(tt, c.w[2], c.w[3]));
                float w = lerp1(tt, wa, wb);
                return pmul(bz, 1.0f / w);
            }
        }
        return {0, 0};
    }

    // next_segment (segments.rs:116-157), with subdivisions (:51-72) inlined.
    Seg4 next_segment(const Cmd& c, Pt first_p, Pt last_p, float dev_x, float dev_y) {
        if (!has_state) {
            float dev2 = dev_x * dev_x + dev_y * dev_y;
            if (dev2 < PIXEL_ACCURACY) return line(first_p, last_p);
            uint64_t count = f2usize(std::ceil(std::sqrt(std::sqrt(dev2) * 2.0f / (8.0f * PIXEL_ACCURACY))));
            uint64_t subs = std::max<uint64_t>(count, 1) - 1;
            if (subs == 0) return line(first_p, last_p);
            has_state = true;
            subdivisions = subs;
            increment = 1.0f / (float)subs;
            t = 0.0f;
            point = first_p;
        }
        if (subdivisions == 1) {
            has_state = false;
            return line(point, last_p);
        }
        t += increment;
        Pt np = eval(c, t);
        Seg4 s = line(point, np);
        point = np;
        subdivisions -= 1;
        return s;
    }

    static float dev3(float a, float b, float c) { return a + c - 2.0f * b; }
    static float dev4(float a, float b, float c, float d) {
        return fmax_r(std::fabs(a + c - 2.0f * b), std::fabs(b + d - 2.0f * c));
    }

    // Iterator::next (segments.rs:233-262)
    bool next(Seg4& out) {
        while (n > 0) {
            Cmd c = first();
            if (c.kind == CGB_CMD_CLOSE) {
                cmds++;
                n--;
                // close (segments.rs:208-223)
                if (has_closing && has_last) {
                    bool emit = !approx_eq(closing_point, last_point);
                    Seg4 s{};
                    if (emit) s = line(last_point, closing_point);
                    has_closing = false;
                    if (emit) {
                        out = s;
                        return true;
                    }
                }
                continue;
            }
            Seg4 s{};
            switch (c.kind) {
                case CGB_CMD_LINE: s = line(c.p[0], c.p[1]); break;
                case CGB_CMD_QUAD:
                    s = next_segment(c, c.p[0], c.p[2], dev3(c.p[0].x, c.p[1].x, c.p[2].x),
                                     dev3(c.p[0].y, c.p[1].y, c.p[2].y));
                    break;
                case CGB_CMD_CUBIC:
                    s = next_segment(c, c.p[0], c.p[3], dev4(c.p[0].x, c.p[1].x, c.p[2].x, c.p[3].x),
                                     dev4(c.p[0].y, c.p[1].y, c.p[2].y, c.p[3].y));
                    break;
                case CGB_CMD_RAT_QUAD: {
                    Pt p0 = from_weighted(c.p[0].x, c.p[0].y, c.w[0]);
                    Pt p1 = from_weighted(c.p[1].x, c.p[1].y, c.w[1]);
                    Pt p2 = from_weighted(c.p[2].x, c.p[2].y, c.w[2]);
                    s = next_segment(c, p0, p2, dev3(p0.x, p1.x, p2.x), dev3(p0.y, p1.y, p2.y));
                    break;
                }
                case CGB_CMD_RAT_CUBIC: {
                    Pt p0 = from_weighted(c.p[0].x, c.p[0].y, c.w[0]);
                    Pt p1 = from_weighted(c.p[1].x, c.p[1].y, c.w[1]);
                    Pt p2 = from_weighted(c.p[2].x, c.p[2].y, c.w[2]);
                    Pt p3 = from_weighted(c.p[3].x, c.p[3].y, c.w[3]);
                    s = next_segment(c, p0, p3, dev4(p0.x, p1.x, p2.x, p3.x),
                                     dev4(p0.y, p1.y, p2.y, p3.y));
                    break;
                }
            }
            if (!has_state) {
                cmds++;
                n--;
            }
            out = s;
            return true;
        }
        return false;
    }
};

static void flatten(const std::vector<Cmd>& cmds, const float* t9, std::vector<Seg4>& out) {
    std::unique_ptr<Transform> tr;
    if (t9) tr.reset(new Transform(t9));
    PathSegments ps{cmds.data(), cmds.size(), tr.get()};
    Seg4 s;
    while (ps.next(s)) out.push_back(s);
}

// ---------------------------------------------------------------------------
// surpass LinesBuilder::build (surpass/src/segment.rs:91-237)
// ---------------------------------------------------------------------------

struct SLayer {  // surpass::Layer (surpass/src/layer.rs:5-20)
    bool is_enabled = true;
    bool has_transform = false;
    float transform[6] = {1, 0, 0, 1, 0, 0};
    bool has_order = false;
    uint32_t order = 0;
};

struct LineParams {
    uint32_t order = 0;
    int32_t start = 0;
    float start_f32 = 0, end_f32 = 0;
    uint32_t length = 0;
    float slope = 0, slope_recip = 0, py_slope_px = 0, px_slope_recip_py = 0;
    uint8_t octant = 0;
};

static LineParams build_line(float p0x, float p0y, float p1x, float p1y, uint32_t layer_id,
                             const SLayer* layer, const float* default_transform) {
    LineParams r;
    if (layer && !layer->is_enabled) return r;
    uint32_t order = (layer && layer->has_order) ? layer->order : layer_id;
    const float* tr = (layer && layer->has_transform) ? layer->transform : default_transform;
    if (tr) {
        float a = std::fma(tr[0], p0x, std::fma(tr[1], p0y, tr[4]));
        float b = std::fma(tr[2], p0x, std::fma(tr[3], p0y, tr[5]));
        float c = std::fma(tr[0], p1x, std::fma(tr[1], p1y, tr[4]));
        float d = std::fma(tr[2], p1x, std::fma(tr[3], p1y, tr[5]));
        p0x = a;
        p0y = b;
        p1x = c;
        p1y = d;
    }
    int32_t p0x_sub = to_sub_pixel(p0x), p0y_sub = to_sub_pixel(p0y);
    int32_t p1x_sub = to_sub_pixel(p1x), p1y_sub = to_sub_pixel(p1y);
    if (p0y_sub == p1y_sub) return r;
    int32_t dx = wsub(p1x_sub, p0x_sub), dy = wsub(p1y_sub, p0y_sub);
    bool dx_dy = wabs(dx) > wabs(dy);
    bool sum_0 = wadd(dx, dy) > 0 || (dx == wsub(0, dy) && dx < dy);
    int32_t start_sub, end_sub;
    if (sum_0 && dx_dy) {
        start_sub = p0x_sub;
        end_sub = p1x_sub;
    } else if (sum_0) {
        start_sub = p0y_sub;
        end_sub = p1y_sub;
    } else if (dx_dy) {
        start_sub = p1x_sub;
        end_sub = p0x_sub;
    } else {
        start_sub = p1y_sub;
        end_sub = p0y_sub;
    }
    int32_t start = start_sub >> PIXEL_SHIFT;
    int32_t end = (end_sub & PIXEL_MASK) == 0 ? end_sub >> PIXEL_SHIFT : (end_sub >> PIXEL_SHIFT) + 1;
    r.length = (uint32_t)wsub(end, start);
    const float rcp = 1.0f / (float)PIXEL_WIDTH;
    r.start_f32 = (float)start_sub * rcp;
    r.end_f32 = (float)end_sub * rcp;
    float fp0x = (float)p0x_sub * rcp, fp0y = (float)p0y_sub * rcp;
    float px = dx_dy ? fp0x : fp0y, py = dx_dy ? fp0y : fp0x;
    float slope = dx_dy ? (float)dy / (float)dx : (float)dx / (float)dy;
    float slope_recip = 1.0f / slope;
    r.order = order;
    r.start = start;
    r.slope = slope;
    r.slope_recip = slope_recip;
    r.py_slope_px = std::fma(slope, -px, py);
    r.px_slope_recip_py = std::fma(slope_recip, -py, px);
    bool xp = dx > 0, yp = dy > 0;
    uint8_t oct;
    if (dx_dy && xp && yp) oct = 0;
    else if (!dx_dy && xp && yp) oct = 1;
    else if (!dx_dy && !xp && yp) oct = 2;
    else if (dx_dy && !xp && yp) oct = 3;
    else if (dx_dy && !xp && !yp) oct = 4;
    else if (!dx_dy && !xp && !yp) oct = 5;
    else if (!dx_dy && xp && !yp) oct = 6;
    else oct = 7;
    r.octant = oct;
    return r;
}

// ---------------------------------------------------------------------------
// CompactSegment (surpass/src/rasterizer/raster_segment.rs:142-160) and the
// D5 widened layout.
// ---------------------------------------------------------------------------

struct Fmt {
    bool wide;
    uint64_t pack(int32_t tile_j, int32_t tile_i_stored, uint32_t layer, uint32_t ty, uint32_t tx,
                  int32_t area, int32_t cover) const {
        uint64_t v = 0;
        if (!wide) {
            v = 0;  // is_none
            v = (v << 12) | ((uint64_t)(int64_t)tile_j & 0xFFF);
            v = (v << 13) | ((uint64_t)(int64_t)tile_i_stored & 0x1FFF);
            v = (v << 16) | ((uint64_t)layer & 0xFFFF);
        } else {
            v = ((uint64_t)(int64_t)tile_j & 0xFFF);
            v = (v << 13) | ((uint64_t)(int64_t)tile_i_stored & 0x1FFF);
            v = (v << 17) | ((uint64_t)layer & 0x1FFFF);
        }
        v = (v << 3) | (ty & 7);
        v = (v << 3) | (tx & 7);
        v = (v << 10) | ((uint64_t)(int64_t)area & 0x3FF);
        v = (v << 6) | ((uint64_t)(int64_t)cover & 0x3F);
        return v;
    }
    static int32_t sext(uint64_t v, int bits) {
        uint64_t m = 1ull << (bits - 1);
        v &= (1ull << bits) - 1;
        return (int32_t)(int64_t)((v ^ m) - m);
    }
    int32_t tile_j(uint64_t s) const { return sext(s >> (wide ? 52 : 51), 12); }
    int32_t tile_i_stored(uint64_t s) const { return sext(s >> (wide ? 39 : 38), 13); }
    uint32_t layer(uint64_t s) const { return wide ? (uint32_t)((s >> 22) & 0x1FFFF) : (uint32_t)((s >> 22) & 0xFFFF); }
    static uint32_t tile_y(uint64_t s) { return (uint32_t)(s >> 19) & 7; }
    static uint32_t tile_x(uint64_t s) { return (uint32_t)(s >> 16) & 7; }
    static int32_t area(uint64_t s) { return sext(s >> 6, 10); }
    static int32_t cover(uint64_t s) { return sext(s, 6); }
    // D1: painter-side tile column.
    int32_t tile_i(uint64_t s) const { return tile_i_stored(s) - 256; }
};

// tiles (rasterizer/mod.rs:134-147)
static inline void tiles(int32_t bx, int32_t by, uint8_t oct, int32_t& ti, int32_t& tj, uint32_t& tx,
                         uint32_t& ty) {
    if (oct == 1 || oct == 2 || oct == 5 || oct == 6) std::swap(bx, by);
    ti = (int16_t)(bx >> TILE_SHIFT);
    tj = (int16_t)(by >> TILE_SHIFT);
    tx = (uint32_t)(bx & TILE_MASK);
    ty = (uint32_t)(by & TILE_MASK);
}

// area_cover (rasterizer/mod.rs:149-172)
static inline void area_cover(int32_t x0, int32_t x1, int32_t y0, int32_t y1, uint8_t oct, int32_t& area,
                              int32_t& cover) {
    int32_t a0 = x0, a1 = x1, b0 = y0, b1 = y1;
    switch (oct) {
        case 0: break;
        case 1: a0 = y0; a1 = y1; b0 = x0; b1 = x1; break;
        case 2: a0 = y1; a1 = y0; b0 = x0; b1 = x1; break;
        case 3: b0 = y1; b1 = y0; break;
        case 4: b0 = y1; b1 = y0; break;
        case 5: a0 = y0; a1 = y1; b0 = x1; b1 = x0; break;
        case 6: a0 = y1; a1 = y0; b0 = x1; b1 = x0; break;
        case 7: break;
    }
    int32_t border = wadd(a0 & ~PIXEL_MASK, PIXEL_WIDTH);
    int32_t height = wsub(b1, b0);
    int16_t triangle = (int16_t)(wmul(height, wsub(a1, a0)) / 2);
    int16_t rectangle = (int16_t)wmul(height, wsub(border, a1));
    area = (int16_t)(uint16_t)((uint16_t)triangle + (uint16_t)rectangle);
    cover = (int8_t)height;
}

static inline uint64_t make_segment(const Fmt& f, uint32_t layer, int32_t x0, int32_t x1, int32_t y0,
                                    int32_t y1, int32_t bx, int32_t by, uint8_t oct) {
    int32_t ti, tj, area, cover;
    uint32_t tx, ty;
    tiles(bx, by, oct, ti, tj, tx, ty);
    area_cover(x0, x1, y0, y1, oct, area, cover);
    int16_t tis = (int16_t)(uint16_t)((uint16_t)(int16_t)std::max(ti, -1) + 256u);
    return f.pack(tj, tis, layer, ty, tx, area, cover);
}

static inline bool intersects_y_border(int32_t y0, int32_t y1) {  // rasterizer/mod.rs:127-132
    return (y0 & PIXEL_MASK) != 0 && (y1 & PIXEL_MASK) != 0 && (y0 >> PIXEL_SHIFT) != (y1 >> PIXEL_SHIFT);
}

// One pixel step (rasterizer/mod.rs:233-281).  Returns the number of real
// segments written (1 or 2).
static inline int rasterize_step(const Fmt& f, const LineParams& l, int32_t pi, uint64_t out[2]) {
    int32_t x0i = wadd(l.start, pi);
    int32_t x1i = wadd(x0i, 1);
    int32_t border_x = x0i;
    float x0 = fmax_r((float)x0i, l.start_f32);
    float x1 = fmin_r((float)x1i, l.end_f32);
    float y0 = std::fma(l.slope, x0, l.py_slope_px);
    float y1 = std::fma(l.slope, x1, l.py_slope_px);
    int32_t x0s = to_sub_pixel(x0), x1s = to_sub_pixel(x1), y0s = to_sub_pixel(y0), y1s = to_sub_pixel(y1);
    if (intersects_y_border(y0s, y1s)) {
        int32_t y = std::max(y0s, y1s) >> PIXEL_SHIFT;
        int32_t ys = wshl(y, PIXEL_SHIFT);
        float x = std::fma(l.slope_recip, (float)y, l.px_slope_recip_py);
        int32_t xs = to_sub_pixel(x);
        int32_t by = std::min(ys, y0s) >> PIXEL_SHIFT;
        out[0] = make_segment(f, l.order, x0s, xs, y0s, ys, border_x, by, l.octant);
        by = std::min(ys, y1s) >> PIXEL_SHIFT;
        out[1] = make_segment(f, l.order, xs, x1s, ys, y1s, border_x, by, l.octant);
        return 2;
    }
    int32_t by = std::min(y0s, y1s) >> PIXEL_SHIFT;
    out[0] = make_segment(f, l.order, x0s, x1s, y0s, y1s, border_x, by, l.octant);
    return 1;
}

// ---------------------------------------------------------------------------
// parallel helpers (the rayon-shaped decomposition of the timed baseline)
// ---------------------------------------------------------------------------

static void parallel_for(size_t n, int threads, const std::function<void(size_t, size_t)>& fn) {
    if (threads <= 1 || n < 2048) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> ts;
    size_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        size_t b = (size_t)t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        ts.emplace_back([&, b, e] { fn(b, e); });
    }
    for (auto& t : ts) t.join();
}

static void parallel_sort(std::vector<uint64_t>& v, int threads) {
    size_t n = v.size();
    if (threads <= 1 || n < (1u << 16)) {
        std::sort(v.begin(), v.end());
        return;
    }
    int parts = 1;
    while (parts < threads) parts <<= 1;
    std::vector<size_t> bounds(parts + 1);
    for (int i = 0; i <= parts; i++) bounds[i] = n * (size_t)i / parts;
    {
        std::vector<std::thread> ts;
        for (int i = 0; i < parts; i++)
            ts.emplace_back([&, i] { std::sort(v.begin() + bounds[i], v.begin() + bounds[i + 1]); });
        for (auto& t : ts) t.join();
    }
    std::vector<uint64_t> tmp(n);
    std::vector<uint64_t>* src = &v;
    std::vector<uint64_t>* dst = &tmp;
    for (int width = 1; width < parts; width <<= 1) {
        std::vector<std::thread> ts;
        for (int i = 0; i < parts; i += 2 * width) {
            size_t b = bounds[i], m = bounds[std::min(i + width, parts)], e = bounds[std::min(i + 2 * width, parts)];
            ts.emplace_back([=] {
                std::merge(src->begin() + b, src->begin() + m, src->begin() + m, src->begin() + e, dst->begin() + b);
            });
        }
        for (auto& t : ts) t.join();
        std::swap(src, dst);
    }
    if (src != &v) v.swap(*src);
}

// ---------------------------------------------------------------------------
// painter styles (surpass/src/painter/style.rs, painter/mod.rs:53-123)
// ---------------------------------------------------------------------------

struct Gradient {
    uint32_t type = 0;
    float start[2] = {0, 0}, end[2] = {0, 0};
    std::vector<std::pair<std::array<float, 4>, float>> stops;
    bool operator==(const Gradient& o) const {
        if (type != o.type || stops.size() != o.stops.size()) return false;
        if (start[0] != o.start[0] || start[1] != o.start[1] || end[0] != o.end[0] || end[1] != o.end[1]) return false;
        for (size_t i = 0; i < stops.size(); i++)
            if (stops[i].first != o.stops[i].first || stops[i].second != o.stops[i].second) return false;
        return true;
    }
};

struct Props {  // Props / Func / Style (painter/mod.rs:125-141, style.rs:427-432)
    uint32_t fill_rule = CGB_FILL_NONZERO;
    uint32_t func = CGB_FUNC_DRAW;
    uint32_t clip_layers = 0;
    bool is_clipped = false;
    uint32_t blend_mode = CGB_BLEND_OVER;
    uint32_t fill_kind = CGB_FILL_SOLID;
    float color[4] = {0, 0, 0, 1};  // Fill::default (style.rs:183-187)
    Gradient gradient;
    bool operator==(const Props& o) const {
        if (fill_rule != o.fill_rule || func != o.func) return false;
        if (func == CGB_FUNC_CLIP) return clip_layers == o.clip_layers;
        if (is_clipped != o.is_clipped || blend_mode != o.blend_mode || fill_kind != o.fill_kind) return false;
        if (fill_kind == CGB_FILL_SOLID)
            return color[0] == o.color[0] && color[1] == o.color[1] && color[2] == o.color[2] && color[3] == o.color[3];
        return gradient == o.gradient;
    }
};

static bool props_from_c(const cgb_props* p, Props& out) {
    if (!p || p->fill_rule > 1 || p->func > 1 || p->blend_mode > 11 || p->fill_kind > 1) return false;
    out = Props{};
    out.fill_rule = p->fill_rule;
    out.func = p->func;
    out.clip_layers = p->clip_layers;
    out.is_clipped = p->is_clipped != 0;
    out.blend_mode = p->blend_mode;
    out.fill_kind = p->fill_kind;
    for (int i = 0; i < 4; i++) out.color[i] = p->color[i];
    if (p->fill_kind == CGB_FILL_GRADIENT) {
        // GradientBuilder::build (style.rs:66-84)
        if (p->n_stops < 2 || !p->stops || p->gradient_type > 1) return false;
        out.gradient.type = p->gradient_type;
        out.gradient.start[0] = p->gradient_start[0];
        out.gradient.start[1] = p->gradient_start[1];
        out.gradient.end[0] = p->gradient_end[0];
        out.gradient.end[1] = p->gradient_end[1];
        float inc = 1.0f / (float)(p->n_stops - 1);
        for (uint32_t i = 0; i < p->n_stops; i++) {
            const float* s = p->stops + 5 * i;
            if (s[4] < 0.0f || s[4] > 1.0f) return false;  // color_with_stop panics
            float stop = s[4] == -0.0f ? (float)i * inc : s[4];
            out.gradient.stops.push_back({{s[0], s[1], s[2], s[3]}, stop});
        }
    }
    return true;
}

// BlendMode::blend_fn (style.rs:206-267)
static float blend_fn(uint32_t mode, float dst, float src) {
    auto multiply = [](float d, float s) { return d * s; };
    auto screen = [](float d, float s) { return d + s - (d * s); };
    auto hard_light = [&](float d, float s) { return d <= 0.5f ? multiply(2.0f * d, s) : screen(2.0f * d - 1.0f, s); };
    switch (mode) {
        case CGB_BLEND_OVER: return src;
        case CGB_BLEND_MULTIPLY: return multiply(dst, src);
        case CGB_BLEND_SCREEN: return screen(dst, src);
        case CGB_BLEND_OVERLAY: return hard_light(src, dst);
        case CGB_BLEND_DARKEN: return fmin_r(dst, src);
        case CGB_BLEND_LIGHTEN: return fmax_r(dst, src);
        case CGB_BLEND_COLOR_DODGE:
            if (src == 0.0f) return 0.0f;
            if (dst == 1.0f) return 1.0f;
            return fmin_r(1.0f, src / (1.0f - dst));
        case CGB_BLEND_COLOR_BURN:
            if (src == 1.0f) return 1.0f;
            if (dst == 0.0f) return 0.0f;
            return 1.0f - fmin_r(1.0f, (1.0f - src) / dst);
        case CGB_BLEND_HARD_LIGHT: return hard_light(dst, src);
        case CGB_BLEND_SOFT_LIGHT: {
            auto d = [](float s) { return s <= 0.25f ? ((16.0f * s - 12.0f) * s + 4.0f) * s : std::sqrt(s); };
            if (dst <= 0.5f) return src - (1.0f - 2.0f * dst) * src * (1.0f - src);
            return src + (2.0f * dst - 1.0f) * (d(src) - src);
        }
        case CGB_BLEND_DIFFERENCE: return std::fabs(dst - src);
        case CGB_BLEND_EXCLUSION: return dst + src - 2.0f * dst * src;
    }
    return src;
}

// BlendMode::blend (style.rs:269-285)
static void blend_scalar(uint32_t mode, const float dst[4], const float src[4], float out[4]) {
    float alpha = src[3];
    float inv = 1.0f - alpha;
    float c0 = blend_fn(mode, dst[0], src[0]) * alpha;
    float c1 = blend_fn(mode, dst[1], src[1]) * alpha;
    float c2 = blend_fn(mode, dst[2], src[2]) * alpha;
    out[0] = std::fma(dst[0], inv, c0);
    out[1] = std::fma(dst[1], inv, c1);
    out[2] = std::fma(dst[2], inv, c2);
    out[3] = std::fma(dst[3], inv, alpha);
}

// blend_function! per lane (style.rs:288-418)
static float blend_vec1(uint32_t mode, float d, float s) {
    switch (mode) {
        case CGB_BLEND_OVER: return s;
        case CGB_BLEND_MULTIPLY: return d * s;
        case CGB_BLEND_SCREEN: return std::fma(d, -s, d) + s;
        case CGB_BLEND_OVERLAY:
            return s <= 0.5f ? (d * s * 2.0f) : 2.0f * (s + d - std::fma(s, d, 0.5f));
        case CGB_BLEND_DARKEN: return fmin_r(d, s);
        case CGB_BLEND_LIGHTEN: return fmax_r(d, s);
        case CGB_BLEND_COLOR_DODGE: return s == 0.0f ? 0.0f : fmin_r(1.0f, s / (1.0f - d));
        case CGB_BLEND_COLOR_BURN: return s == 1.0f ? 1.0f : 1.0f - fmin_r(1.0f, (1.0f - s) / d);
        case CGB_BLEND_HARD_LIGHT:
            return d <= 0.5f ? (d * s * 2.0f) : 2.0f * (s + d - std::fma(s, d, 0.5f));
        case CGB_BLEND_SOFT_LIGHT: {
            float dd = s <= 0.25f ? std::fma(std::fma(16.0f, s, -12.0f), s, 4.0f) * s : std::sqrt(s);
            float k = std::fma(2.0f, d, -1.0f);
            return d <= 0.5f ? std::fma(s * (1.0f - s), k, s) : std::fma(dd - s, k, s);
        }
        case CGB_BLEND_DIFFERENCE: return std::fabs(d - s);
        case CGB_BLEND_EXCLUSION: return std::fma(-2.0f * d, s, d) + s;
    }
    return s;
}

// linear_to_srgb_approx[_simd] (painter/mod.rs:73-106): same operations.
static inline float linear_to_srgb(float l) {
    const float a = 0.20101772f, b = -0.51280147f, c = 1.344401f, d = -0.030656587f;
    float s = std::sqrt(l);
    float s2 = l;
    float s3 = s2 * s;
    float m = l * 12.92f;
    float n = std::fma(a, s3, std::fma(b, s2, std::fma(c, s, d)));
    return l <= 0.0031308f ? m : n;
}
// to_byte / to_bytes (painter/mod.rs:108-123)
static inline uint8_t to_byte(float n) { return f2u8(std::fma(n, 255.0f, 0.5f)); }
static void to_bytes(const float color[4], uint8_t out[4]) {
    float ar = 1.0f / color[3];
    out[0] = to_byte(linear_to_srgb(color[0] * ar));
    out[1] = to_byte(linear_to_srgb(color[1] * ar));
    out[2] = to_byte(linear_to_srgb(color[2] * ar));
    out[3] = to_byte(color[3]);
}
// u8x8::from(f32x8) (simd/auto.rs:73-86)
static inline uint8_t round_u8(float v) { return f2u8(std::round(v)); }

// Gradient::get_t / color_at (style.rs:96-174) for 8 rows.
static void gradient_color_at(const Gradient& g, float x, float y, float out[4][8]) {
    float dx = g.end[0] - g.start[0];
    float dy = g.end[1] - g.start[1];
    float dot = dx * dx + dy * dy;
    float dot_recip = 1.0f / dot;
    float t[8];
    if (g.type == CGB_GRADIENT_LINEAR) {
        float tx = (x - g.start[0]) * dx * dot_recip;
        float ty = y - g.start[1];
        for (int k = 0; k < 8; k++) t[k] = std::fma(((float)k + ty) * dy, dot_recip, tx);
    } else {
        float px = x - g.start[0];
        float px2 = px * px;
        for (int k = 0; k < 8; k++) {
            float py = (float)k + (y - g.start[1]);
            t[k] = std::sqrt(std::fma(py, py, px2) * dot_recip);
        }
    }
    for (int ch = 0; ch < 4; ch++)
        for (int k = 0; k < 8; k++) out[ch][k] = 0.0f;
    bool mask[8], acc[8];
    bool any = false;
    for (int k = 0; k < 8; k++) {
        mask[k] = t[k] <= g.stops[0].second;
        any |= mask[k];
    }
    if (any)
        for (int ch = 0; ch < 4; ch++)
            for (int k = 0; k < 8; k++) out[ch][k] = fbits_or(out[ch][k], mask[k] ? g.stops[0].first[ch] : 0.0f);
    float start_stop = 0.0f;
    std::array<float, 4> start_color = g.stops[0].first;
    for (int k = 0; k < 8; k++) acc[k] = mask[k];
    for (size_t si = 1; si < g.stops.size(); si++) {
        const auto& color = g.stops[si].first;
        float end_stop = g.stops[si].second;
        bool m[8];
        bool any2 = false;
        for (int k = 0; k < 8; k++) {
            m[k] = acc[k] ^ (t[k] < end_stop);
            any2 |= m[k];
        }
        if (any2) {
            float d = end_stop - start_stop;
            float dr = 1.0f / d;
            for (int k = 0; k < 8; k++) {
                float lt = (t[k] - start_stop) * dr;
                for (int ch = 0; ch < 4; ch++) {
                    float v = std::fma(lt, color[ch], std::fma(-lt, start_color[ch], start_color[ch]));
                    out[ch][k] = fbits_or(out[ch][k], m[k] ? v : 0.0f);
                }
            }
            for (int k = 0; k < 8; k++) acc[k] = acc[k] || m[k];
        }
        start_stop = end_stop;
        start_color = color;
    }
    bool any3 = false;
    for (int k = 0; k < 8; k++) any3 |= !acc[k];
    if (any3) {
        const auto& last = g.stops.back().first;
        for (int ch = 0; ch < 4; ch++)
            for (int k = 0; k < 8; k++) out[ch][k] = fbits_or(out[ch][k], !acc[k] ? last[ch] : 0.0f);
    }
}

// from_area (painter/mod.rs:53-71)
static inline float from_area(int32_t area, uint32_t fill_rule) {
    if (fill_rule == CGB_FILL_NONZERO) return clamp_r(std::fabs((float)area * (1.0f / 256.0f)), 0.0f, 1.0f);
    int32_t number = area >> 8;
    float capped = (float)(area & 255) * (1.0f / 256.0f);
    return (number & 1) == 0 ? capped : 1.0f - capped;
}

// ---------------------------------------------------------------------------
// Cover (painter/mod.rs:148-199 with D2)
// ---------------------------------------------------------------------------

struct Cover {
    int8_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    void add(const Cover& o) {
        for (int i = 0; i < 8; i++) c[i] = (int8_t)(uint8_t)((uint8_t)c[i] + (uint8_t)o.c[i]);
    }
    bool is_empty(uint32_t fr) const {
        for (int i = 0; i < 8; i++) {
            if (fr == CGB_FILL_NONZERO) {
                if (c[i] != 0) return false;
            } else if ((abs8(c[i]) & 31) != 0) {
                return false;
            }
        }
        return true;
    }
    bool is_full(uint32_t fr) const {
        for (int i = 0; i < 8; i++) {
            if (fr == CGB_FILL_NONZERO) {
                if (abs8(c[i]) != PIXEL_WIDTH) return false;
            } else if ((abs8(c[i]) & 31) != 16) {
                return false;
            }
        }
        return true;
    }
};
static inline void add8(int8_t& a, int32_t b) { a = (int8_t)(uint8_t)((uint8_t)a + (uint8_t)(int8_t)b); }

struct CoverCarry {
    Cover cover;
    uint32_t layer;
};

// LayerProps (painter/mod.rs:143-146) over the composition's tables.
struct PropsView {
    const std::vector<const Props*>* by_order;  // indexed by order; null = missing
    const std::vector<uint8_t>* unchanged;      // indexed by order (cache only)
    const Props& get(uint32_t order) const {
        static const Props def{};
        if (order < by_order->size() && (*by_order)[order]) return *(*by_order)[order];
        return def;
    }
    bool is_unchanged(uint32_t order) const {
        if (!unchanged) return false;
        return order < unchanged->size() && (*unchanged)[order];
    }
};

// ---------------------------------------------------------------------------
// Painter (painter/mod.rs:207-468)
// ---------------------------------------------------------------------------

struct Painter {
    int16_t areas[64];
    int8_t covers[72];
    bool has_clip = false;
    float clip_mask[64];
    uint32_t clip_last = 0;
    float c0[64], c1[64], c2[64], alpha[64];

    void clear_cells() {
        std::memset(areas, 0, sizeof(areas));
        std::memset(covers, 0, sizeof(covers));
    }
    void acc_segment(uint64_t s) {
        uint32_t x = Fmt::tile_x(s), y = Fmt::tile_y(s);
        areas[x * 8 + y] = (int16_t)(uint16_t)((uint16_t)areas[x * 8 + y] + (uint16_t)(int16_t)Fmt::area(s));
        add8(covers[(x + 1) * 8 + y], Fmt::cover(s));
    }
    void acc_cover(const Cover& c) {
        for (int y = 0; y < 8; y++) add8(covers[y], c.c[y]);  // add_cover_to (column 0)
    }
    void clear(const float col[4]) {
        for (int i = 0; i < 64; i++) {
            c0[i] = col[0];
            c1[i] = col[1];
            c2[i] = col[2];
            alpha[i] = col[3];
        }
    }
    void fill_at(int x, int y, const Props& p, float fill[4][8]) {
        if (p.fill_kind == CGB_FILL_SOLID) {
            for (int ch = 0; ch < 4; ch++)
                for (int k = 0; k < 8; k++) fill[ch][k] = p.color[ch];
        } else {
            gradient_color_at(p.gradient, (float)x, (float)y, fill);
        }
    }
    void blend_at(int x, const float cov[8], bool is_clipped, const float fill[4][8], uint32_t mode) {
        for (int y = 0; y < 8; y++) {
            int i = x * 8 + y;
            float a = fill[3][y] * cov[y];
            if (is_clipped && has_clip) a *= clip_mask[i];
            float inv = 1.0f - a;
            float f0 = blend_vec1(mode, c0[i], fill[0][y]) * a;
            float f1 = blend_vec1(mode, c1[i], fill[1][y]) * a;
            float f2 = blend_vec1(mode, c2[i], fill[2][y]) * a;
            c0[i] = std::fma(c0[i], inv, f0);
            c1[i] = std::fma(c1[i], inv, f1);
            c2[i] = std::fma(c2[i], inv, f2);
            alpha[i] = std::fma(alpha[i], inv, a);
        }
    }
    void clip_at(int x, const float cov[8], uint32_t last_layer) {
        if (!has_clip) {
            has_clip = true;
            for (int i = 0; i < 64; i++) clip_mask[i] = 0.0f;
            clip_last = last_layer;
        }
        for (int y = 0; y < 8; y++) clip_mask[x * 8 + y] = cov[y];
    }
    // paint_layer (painter/mod.rs:260-317) with D2/D3.
    Cover paint_layer(int tile_i, int tile_j, uint32_t layer, const Props& p, bool apply_clip, bool wide) {
        int8_t run[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        float cov[8];
        if (has_clip && clip_last < layer) has_clip = false;
        for (int x = 0; x <= TILE_WIDTH; x++) {
            if (x != 0) {
                for (int y = 0; y < 8; y++) {
                    int32_t a = PIXEL_WIDTH * (int32_t)run[y] + (int32_t)areas[(x - 1) * 8 + y];
                    cov[y] = from_area(a, p.fill_rule);
                }
                if (p.func == CGB_FUNC_DRAW) {
                    bool all_zero = true;
                    for (int y = 0; y < 8; y++) all_zero &= cov[y] == 0.0f;
                    if (!all_zero && !(apply_clip && !has_clip)) {
                        float fill[4][8];
                        fill_at(x + tile_i * TILE_WIDTH, tile_j * TILE_HEIGHT, p, fill);
                        blend_at(x - 1, cov, apply_clip, fill, p.blend_mode);
                    }
                } else {
                    // `layer + *layers as u16` (u16 arithmetic; 17 bits in D5)
                    uint32_t last = wide ? ((layer + p.clip_layers) & 0x1FFFF) : ((layer + p.clip_layers) & 0xFFFF);
                    clip_at(x - 1, cov, last);
                }
            }
            for (int y = 0; y < 8; y++) add8(run[y], covers[x * 8 + y]);
        }
        Cover out;
        for (int y = 0; y < 8; y++) out.c[y] = run[y];
        return out;
    }
    // compute_srgb + write_to_tile (painter/mod.rs:418-493)
    void write_color_buffer(uint8_t* tile_px, size_t stride_px, int w, int h) {
        for (int x = 0; x < w; x++)
            for (int y = 0; y < h; y++) {
                int i = x * 8 + y;
                float a = alpha[i];
                uint8_t* o = tile_px + ((size_t)y * stride_px + x) * 4;
                o[0] = round_u8((linear_to_srgb(c0[i]) * a) * 255.0f);
                o[1] = round_u8((linear_to_srgb(c1[i]) * a) * 255.0f);
                o[2] = round_u8((linear_to_srgb(c2[i]) * a) * 255.0f);
                o[3] = round_u8(std::fma(a, 255.0f, 0.5f));
            }
    }
};

// ---------------------------------------------------------------------------
// LayerWorkbench (surpass/src/painter/layer_workbench.rs:120-486)
// ---------------------------------------------------------------------------

enum class TileOp { None, Solid, ColorBuffer };

struct Workbench {
    std::vector<uint32_t> ids;
    std::vector<uint8_t> mask;
    size_t skipped = 0;
    std::unordered_map<uint32_t, std::pair<size_t, size_t>> ranges;  // [b, e) in the tile's segments
    std::unordered_map<uint32_t, size_t> queue_indices;
    std::unordered_set<uint32_t> skip_clipping;
    std::vector<CoverCarry> queue, next_queue;

    struct Ctx {
        int tile_i, tile_j;
        const uint64_t* segs;
        size_t n;
        const PropsView* props;
        int32_t* previous_layers;  // -1 = None; null when no cache
        const float* clear_color;
        const Fmt* fmt;
    };

    void init(std::vector<CoverCarry>&& carries) {
        queue = std::move(carries);
    }
    void next_tile() {
        ids.clear();
        mask.clear();
        skipped = 0;
        ranges.clear();
        queue_indices.clear();
        skip_clipping.clear();
        std::swap(queue, next_queue);
        next_queue.clear();
    }
    const Cover* cover(uint32_t id) const {
        auto it = queue_indices.find(id);
        return it == queue_indices.end() ? nullptr : &queue[it->second].cover;
    }
    bool has_segments(uint32_t id) const { return ranges.count(id) != 0; }
    bool layer_is_full(const Ctx& c, uint32_t id, uint32_t fr) const {
        if (has_segments(id)) return false;
        const Cover* cv = cover(id);
        return cv ? cv->is_full(fr) : false;
    }
    bool cover_carry(const Ctx& c, uint32_t id, CoverCarry& out) const {
        Cover acc;
        auto it = ranges.find(id);
        if (it != ranges.end())
            for (size_t k = it->second.first; k < it->second.second; k++)
                add8(acc.c[Fmt::tile_y(c.segs[k])], Fmt::cover(c.segs[k]));
        if (const Cover* cv = cover(id)) acc.add(*cv);
        if (acc.is_empty(c.props->get(id).fill_rule)) return false;
        out = {acc, id};
        return true;
    }
    bool masked(size_t i) const { return i >= skipped && mask[i]; }

    // tile_unchanged_pass (:200-222)
    bool tile_unchanged_pass(const Ctx& c) {
        if (!c.previous_layers) return false;
        uint32_t layers = (uint32_t)(ids.size() & 0xFFFF);
        bool unchanged;
        if (*c.previous_layers >= 0) {
            int32_t old = *c.previous_layers;
            *c.previous_layers = (int32_t)layers;
            unchanged = (uint32_t)old == layers;
            if (unchanged)
                for (uint32_t id : ids)
                    if (!c.props->is_unchanged(id)) {
                        unchanged = false;
                        break;
                    }
        } else {
            *c.previous_layers = (int32_t)layers;
            unchanged = false;
        }
        return unchanged;
    }

    // skip_trivial_clips_pass (:224-308)
    void skip_trivial_clips_pass(const Ctx& c, bool wide) {
        struct Clip {
            bool is_full;
            uint32_t last;
            size_t i;
            bool is_used;
        };
        bool has = false;
        Clip clip{};
        for (size_t i = skipped; i < ids.size(); i++) {
            if (!mask[i]) continue;
            uint32_t id = ids[i];
            const Props& p = c.props->get(id);
            if (p.func == CGB_FUNC_CLIP) {
                bool full = layer_is_full(c, id, p.fill_rule);
                uint32_t last = wide ? ((id + p.clip_layers) & 0x1FFFF) : ((id + p.clip_layers) & 0xFFFF);
                has = true;
                clip = {full, last, i, false};
                if (full) mask[i] = 0;
            }
            if (p.func == CGB_FUNC_DRAW && p.is_clipped) {
                if (has && id <= clip.last) {
                    if (clip.is_full) skip_clipping.insert(id);
                    else clip.is_used = true;
                } else {
                    mask[i] = 0;
                }
            }
            if (has && id > clip.last) {
                has = false;
                if (!clip.is_used) mask[clip.i] = 0;
            }
        }
        if (has && !clip.is_used) mask[clip.i] = 0;
    }

    // skip_fully_covered_layers (:310-388).  Returns true with `color` set
    // when the tile resolves to TileWriteOp::Solid.
    bool skip_fully_covered_layers(const Ctx& c, float color[4]) {
        enum { NONE_, OPAQUE, INCOMPLETE } first = NONE_;
        float opaque[4] = {0, 0, 0, 0};
        for (size_t ii = ids.size(); ii-- > skipped;) {
            if (!mask[ii]) continue;
            uint32_t id = ids[ii];
            const Props& p = c.props->get(id);
            bool clipped = p.func == CGB_FUNC_DRAW && p.is_clipped && !skip_clipping.count(id);
            if (clipped || !layer_is_full(c, id, p.fill_rule)) {
                if (first == NONE_) first = INCOMPLETE;
            } else if (p.func == CGB_FUNC_DRAW && p.fill_kind == CGB_FILL_SOLID && p.blend_mode == CGB_BLEND_OVER) {
                if (p.color[3] == 1.0f) {
                    if (first == NONE_) {
                        first = OPAQUE;
                        std::memcpy(opaque, p.color, sizeof(opaque));
                    }
                    skipped = ii;
                    break;
                }
            }
        }
        size_t skip_n;
        float dst[4];
        if (first == OPAQUE) {
            skip_n = 1;
            std::memcpy(dst, opaque, sizeof(dst));
        } else if (first == NONE_) {
            skip_n = 0;
            std::memcpy(dst, c.clear_color, sizeof(dst));
        } else {
            return false;
        }
        size_t seen = 0;
        for (size_t i = skipped; i < ids.size(); i++) {
            if (!mask[i]) continue;
            if (seen++ < skip_n) continue;
            const Props& p = c.props->get(ids[i]);
            if (!(p.func == CGB_FUNC_DRAW && p.fill_kind == CGB_FILL_SOLID)) return false;
            float out[4];
            blend_scalar(p.blend_mode, dst, p.color, out);
            std::memcpy(dst, out, sizeof(dst));
        }
        std::memcpy(color, dst, sizeof(dst));
        return true;
    }

    // populate_layers (:401-428)
    void populate_layers(const Ctx& c) {
        size_t start = 0;
        while (start < c.n) {
            uint32_t id = c.fmt->layer(c.segs[start]);
            size_t e = start + 1;
            while (e < c.n && c.fmt->layer(c.segs[e]) == id) e++;
            ranges[id] = {start, e};
            start = e;
        }
        for (size_t i = 0; i < queue.size(); i++) queue_indices[queue[i].layer] = i;
        for (auto& kv : ranges) ids.push_back(kv.first);
        for (auto& kv : queue_indices) ids.push_back(kv.first);
        std::sort(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        mask.assign(ids.size(), 1);
        skipped = 0;
    }

    // drive_tile_painting (:430-486)
    TileOp drive(Painter& painter, const Ctx& c, float solid[4], bool wide) {
        populate_layers(c);
        bool brk = false;
        TileOp op = TileOp::ColorBuffer;
        if (tile_unchanged_pass(c)) {
            brk = true;
            op = TileOp::None;
        } else {
            skip_trivial_clips_pass(c, wide);
            if (skip_fully_covered_layers(c, solid)) {
                brk = true;
                op = TileOp::Solid;
            }
        }
        if (brk) {
            for (uint32_t id : ids) {
                CoverCarry cc;
                if (cover_carry(c, id, cc)) next_queue.push_back(cc);
            }
            next_tile();
            return op;
        }
        painter.clear(c.clear_color);
        for (size_t i = 0; i < ids.size(); i++) {
            uint32_t id = ids[i];
            if (masked(i)) {
                painter.clear_cells();
                auto it = ranges.find(id);
                if (it != ranges.end())
                    for (size_t k = it->second.first; k < it->second.second; k++) painter.acc_segment(c.segs[k]);
                if (const Cover* cv = cover(id)) painter.acc_cover(*cv);
                const Props& p = c.props->get(id);
                bool apply_clip = p.func == CGB_FUNC_DRAW && p.is_clipped && !skip_clipping.count(id);
                Cover out = painter.paint_layer(c.tile_i, c.tile_j, id, p, apply_clip, wide);
                if (!out.is_empty(p.fill_rule)) next_queue.push_back({out, id});
            } else {
                CoverCarry cc;
                if (cover_carry(c, id, cc)) next_queue.push_back(cc);
            }
        }
        next_tile();
        return TileOp::ColorBuffer;
    }
};

struct TileRect {  // Rect in tiles (buffer_layout.rs:37-50)
    int64_t h0, h1, v0, v1;
};

// Painter::paint_tile_row (painter/mod.rs:495-596) with D1.
static void paint_tile_row(Painter& painter, Workbench& wb, const Fmt& fmt, int j, const uint64_t* segs, size_t n,
                           const PropsView& props, const float clear[4], int32_t* layers_per_row, uint8_t* pixels,
                           size_t width, size_t height, size_t stride, size_t row_len, const TileRect* crop) {
    std::map<uint32_t, Cover> left;
    size_t k = 0;
    auto acc = [&](size_t b, size_t e) {
        for (size_t q = b; q < e; q++) add8(left[fmt.layer(segs[q])].c[Fmt::tile_y(segs[q])], Fmt::cover(segs[q]));
    };
    // populate_covers(None): the head run of left-of-canvas segments (D1).
    while (k < n && fmt.tile_i(segs[k]) == -1) k++;
    acc(0, k);
    if (crop && crop->h0 > 0) {
        int64_t limit = crop->h0 - 1;
        size_t b = k;
        while (k < n && fmt.tile_i(segs[k]) >= -1 && fmt.tile_i(segs[k]) <= limit) k++;
        acc(b, k);
    }
    std::vector<CoverCarry> init;
    for (auto& kv : left) init.push_back({kv.second, kv.first});
    wb.init(std::move(init));
    size_t th = std::min<size_t>(TILE_HEIGHT, height - (size_t)j * TILE_HEIGHT);
    for (size_t i = 0; i < row_len; i++) {
        if (crop && !((int64_t)i >= crop->h0 && (int64_t)i < crop->h1)) continue;
        size_t b = k;
        while (k < n && fmt.tile_i(segs[k]) == (int32_t)i) k++;
        Workbench::Ctx ctx{(int)i, j, segs + b, k - b, &props, layers_per_row ? &layers_per_row[i] : nullptr, clear, &fmt};
        painter.has_clip = false;
        float solid[4];
        TileOp op = wb.drive(painter, ctx, solid, fmt.wide);
        size_t tw = std::min<size_t>(TILE_WIDTH, width - i * TILE_WIDTH);
        uint8_t* tp = pixels + (((size_t)j * TILE_HEIGHT) * stride + i * TILE_WIDTH) * 4;
        if (op == TileOp::Solid) {
            uint8_t b4[4];
            to_bytes(solid, b4);
            for (size_t y = 0; y < th; y++)
                for (size_t x = 0; x < tw; x++) std::memcpy(tp + (y * stride + x) * 4, b4, 4);
        } else if (op == TileOp::ColorBuffer) {
            painter.write_color_buffer(tp, stride, (int)tw, (int)th);
        }
    }
}

// BufferLayout::print (buffer_layout.rs:170-231).  `segs` are the sorted real
// segments.
static void print(const Fmt& fmt, const std::vector<uint64_t>& segs, const PropsView& props, const float clear[4],
                  uint8_t* pixels, size_t width, size_t height, size_t stride, int32_t* layers_per_tile,
                  const TileRect* crop, int threads) {
    size_t row_len = (width + TILE_WIDTH - 1) / TILE_WIDTH;
    size_t rows = (height + TILE_HEIGHT - 1) / TILE_HEIGHT;
    // Cut the negative-tile_j tail (:187-191).
    size_t n = segs.size();
    {
        size_t lo = 0, hi = n;
        while (lo < hi) {  // first index whose tile_j is negative
            size_t mid = (lo + hi) / 2;
            if (fmt.tile_j(segs[mid]) < 0) hi = mid;
            else lo = mid + 1;
        }
        n = lo;
    }
    auto row_range = [&](int64_t j, size_t& b, size_t& e) {
        auto lb = [&](int64_t v) {
            size_t lo = 0, hi = n;
            while (lo < hi) {
                size_t mid = (lo + hi) / 2;
                if (fmt.tile_j(segs[mid]) < v) lo = mid + 1;
                else hi = mid;
            }
            return lo;
        };
        b = lb(j);
        e = lb(j + 1);
    };
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        Painter painter;
        Workbench wb;
        for (;;) {
            size_t j = next.fetch_add(1);
            if (j >= rows) break;
            if (crop && !((int64_t)j >= crop->v0 && (int64_t)j < crop->v1)) continue;
            size_t b, e;
            row_range((int64_t)j, b, e);
            paint_tile_row(painter, wb, fmt, (int)j, segs.data() + b, e - b, props, clear,
                           layers_per_tile ? layers_per_tile + j * row_len : nullptr, pixels, width, height, stride,
                           row_len, crop);
        }
    };
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> ts;
        for (int t = 0; t < threads; t++) ts.emplace_back(worker);
        for (auto& t : ts) t.join();
    }
}

// ---------------------------------------------------------------------------
// mold::Composition (mold/src/composition.rs, layer.rs, buffer.rs)
// ---------------------------------------------------------------------------

struct MLayer {
    SLayer inner;
    Props props;
    uint32_t unchanged = 0;  // SmallBitSet (layer.rs:101-142)
    size_t len = 0;
};

struct Cache {
    std::vector<int32_t> layers_per_tile;  // -1 = None
};

struct Composition {
    Fmt fmt;
    uint32_t max_ids;
    std::vector<float> p0x, p0y, p1x, p1y;
    std::vector<uint32_t> lids;
    std::map<uint32_t, MLayer> layers;
    std::set<uint32_t> used_ids;
    std::map<uint32_t, uint32_t> orders_to_layers;
    uint32_t caches_used = 0;
    std::map<int32_t, Cache> caches;
    orc_stats stats{};

    explicit Composition(bool wide) : fmt{wide}, max_ids(wide ? (1u << 17) : (1u << 16)) {}

    size_t actual_len() const {
        size_t s = 0;
        for (auto& kv : layers)
            if (kv.second.inner.is_enabled) s += kv.second.len;
        return s;
    }
    // IdSet::acquire (mold/src/layer.rs:61-72), lowest free id first.
    uint32_t next_fresh = 0;
    std::set<uint32_t> released;  // freed ids below next_fresh
    bool acquire(uint32_t& id) {
        if (!released.empty()) {
            id = *released.begin();
            released.erase(released.begin());
        } else {
            while (used_ids.count(next_fresh)) next_fresh++;
            if (next_fresh >= max_ids) return false;
            id = next_fresh++;
        }
        used_ids.insert(id);
        return true;
    }
    void release(uint32_t id) {  // IdSet::release (mold/src/layer.rs:74-98)
        used_ids.erase(id);
        if (id < next_fresh) released.insert(id);
    }
    MLayer& insert_bookkeeping(uint32_t id, size_t n) {  // insert_segments (composition.rs:58-79)
        MLayer& l = layers[id];
        l.inner.has_order = true;
        l.inner.order = id;
        l.inner.is_enabled = true;
        l.len += n;
        used_ids.insert(id);
        released.erase(id);
        return l;
    }
    void push(uint32_t id, const Seg4& s) {
        p0x.push_back(s.x0);
        p0y.push_back(s.y0);
        p1x.push_back(s.x1);
        p1y.push_back(s.y1);
        lids.push_back(id);
    }
    void remove_disabled() {  // composition.rs:124-142
        if (p0x.size() >= actual_len() * 2) {
            size_t w = 0;
            for (size_t i = 0; i < p0x.size(); i++) {
                auto it = layers.find(lids[i]);
                bool keep = it != layers.end() && it->second.inner.is_enabled;
                if (!keep) continue;
                p0x[w] = p0x[i];
                p0y[w] = p0y[i];
                p1x[w] = p1x[i];
                p1y[w] = p1y[i];
                lids[w] = lids[i];
                w++;
            }
            p0x.resize(w);
            p0y.resize(w);
            p1x.resize(w);
            p1y.resize(w);
            lids.resize(w);
            for (auto it = layers.begin(); it != layers.end();) {
                if (!it->second.inner.is_enabled) {
                    release(it->first);
                    it = layers.erase(it);
                } else {
                    ++it;
                }
            }
        }
    }

    // LinesBuilder::build + Rasterizer::rasterize + sort (composition.rs:292-297).
    void segments(std::vector<uint64_t>& out, uint64_t& steps, int threads) {
        size_t L = p0x.size();
        std::vector<LineParams> lp(L);
        std::vector<const SLayer*> table;
        uint32_t max_id = 0;
        for (auto& kv : layers) max_id = std::max(max_id, kv.first + 1);
        table.assign(max_id, nullptr);
        for (auto& kv : layers) table[kv.first] = &kv.second.inner;
        auto t0 = std::chrono::steady_clock::now();
        parallel_for(L, threads, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; i++) {
                const SLayer* sl = lids[i] < table.size() ? table[lids[i]] : nullptr;
                lp[i] = build_line(p0x[i], p0y[i], p1x[i], p1y[i], lids[i], sl, nullptr);
            }
        });
        auto t1 = std::chrono::steady_clock::now();
        std::vector<uint64_t> off(L + 1, 0);
        for (size_t i = 0; i < L; i++) off[i + 1] = off[i] + lp[i].length;
        steps = off[L];
        std::vector<uint64_t> slots(2 * steps);
        std::vector<uint8_t> nseg(steps);
        parallel_for(L, threads, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; i++)
                for (uint32_t pi = 0; pi < lp[i].length; pi++) {
                    uint64_t s[2];
                    size_t k = off[i] + pi;
                    nseg[k] = (uint8_t)rasterize_step(fmt, lp[i], (int32_t)pi, s);
                    slots[2 * k] = s[0];
                    slots[2 * k + 1] = s[1];
                }
        });
        out.clear();
        out.reserve(steps * 2);
        for (size_t k = 0; k < steps; k++) {
            out.push_back(slots[2 * k]);
            if (nseg[k] == 2) out.push_back(slots[2 * k + 1]);
        }
        auto t2 = std::chrono::steady_clock::now();
        parallel_sort(out, threads);
        auto t3 = std::chrono::steady_clock::now();
        stats.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        stats.rasterize_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
        stats.sort_ms = std::chrono::duration<double, std::milli>(t3 - t2).count();
        stats.lines = L;
        stats.steps = steps;
        stats.segments = out.size();
    }
};

}  // namespace orc

using namespace orc;

struct orc_composition {
    Composition c;
    explicit orc_composition(bool wide) : c(wide) {}
};

extern "C" {

size_t orc_flatten(const uint32_t* kinds, size_t n_cmds, const float* points, const float* transform9,
                   float* out_segments, size_t cap) {
    std::vector<Cmd> cmds;
    if (!decode_cmds(kinds, n_cmds, points, cmds)) return 0;
    std::vector<Seg4> segs;
    flatten(cmds, transform9, segs);
    for (size_t i = 0; i < segs.size() && i < cap; i++) {
        out_segments[4 * i] = segs[i].x0;
        out_segments[4 * i + 1] = segs[i].y0;
        out_segments[4 * i + 2] = segs[i].x1;
        out_segments[4 * i + 3] = segs[i].y1;
    }
    return segs.size();
}

void orc_build_lines(size_t n, const float* p0x, const float* p0y, const float* p1x, const float* p1y,
                     const uint32_t* layer_ids, const float* default_transform6, uint32_t* orders, int32_t* starts,
                     float* starts_f32, float* ends_f32, uint32_t* lengths, float* slopes, float* slopes_recip,
                     float* py_slope_pxs, float* px_slope_recip_pys, uint8_t* octants) {
    for (size_t i = 0; i < n; i++) {
        LineParams l = build_line(p0x[i], p0y[i], p1x[i], p1y[i], layer_ids[i], nullptr, default_transform6);
        orders[i] = l.order;
        starts[i] = l.start;
        starts_f32[i] = l.start_f32;
        ends_f32[i] = l.end_f32;
        lengths[i] = l.length;
        slopes[i] = l.slope;
        slopes_recip[i] = l.slope_recip;
        py_slope_pxs[i] = l.py_slope_px;
        px_slope_recip_pys[i] = l.px_slope_recip_py;
        octants[i] = l.octant;
    }
}

size_t orc_rasterize_lines(size_t n, const float* p0x, const float* p0y, const float* p1x, const float* p1y,
                           const uint32_t* layer_ids, uint64_t* out, size_t cap) {
    Fmt f{false};
    size_t k = 0;
    for (size_t i = 0; i < n; i++) {
        LineParams l = build_line(p0x[i], p0y[i], p1x[i], p1y[i], layer_ids[i], nullptr, nullptr);
        for (uint32_t pi = 0; pi < l.length; pi++) {
            uint64_t s[2];
            int m = rasterize_step(f, l, (int32_t)pi, s);
            if (k < cap) out[k] = s[0];
            if (k + 1 < cap) out[k + 1] = m == 2 ? s[1] : NONE;
            k += 2;
        }
    }
    return k;
}

void orc_blend_scalar(uint32_t mode, const float dst[4], const float src[4], float out[4]) {
    blend_scalar(mode, dst, src, out);
}

void orc_blend_vector(uint32_t mode, const float dst[3], const float src[3], float out[3]) {
    for (int i = 0; i < 3; i++) out[i] = blend_vec1(mode, dst[i], src[i]);
}

void orc_gradient_color_at(const cgb_props* props, float x, float y, float out[32]) {
    Props p;
    if (!props_from_c(props, p) || p.fill_kind != CGB_FILL_GRADIENT) {
        std::memset(out, 0, 32 * sizeof(float));
        return;
    }
    float o[4][8];
    gradient_color_at(p.gradient, x, y, o);
    for (int ch = 0; ch < 4; ch++)
        for (int k = 0; k < 8; k++) out[ch * 8 + k] = o[ch][k];
}

void orc_to_bytes(const float color[4], uint8_t out[4]) { to_bytes(color, out); }

orc_composition* orc_comp_new(uint32_t flags) { return new orc_composition((flags & CGB_COMPOSITION_WIDE_LAYERS) != 0); }
void orc_comp_free(orc_composition* c) { delete c; }

int orc_comp_create_layer(orc_composition* c, uint32_t* out_id) {
    return c->c.acquire(*out_id) ? CGB_OK : CGB_ERR_LAYER_LIMIT;
}

int orc_comp_insert_path(orc_composition* c, uint32_t layer_id, const uint32_t* kinds, size_t n_cmds,
                         const float* points, const float* transform9) {
    if (layer_id >= c->c.max_ids) return CGB_ERR_LAYER_LIMIT;
    std::vector<Cmd> cmds;
    if (!decode_cmds(kinds, n_cmds, points, cmds)) return CGB_ERR_INVALID_ARG;
    std::vector<Seg4> segs;
    flatten(cmds, transform9, segs);
    for (auto& s : segs) c->c.push(layer_id, s);
    c->c.insert_bookkeeping(layer_id, segs.size());
    return CGB_OK;
}

int orc_comp_insert_lines(orc_composition* c, uint32_t layer_id, const float* segments, size_t n) {
    if (layer_id >= c->c.max_ids) return CGB_ERR_LAYER_LIMIT;
    for (size_t i = 0; i < n; i++)
        c->c.push(layer_id, Seg4{segments[4 * i], segments[4 * i + 1], segments[4 * i + 2], segments[4 * i + 3]});
    c->c.insert_bookkeeping(layer_id, n);
    return CGB_OK;
}

int orc_comp_insert_paths(orc_composition* c, size_t n_paths, const uint32_t* layer_ids, const uint64_t* cmd_offsets,
                          const uint32_t* kinds, const uint64_t* point_offsets, const float* points,
                          const float* transforms9, const uint8_t* has_transform) {
    for (size_t k = 0; k < n_paths; k++) {
        const float* t = (transforms9 && has_transform && has_transform[k]) ? transforms9 + 9 * k : nullptr;
        int st = orc_comp_insert_path(c, layer_ids[k], kinds + cmd_offsets[k], cmd_offsets[k + 1] - cmd_offsets[k],
                                      points + point_offsets[k], t);
        if (st) return st;
    }
    return CGB_OK;
}

static MLayer* find_layer(orc_composition* c, uint32_t id) {
    auto it = c->c.layers.find(id);
    return it == c->c.layers.end() ? nullptr : &it->second;
}

int orc_layer_set_enabled(orc_composition* c, uint32_t id, int enabled) {
    MLayer* l = find_layer(c, id);
    if (!l) return CGB_ERR_NOT_FOUND;
    l->inner.is_enabled = enabled != 0;
    return CGB_OK;
}

int orc_layer_set_transform(orc_composition* c, uint32_t id, const float* t, uint32_t flags) {
    MLayer* l = find_layer(c, id);
    if (!l) return CGB_ERR_NOT_FOUND;
    // Layer::set_transform (mold/src/layer.rs:182-201)
    static const float I[6] = {1, 0, 0, 1, 0, 0};
    bool identity = !t || (t[0] == I[0] && t[1] == I[1] && t[2] == I[2] && t[3] == I[3] && t[4] == I[4] && t[5] == I[5]);
    bool has = !identity;
    if (has && !(flags & CGB_TRANSFORM_UNCHECKED)) {
        if (t[0] * t[0] + t[2] * t[2] > 1.001f || t[1] * t[1] + t[3] * t[3] > 1.001f) return CGB_ERR_SCALE;
    }
    bool changed = has != l->inner.has_transform;
    if (!changed && has)
        for (int i = 0; i < 6; i++) changed |= l->inner.transform[i] != t[i];
    if (changed) {
        l->unchanged = 0;
        l->inner.has_transform = has;
        if (has)
            for (int i = 0; i < 6; i++) l->inner.transform[i] = t[i];
    }
    return CGB_OK;
}

int orc_layer_set_order(orc_composition* c, uint32_t id, uint32_t order) {
    MLayer* l = find_layer(c, id);
    if (!l) return CGB_ERR_NOT_FOUND;
    if (order >= c->c.max_ids) return CGB_ERR_LAYER_LIMIT;
    if (!(l->inner.has_order && l->inner.order == order)) {
        l->unchanged = 0;
        l->inner.has_order = true;
        l->inner.order = order;
    }
    return CGB_OK;
}

int orc_layer_set_props(orc_composition* c, uint32_t id, const cgb_props* props) {
    MLayer* l = find_layer(c, id);
    if (!l) return CGB_ERR_NOT_FOUND;
    Props p;
    if (!props_from_c(props, p)) return CGB_ERR_INVALID_ARG;
    if (!(l->props == p)) {
        l->unchanged = 0;
        l->props = p;
    }
    return CGB_OK;
}

int orc_layers_set_solid(orc_composition* c, size_t n, const uint32_t* ids, const uint32_t* fill_rules,
                         const uint32_t* blend_modes, const float* colors) {
    for (size_t i = 0; i < n; i++) {
        cgb_props p{};
        p.fill_rule = fill_rules[i];
        p.func = CGB_FUNC_DRAW;
        p.blend_mode = blend_modes[i];
        p.fill_kind = CGB_FILL_SOLID;
        for (int k = 0; k < 4; k++) p.color[k] = colors[4 * i + k];
        int st = orc_layer_set_props(c, ids[i], &p);
        if (st) return st;
    }
    return CGB_OK;
}

int orc_layers_set_transforms(orc_composition* c, size_t n, const uint32_t* ids, const float* affine6,
                              uint32_t flags) {
    for (size_t i = 0; i < n; i++) {
        int st = orc_layer_set_transform(c, ids[i], affine6 + 6 * i, flags);
        if (st) return st;
    }
    return CGB_OK;
}

int orc_comp_remove_disabled(orc_composition* c) {
    c->c.remove_disabled();
    return CGB_OK;
}

void orc_comp_lens(orc_composition* c, uint64_t* builder_len, uint64_t* actual_len) {
    *builder_len = c->c.p0x.size();
    *actual_len = c->c.actual_len();
}

int orc_comp_create_cache(orc_composition* c, int32_t* out_id) {
    // SmallBitSet::first_empty_slot (mold/src/layer.rs:137-141)
    uint32_t bits = c->c.caches_used;
    int slot = 0;
    while (slot < 32 && (bits >> slot) & 1) slot++;
    if (slot >= 32) return CGB_ERR_LAYER_LIMIT;
    c->c.caches_used |= 1u << slot;
    c->c.caches[slot] = Cache{};
    *out_id = slot;
    return CGB_OK;
}

int orc_comp_release_cache(orc_composition* c, int32_t id) {
    if (id < 0 || id >= 32 || !((c->c.caches_used >> id) & 1)) return CGB_ERR_NOT_FOUND;
    c->c.caches_used &= ~(1u << id);
    c->c.caches.erase(id);
    return CGB_OK;
}

int orc_comp_render(orc_composition* oc, uint8_t* pixels, size_t width, size_t height, size_t stride,
                    const float background[4], const int64_t* crop, int32_t cache_id, int threads) {
    Composition& c = oc->c;
    if (stride == 0) stride = width;
    if (!pixels || width == 0 || stride < width || height == 0) return CGB_ERR_INVALID_ARG;
    Cache* cache = nullptr;
    if (cache_id >= 0) {
        auto it = c.caches.find(cache_id);
        if (it == c.caches.end()) return CGB_ERR_NOT_FOUND;
        cache = &it->second;
        // Buffer::tiles_len (mold/src/buffer.rs:37-44) and the resize/clear at composition.rs:218-225.
        size_t tiles_len = ((width + 7) / 8) * ((height + 7) / 8);
        if (cache->layers_per_tile.size() != tiles_len) cache->layers_per_tile.assign(tiles_len, -1);
    }
    c.remove_disabled();
    for (auto& kv : c.layers)
        if (kv.second.inner.is_enabled) c.orders_to_layers[kv.second.inner.order] = kv.first;
    std::vector<uint64_t> segs;
    uint64_t steps = 0;
    c.segments(segs, steps, threads);
    // LayerProps view by order (composition.rs:247-284).
    std::vector<const Props*> by_order;
    std::vector<uint8_t> unchanged;
    uint32_t max_order = 0;
    for (auto& kv : c.orders_to_layers) max_order = std::max(max_order, kv.first + 1);
    by_order.assign(max_order, nullptr);
    if (cache) unchanged.assign(max_order, 0);
    for (auto& kv : c.orders_to_layers) {
        auto it = c.layers.find(kv.second);
        if (it == c.layers.end()) continue;
        by_order[kv.first] = &it->second.props;
        if (cache) unchanged[kv.first] = (it->second.unchanged >> cache_id) & 1;
    }
    PropsView pv{&by_order, cache ? &unchanged : nullptr};
    TileRect tr{}, *trp = nullptr;
    if (crop) {
        tr = {crop[0] / 8, (crop[1] + 7) / 8, crop[2] / 8, (crop[3] + 7) / 8};
        trp = &tr;
    }
    auto t0 = std::chrono::steady_clock::now();
    print(c.fmt, segs, pv, background, pixels, width, height, stride,
          cache ? cache->layers_per_tile.data() : nullptr, trp, threads);
    auto t1 = std::chrono::steady_clock::now();
    c.stats.paint_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (cache)
        for (auto& kv : c.layers) {
            if (kv.second.inner.is_enabled) kv.second.unchanged |= 1u << cache_id;
            else kv.second.unchanged &= ~(1u << cache_id);
        }
    return CGB_OK;
}

int orc_comp_pixel_segments(orc_composition* oc, uint64_t* out, size_t cap, uint64_t* out_len, uint64_t* out_none,
                            int threads) {
    Composition& c = oc->c;
    c.remove_disabled();
    std::vector<uint64_t> segs;
    uint64_t steps = 0;
    c.segments(segs, steps, threads);
    *out_len = segs.size();
    *out_none = 2 * steps - segs.size();
    if (cap < segs.size()) return CGB_ERR_CAPACITY;
    if (!segs.empty()) std::memcpy(out, segs.data(), segs.size() * 8);
    return CGB_OK;
}

void orc_comp_stats(orc_composition* c, orc_stats* out) { *out = c->c.stats; }

}  // extern "C"
