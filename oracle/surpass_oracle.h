/*
 * CPU restatement of the surpass/mold rasterize -> sort -> paint path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GPU implementation in cassia_gb300/: only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline leg load it, and only as the checker or as the
 * timed CPU baseline.  The product never links or calls it.
 *
 * Every function restates the reference statement by statement; the file:line
 * citations are relative to the Kangz/cassia project root.  Deviations from
 * the reference (it cannot run at HEAD, see surpass_oracle.cpp) are named
 * D1..D5 and listed at the top of surpass_oracle.cpp.
 */
#ifndef CASSIA_GB300_SURPASS_ORACLE_H
#define CASSIA_GB300_SURPASS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/cassia_gb300.h" /* shared plain-data types (cgb_props, command kinds) */

#ifdef __cplusplus
extern "C" {
#endif

/* ---- stage-level entry points (known-answer tests) ---------------------- */

/* mold PathSegments (mold/src/path/segments.rs:97-263): flattens one path.
 * `points` holds the floats of each command as passed to mold's Path API
 * (see CGB_CMD_* in cassia_gb300.h).  `transform9` may be NULL.  Writes up to
 * `cap` segments as (p0x, p0y, p1x, p1y) and returns the total count. */
size_t orc_flatten(const uint32_t* kinds, size_t n_cmds, const float* points,
                   const float* transform9, float* out_segments, size_t cap);

/* surpass LinesBuilder::build (surpass/src/segment.rs:91-237) for lines with
 * no per-layer table (layers(_) == None).  Outputs are arrays of length n. */
void orc_build_lines(size_t n, const float* p0x, const float* p0y, const float* p1x,
                     const float* p1y, const uint32_t* layer_ids, const float* default_transform6,
                     uint32_t* orders, int32_t* starts, float* starts_f32, float* ends_f32,
                     uint32_t* lengths, float* slopes, float* slopes_recip, float* py_slope_pxs,
                     float* px_slope_recip_pys, uint8_t* octants);

/* Rasterizer::rasterize (surpass/src/rasterizer/mod.rs:214-285) for lines with
 * no layer table: writes the reference's 2*S array ([seg0, seg1 or NONE] per
 * pixel step, u16 layer format) and returns 2*S. */
size_t orc_rasterize_lines(size_t n, const float* p0x, const float* p0y, const float* p1x,
                           const float* p1y, const uint32_t* layer_ids, uint64_t* out, size_t cap);

/* BlendMode::blend (scalar, style.rs:269-285) and blend_function! (vector
 * formula, style.rs:288-418) on single values. */
void orc_blend_scalar(uint32_t mode, const float dst[4], const float src[4], float out[4]);
void orc_blend_vector(uint32_t mode, const float dst[3], const float src[3], float out[3]);

/* Gradient::color_at (style.rs:121-174) for an 8-row column at (x, y). */
void orc_gradient_color_at(const cgb_props* props, float x, float y, float out[32]);

/* linear_to_srgb_approx + to_bytes (painter/mod.rs:90-123). */
void orc_to_bytes(const float color[4], uint8_t out[4]);

/* ---- mold::Composition ---------------------------------------------------- */

typedef struct orc_composition orc_composition;

orc_composition* orc_comp_new(uint32_t flags /* CGB_COMPOSITION_WIDE_LAYERS */);
void orc_comp_free(orc_composition* c);
int orc_comp_create_layer(orc_composition* c, uint32_t* out_id);
int orc_comp_insert_path(orc_composition* c, uint32_t layer_id, const uint32_t* kinds,
                         size_t n_cmds, const float* points, const float* transform9);
int orc_comp_insert_lines(orc_composition* c, uint32_t layer_id, const float* segments, size_t n);
/* Batched insert_in_layer (same layout as cgb_insert_paths). */
int orc_comp_insert_paths(orc_composition* c, size_t n_paths, const uint32_t* layer_ids,
                          const uint64_t* cmd_offsets, const uint32_t* kinds,
                          const uint64_t* point_offsets, const float* points,
                          const float* transforms9, const uint8_t* has_transform);
/* Batched set_props with Fill::Solid styles, and batched set_transform. */
int orc_layers_set_solid(orc_composition* c, size_t n, const uint32_t* ids, const uint32_t* fill_rules,
                         const uint32_t* blend_modes, const float* colors);
int orc_layers_set_transforms(orc_composition* c, size_t n, const uint32_t* ids, const float* affine6,
                              uint32_t flags);
int orc_layer_set_enabled(orc_composition* c, uint32_t id, int enabled);
int orc_layer_set_transform(orc_composition* c, uint32_t id, const float* affine6, uint32_t flags);
int orc_layer_set_order(orc_composition* c, uint32_t id, uint32_t order);
int orc_layer_set_props(orc_composition* c, uint32_t id, const cgb_props* props);
int orc_comp_remove_disabled(orc_composition* c);
void orc_comp_lens(orc_composition* c, uint64_t* builder_len, uint64_t* actual_len);
int orc_comp_create_cache(orc_composition* c, int32_t* out_id);
int orc_comp_release_cache(orc_composition* c, int32_t id);

/* Composition::render (mold/src/composition.rs:212-329) into a host RGBA8
 * buffer of `height` rows of `width_stride` pixels.  `crop` is
 * {x0, x1, y0, y1} in pixels or NULL.  `cache_id` < 0 means no layer cache.
 * `threads` > 1 runs the rayon-shaped std::thread decomposition. */
int orc_comp_render(orc_composition* c, uint8_t* pixels, size_t width, size_t height,
                    size_t width_stride, const float background[4], const int64_t* crop,
                    int32_t cache_id, int threads);

/* Composition::pixel_segments (mold/src/composition.rs:153-188): the P real
 * segments sorted by the full u64 (canonical refinement of the reference's
 * key>>22 order), plus the count of NONE slots of the reference's 2*S array. */
int orc_comp_pixel_segments(orc_composition* c, uint64_t* out, size_t cap, uint64_t* out_len,
                            uint64_t* out_none, int threads);

/* Per-stage wall times (ms) and sizes of the last render / pixel_segments. */
typedef struct orc_stats {
    double build_ms, rasterize_ms, sort_ms, paint_ms;
    uint64_t lines, steps, segments;
} orc_stats;
void orc_comp_stats(orc_composition* c, orc_stats* out);

#ifdef __cplusplus
}
#endif
#endif
