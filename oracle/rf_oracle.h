/*
 * rf_oracle.h — CPU oracle for the retrofire triangle render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of the
 * reference's CPU renderer (retrofire-core, `render()` and everything it
 * calls for triangles).  It exists so that tests/, bench.py's CPU-baseline
 * leg and __graft_entry__.smoke() can check the CUDA library against the
 * reference's arithmetic.  Nothing in the product (retrofire_gb300/,
 * include/) may link, load or call it.
 *
 * Parity is pinned by the reference's own golden images and unit-test
 * vectors (core/tests/rendering.rs + textured_quad.ppm, core/examples/
 * hello_tri.rs + triangle.ppm, raster.rs/clip.rs/tex.rs/pixfmt.rs tests);
 * see tests/test_oracle_pins.py.
 *
 * Built with -O2 -ffp-contract=off (no FMA contraction, no fast-math):
 * Rust never contracts a*b+c, so neither may the oracle.
 */
#ifndef RF_ORACLE_H
#define RF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shader families (fragment side); vertex side is `mvp.apply(pos)`. */
enum { RFO_FLAT = 0, RFO_GOURAUD = 1, RFO_TEXTURED = 2, RFO_TEX_GOURAUD = 3,
       RFO_GOURAUD_SRGB = 4 };
/* Samplers (core/src/render/tex.rs). */
enum { RFO_REPEAT_POT = 0, RFO_CLAMP = 1, RFO_ONCE = 2 };
/* Pixel formats of the u32 colour buffer (core/src/util/pixfmt.rs). */
enum { RFO_ARGB8888 = 0, RFO_XRGB8888 = 1, RFO_RGBA8888 = 2, RFO_BGRA8888 = 3 };
/* Context::depth_test: None / Some(Less) / Some(Equal) / Some(Greater). */
enum { RFO_DEPTH_NONE = 0, RFO_DEPTH_LESS = 1, RFO_DEPTH_EQUAL = 2,
       RFO_DEPTH_GREATER = 3 };
/* Context::face_cull: None / Some(Back) / Some(Front). */
enum { RFO_CULL_NONE = 0, RFO_CULL_BACK = 1, RFO_CULL_FRONT = 2 };

typedef struct {
    const float *verts;     /* nverts * (pos_dim + nattr) floats */
    uint32_t nverts;
    uint32_t pos_dim;       /* 3: model-space point through mvp; 4: clip-space passthrough */
    uint32_t nattr;         /* attribute floats per vertex, matching the shader */
    const uint32_t *idx;    /* ntri * 3 vertex indices */
    uint32_t ntri;
    int32_t shader;
    float mvp[16];          /* row-major, Matrix.0[row][col] */
    uint32_t flat_rgba;     /* Color4 bytes r,g,b,a packed little-endian */
    const uint32_t *tex;    /* tw*th texels, Color4 bytes r,g,b,a little-endian */
    uint32_t tw, th;
    int32_t sampler;
} rfo_draw;

/* Context::depth_sort: None / Some(FrontToBack) / Some(BackToFront). */
enum { RFO_SORT_NONE = 0, RFO_SORT_FRONT_TO_BACK = 1, RFO_SORT_BACK_TO_FRONT = 2 };

typedef struct {
    int32_t depth_test;
    int32_t color_write;
    int32_t depth_write;
    int32_t face_cull;
    int32_t depth_sort;
} rfo_ctx;

typedef struct {
    uint64_t calls, prims_i, prims_o, verts_i, verts_o, frags_i, frags_o, oob;
} rfo_stats;

/* One `render()` call into a colour target (u32, pixfmt) and an optional
 * f32 depth buffer (NULL selects the colour-only `rasterize` path).
 * Stats are ADDED into *st, like `ctx.stats += ...` in render.rs. */
void rfo_render(const rfo_draw *d, const float viewport[16],
                uint32_t *color, float *depth, uint32_t w, uint32_t h,
                int32_t pixfmt, const rfo_ctx *ctx, rfo_stats *st);

/* Frame::clear semantics (front/src/lib.rs:103-120). */
void rfo_clear(uint32_t *color, float *depth, uint32_t w, uint32_t h,
               int32_t pixfmt, const uint32_t *clear_rgba,
               const float *depth_clear);

/* Pack Color4 (bytes r,g,b,a little-endian) into a u32 pixel. */
uint32_t rfo_pack(uint32_t rgba, int32_t pixfmt);

/* Clip n triangles (clip-space positions, 12 floats each; attrib = one f32
 * per vertex) against the view frustum.  counts[i] = number of output
 * triangles.  If out_pos != NULL it receives 7*12 floats per input tri.
 * Returns 1 iff every output vertex is within |x/w|,|y/w|,|z/w| <= 1.00001
 * (the in_bounds check of clip.rs tests). */
int32_t rfo_clip_batch(uint32_t n, const float *pos, const float *attr,
                       uint32_t *counts, float *out_pos, float *out_attr);

/* tri_fill on three screen-space vertices (x,y,z each) with nattr
 * attributes; zdiv_mask bit i set => attribute i is divided by pos.z in
 * Scanline::fragments.  Emits each scanline (y, xs.start, xs.end) into
 * rows (3 u64 per row) and every fragment's z_div'ed attributes into frags
 * (nattr floats per fragment, in emission order).  Returns number of rows;
 * *nfrags receives the number of fragments. */
uint32_t rfo_tri_fill(const float *screen, const float *attr, uint32_t nattr,
                      uint32_t zdiv_mask, uint64_t *rows, uint32_t max_rows,
                      float *frags, uint64_t max_frags, uint64_t *nfrags);

/* Texture sampling (tex.rs) of one texel; returns the Color4 as packed
 * little-endian bytes. */
uint32_t rfo_sample(const uint32_t *tex, uint32_t tw, uint32_t th,
                    int32_t sampler, float u, float v);

#ifdef __cplusplus
}
#endif
#endif
