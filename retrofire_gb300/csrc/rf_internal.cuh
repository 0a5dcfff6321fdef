// rf_internal.cuh — device-side records shared by the kernels and the host
// driver of librfgpu.
//
// Frame layout in HBM (one "job" = one target, possibly many draws):
//   cpos[v]  float4   clip-space position of every vertex of every draw
//   coc[v]   u8       outcode (clip.rs:240-242)
//   tcnt[t]  u32      clipped triangles produced by input triangle t (0..7)
//   toff[t]  u32      first output prim of t: t's fan holds prims toff[t] ..
//                     toff[t] + tcnt[t] (a block taken from a running total
//                     by k_clip, RF_MAX_FAN long for a clipped t; the
//                     exclusive prefix sum of tcnt in depth-sorted frames)
//   tpoly[t] u32      pool slot of t's clipped polygon (clipped tris only)
//   pool     PolyVert[slot][RF_POLY_STORE] Sutherland-Hodgman output polygons
//   prim[p]  PrimRec  triangle setup: two ScanlineIter starts (raster.rs:248-302)
//   mask     u32      per tile, one bit per input triangle of the job that
//                     touches the tile; bit order = submission order
#ifndef RF_INTERNAL_CUH
#define RF_INTERNAL_CUH

#include <stddef.h>
#include <stdint.h>

#define RF_MAX_ATTR 5        // (Color3f, TexCoord) is the widest varying
#define RF_NC (1 + RF_MAX_ATTR)  // interpolated components: screen z + attributes
#define RF_POLY_CAP 16       // clip working-buffer capacity
#define RF_POLY_STORE 9      // stored polygon vertices: a triangle clipped by 6 planes has <= 9
#define RF_MAX_FAN (RF_POLY_STORE - 2)  // fan triangles per input triangle
#define RF_TILE_H 32         // tile height = one warp lane per row

struct DrawDev {
    const float *verts;
    const uint32_t *idx;
    const uint32_t *tex;
    uint32_t nverts, ntri, pos_dim, nattr, stride;
    int32_t shader, sampler;
    uint32_t tw, th, flat_rgba;
    uint32_t vert_base;  // first global vertex of this draw
    uint32_t tri_base;   // first global input triangle of this draw
    uint32_t job;
    uint32_t flags;   // RF_DRAW_CULL_BBOX
    uint32_t culled;  // set on the device: the draw's bbox is Hidden
    uint32_t src_tri_base;  // first global input triangle (== tri_base except in a
                            // depth-sorted frame's setup, where tri_base counts
                            // clipped triangles)
    const float *bbox;  // BBox::of the positions (device): low x,y,z, high x,y,z
    float mvp[16];
};

struct JobDev {
    uint32_t *color;
    float *depth;  // nullptr: colour-only target
    uint32_t w, h;
    int32_t pixfmt;
    int32_t depth_test, color_write, depth_write, face_cull;
    uint32_t tiles_x, tiles_y, tile_base;
    uint32_t tri_base, ntri;  // global input-triangle range of the job
    uint32_t mask_words;      // bitmask words per tile
    uint64_t mask_base;       // word offset of the job's tile 0
    uint32_t clear_flags;     // bit0: colour clear pending, bit1: depth clear pending
    uint32_t clear_px;
    float clear_z;
    uint32_t sum_words;       // summary words per tile: bit b of word s = mask word 32 s + b is nonzero
    int32_t depth_sort;       // Context::depth_sort: 0 none, 1 front to back, 2 back to front
    uint64_t sum_base;        // word offset of the job's tile-0 summary (after every job's masks)
    float vp[16];             // Mat4<Ndc, Screen>
};

struct StatsDev {
    unsigned long long prims_o, verts_o, frags_i, frags_o, oob;
    // object culling: draws tested / drawn, and the host counts of the
    // culled draws (taken back out of calls, prims_i, verts_i)
    unsigned long long objs_i, objs_o, cull_calls, cull_prims, cull_verts;
};

struct PolyVert {
    float pos[4];
    float a[RF_MAX_ATTR];
};

// One ScanlineIter after scan() (raster.rs:45-51, 248-302): rows y0r,
// y0r+1, ... (n of them).  Row quantity r (RF_R_LX left edge x, RF_R_RX right
// edge x, RF_R_C + c interpolated component c: c = 0 screen z, c >= 1 the
// attributes) is the running sum b0[r] + d[r] + ... over rows; dvdx = the
// per-pixel step.
#define RF_R_LX 0
#define RF_R_RX 1
#define RF_R_C 2
#define RF_NR (RF_R_C + RF_NC)
struct HalfRec {
    float y0r;
    uint32_t n;
    uint32_t b0[RF_NR];
    float d[RF_NR];
    float dvdx[RF_NC];
};

// The exact value of every row of a half as two single-binade runs
// (rfx::fast_params): rows 0..e0[r] have bits b0[r] + j * i0[r]; one explicit
// addition later, rows e0[r]+1..e1[r] have bits b1[r] + (j - e0[r] - 1) *
// i1[r]; rows past e1[r] continue from the second run with the general loop.
// Only triangles rasterised without row records need them.
struct HalfRuns {
    int32_t i0[RF_NR];
    uint32_t e0[RF_NR];
    uint32_t b1[RF_NR];
    int32_t i1[RF_NR];
    uint32_t e1[RF_NR];
};

struct PrimRec {
    uint32_t draw;
    uint32_t live;    // 1: passed the face-cull test (only those get a record)
    uint32_t tri;     // global input triangle it was clipped from
    int32_t kind;     // shader kind of its draw
    uint32_t rloc;    // word offset of its row records in the frame's row buffer
    uint32_t rwords;  // words of row records; 0 = rasterised from this record instead
    uint32_t job;     // scene (job) of its draw
    uint32_t pad_;
    HalfRec half[2];  // what the binning pass reads (RF_PRIM_CORE_BYTES)
    HalfRuns runs[2]; // written only for a triangle without row records
};
#define RF_PRIM_CORE_BYTES 224u
static_assert(offsetof(PrimRec, runs) == RF_PRIM_CORE_BYTES && RF_PRIM_CORE_BYTES % 16 == 0 &&
                  sizeof(PrimRec) % 16 == 0,
              "PrimRec layout");

// Row records: for every scanline of a triangle that lands on a row of the
// target, word 0 = first pixel | (one past the last pixel) << 16 (the span
// xs..xe after zip truncation and clipping to the target; 0 when empty),
// words 1..NC = the varyings of the span's first fragment after the x0
// adjustment of raster.rs:102, and words NC+1..2NC = the varyings at the
// span's first tile boundary (the first pixel of the next tile column).
// Written once by the binning pass from a sequential walk of the scanlines
// (the reference's own running sums).
//
// RasterPrim: the rasteriser's view of one output triangle.
#define RF_RP_LIVE 1u
#define RF_RP_ROWS 2u  // row records present (else rasterise from the PrimRec)
struct RasterPrim {
    uint32_t draw;
    uint32_t flags;
    int32_t kind;
    uint32_t base;    // word offset of the first row record
    uint32_t stride;  // words per row record (1 + 2 NC)
    uint32_t y0, c0;  // upper half: rows y0 .. y0+c0-1, records 0 .. c0-1
    uint32_t y1, c1;  // lower half: rows y1 .. y1+c1-1, records c0 .. c0+c1-1
    float dvdx[2][RF_NC];
    float zmax;       // >= the depth of every fragment it writes into the target
                      // (+inf when unknown): a tile whose current depths are all
                      // >= zmax cannot pass any of them under the Less test
    uint32_t pad_[2];
};

// One line after clipping and to_screen (raster.rs:121-173): it steps
// along x (wide) or y, n pixels from `begin`; the other coordinate of
// pixel k is the k-step running sum s0 + d + ... (as usize); every pixel has
// depth z and the packed colour of the line's fragment.
#define RF_LINE_MAX_SPAN 4194304u  // longer lines (2^22 px) count in oob, not drawn
struct LineRec {
    uint32_t live, wide;
    uint64_t begin;
    uint32_t n;
    float s0, d, z;
    uint32_t color;
    uint32_t pad_;
};

#endif
