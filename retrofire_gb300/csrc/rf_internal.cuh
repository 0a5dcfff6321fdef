// rf_internal.cuh — device-side records shared by the kernels and the host
// driver of librfgpu.
//
// Frame layout in HBM (one "job" = one target, possibly many draws):
//   cpos[v]  float4   clip-space position of every vertex of every draw
//   coc[v]   u8       outcode (clip.rs:240-242)
//   tcnt[t]  u32      clipped triangles produced by input triangle t (0..7)
//   toff[t]  u32      exclusive prefix sum of tcnt = first output prim of t
//   tpoly[t] u32      pool slot of t's clipped polygon (clipped tris only)
//   pool     PolyVert[slot][RF_POLY_STORE] Sutherland-Hodgman output polygons
//   prim[p]  PrimRec  triangle setup: two ScanlineIter starts (raster.rs:248-302)
//   mask     u32      per tile, one bit per input triangle of the job that
//                     touches the tile; bit order = submission order
#ifndef RF_INTERNAL_CUH
#define RF_INTERNAL_CUH

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
    uint32_t pad_;
    float vp[16];             // Mat4<Ndc, Screen>
};

struct StatsDev {
    unsigned long long prims_o, verts_o, frags_i, frags_o, oob;
};

struct PolyVert {
    float pos[4];
    float a[RF_MAX_ATTR];
};

// One ScanlineIter after scan() (raster.rs:45-51, 248-302): rows
// y0r, y0r+1, ... (n of them); left edge x and interpolated components
// c[0] = screen z, c[1..] = attributes, stepped by dl per row; right edge x
// stepped by drx; dvdx = per-pixel step.
struct HalfRec {
    float y0r;
    uint32_t n;
    float lx, dlx, rx, drx;
    float c[RF_NC];
    float dc[RF_NC];
    float dvdx[RF_NC];
};

struct PrimRec {
    uint32_t draw;
    uint32_t live;  // 0: culled by the face-cull test
    uint32_t pad_[2];
    HalfRec half[2];
};

#endif
