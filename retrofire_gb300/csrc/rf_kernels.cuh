// rf_kernels.cuh — constants and launch helpers shared by rf_kernels.cu and
// the C-ABI driver rf_api.cu.
#ifndef RF_KERNELS_CUH
#define RF_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "rf_internal.cuh"

// Mirrors of the public enums in include/rfgpu.h.
#define RF_K_FLAT 0
#define RF_K_GOURAUD 1
#define RF_K_TEXTURED 2
#define RF_K_TEX_GOURAUD 3
#define RF_K_GOURAUD_SRGB 4
#define RF_K_ANY 5  // rasteriser kernel that dispatches on each triangle's kind
#define RF_K_REPEAT_POT 0
#define RF_K_CLAMP 1
#define RF_K_ONCE 2
#define RF_K_ARGB8888 0
#define RF_K_XRGB8888 1
#define RF_K_RGBA8888 2
#define RF_K_BGRA8888 3
#define RF_K_DEPTH_NONE 0
#define RF_K_DEPTH_LESS 1
#define RF_K_DEPTH_EQUAL 2
#define RF_K_DEPTH_GREATER 3
#define RF_K_CULL_NONE 0
#define RF_K_CULL_BACK 1
#define RF_K_CULL_FRONT 2
#define RF_K_DRAW_CULL_BBOX 1u

#define RF_NO_POLY 0xFFFFFFFFu
// Scanline y origins beyond +-2^22 px are outside the supported domain: the
// row arithmetic y0r + j must stay exact in f32.  Such halves count in oob.
#define RF_MAX_COORD 4194304.0f
#define RF_RASTER_MAX_THREADS 256

// counters[] slots
#define RF_CNT_POOL 0     // pool slots used
#define RF_CNT_POOLOVF 1  // polygons dropped for lack of pool slots
#define RF_CNT_POLYOVF 2  // polygons that exceeded RF_POLY_CAP vertices
#define RF_CNT_BADIDX 3   // triangles with an out-of-range vertex index
#define RF_CNT_PRIMS 4    // total output prims (scan total)
#define RF_CNT_QUEUE 5    // tile queue head
#define RF_CNT_ROWSOVF 6  // triangles rasterised without row records (buffer full)
#define RF_CNT_LIVE 7     // output triangles that passed the face-cull test
#define RF_CNT_ITEMS 8    // rasteriser work items after the first ntiles (slices of crowded tiles)
#define RF_CNT_CLIPQ 10   // triangles queued for clipping
#define RF_CNT_LIVE_SMALL 11  // live triangles binned eight lanes each (at most 8 rows)
#define RF_CNT_LIVE_MID 12    // live triangles binned sixteen lanes each (9 to 16 rows)
#define RF_CNT_N 16
#define RF_SCAN_BLOCK_ITEMS 4096u  // values one scan block takes (one launch instead of three)

namespace rfk {
// counters (optional): POOL, QUEUE, LIVE (all three lists), PRIMS and CLIPQ
// zeroed for the kernels after it, and *marks (the binning pass's total of
// (triangle, tile) bits).
cudaError_t launch_vertex(const DrawDev *draws, uint32_t nd, uint32_t nv, float4 *cpos,
                          uint8_t *coc, uint32_t *counters, unsigned long long *marks,
                          int nsm, cudaStream_t s);
// Clip status, the clipping of the triangles that cross a plane, and each
// input triangle's fan count tcnt.  queue: room for nt triangle indices.
// place: each input triangle's first output slot into toff, taken from a
// running total (counters[RF_CNT_PRIMS]): one slot for a visible triangle,
// RF_MAX_FAN for one that is clipped (its fan fills the first tcnt), the
// triangles' blocks in any order -- every later pass finds a triangle's
// outputs through toff and tcnt.  Otherwise toff is left to the scan
// (launch_scan), which packs the outputs in clipped order for the depth
// sort, and the queue may be the scan's output array.
cudaError_t launch_clip(const DrawDev *draws, uint32_t nd, uint32_t nt, const float4 *cpos,
                        const uint8_t *coc, uint32_t *tcnt, uint32_t *tpoly, uint32_t *queue,
                        PolyVert *pool, uint32_t pool_cap, uint32_t *counters, int nsm, cudaStream_t s,
                        uint32_t *toff, bool place);
// BBox::of a mesh's positions (the first three floats of each vertex of
// stride floats) into bbox[0..6); bbox[6 ..) is scratch for the per-block
// parts: bbox holds RF_MESH_BBOX_FLOATS floats.
#define RF_MESH_BBOX_BLOCKS 64u
#define RF_MESH_BBOX_FLOATS (6u + 6u * RF_MESH_BBOX_BLOCKS)
cudaError_t launch_mesh_bbox(const float *verts, uint32_t nverts, uint32_t stride, float *bbox,
                             cudaStream_t s);
size_t scan_scratch_words(uint32_t n);
cudaError_t launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *scratch,
                        uint32_t *total, cudaStream_t s);
// Triangle setup (k_setup), then scanline statistics, row records and tile
// binning (k_bin_small for triangles of at most 8 and of 9 to 16 rows,
// then k_bin).  rows holds rows_cap words; rows_total (zeroed here)
// receives the words the frame asked for, each triangle's records placed
// by k_setup from it; live (room for three times every output triangle)
// receives the index of each triangle that passes the face-cull test: the
// regular ones with at most 8 rows on the target (counters[RF_CNT_LIVE_SMALL]) in its second
// third, with 9 to 16 rows (counters[RF_CNT_LIVE_MID]) in its last, the
// rest (counters[RF_CNT_LIVE]) in its first; *marks receives the
// (triangle, tile) bits set in all.  kind: the shader kind of every draw,
// or RF_K_ANY (the binning kernels are specialised for the first).
cudaError_t launch_setup(const DrawDev *draws, uint32_t nd, const JobDev *jobs, uint32_t nt,
                         uint32_t tile_w, const float4 *cpos, const uint32_t *tcnt,
                         const uint32_t *toff, const uint32_t *tpoly, const PolyVert *pool,
                         PrimRec *prims, unsigned long long *rows_total, uint32_t *rows,
                         unsigned long long rows_cap, RasterPrim *rprims, uint32_t *mask, uint32_t *live,
                         unsigned long long *marks, StatsDev *stats, uint32_t *counters, int nsm,
                         cudaStream_t s, const uint32_t *perm = nullptr, const uint32_t *ptri = nullptr,
                         int kind = RF_K_ANY);
// The rasteriser's work list from the tile masks and the marks total
// (slots: the warps the rasteriser keeps resident, about).  items (room
// for (RF_SPLIT_K + 1) * ntiles): items[ntiles .. ntiles + extra) first --
// heavy tiles (tile << RF_ITEM_SHIFT) and the row slices of crowded tiles
// (tile << RF_ITEM_SHIFT | k, k = 1 .. RF_SPLIT_K) -- then items[0 .. ntiles):
// tile t << RF_ITEM_SHIFT in index
// order, RF_ITEM_SKIP for the tiles already listed; extra is
// counters[RF_CNT_ITEMS] (zeroed by launch_setup).
cudaError_t launch_items(const JobDev *jobs, uint32_t nj, const uint32_t *mask, uint32_t ntiles,
                         const unsigned long long *marks, uint32_t slots, uint32_t *items,
                         uint32_t *counters, cudaStream_t s);
#ifndef RF_SPLIT_K
#define RF_SPLIT_K 4  // row slices of a crowded tile (RF_TILE_H / RF_SPLIT_K rows each)
#endif
// A work item is tile << RF_ITEM_SHIFT | k (k = 0: the whole tile, 1..RF_SPLIT_K: a slice).
#define RF_ITEM_SHIFT (RF_SPLIT_K < 8 ? 3u : 4u)
static_assert(RF_TILE_H % RF_SPLIT_K == 0 && RF_SPLIT_K < 16, "row slices");
#define RF_ITEM_SKIP 0xFFFFFFFEu  // a work-list entry taken elsewhere in the list
#define RF_MAX_TILES (1u << (31 - RF_ITEM_SHIFT))  // tiles of one frame or batch
cudaError_t launch_raster(uint32_t tile_w, int kind, bool fast, const JobDev *jobs, uint32_t nj,
                          const DrawDev *draws, const PrimRec *prims, const RasterPrim *rprims,
                          const uint32_t *rows, const uint32_t *tcnt, const uint32_t *toff,
                          const uint32_t *mask, uint32_t ntiles, const uint32_t *items, const uint32_t *nitems,
                          uint32_t *queue,
                          StatsDev *stats, uint32_t warps, int nsm, cudaStream_t s);
#define RF_DECL_RASTER_TW(TW)                                                                  \
    cudaError_t launch_raster_tw##TW(int kind, bool fast, const JobDev *jobs, uint32_t nj,      \
                                     const DrawDev *draws, const PrimRec *prims,                \
                                     const RasterPrim *rprims, const uint32_t *rows,            \
                                     const uint32_t *tcnt, const uint32_t *toff,                \
                                     const uint32_t *mask, uint32_t ntiles, const uint32_t *items, \
                                     const uint32_t *nitems, uint32_t *queue, StatsDev *stats,    \
                                     uint32_t warps, int nsm, cudaStream_t s);
RF_DECL_RASTER_TW(8)
RF_DECL_RASTER_TW(16)
RF_DECL_RASTER_TW(32)
RF_DECL_RASTER_TW(64)
#undef RF_DECL_RASTER_TW
cudaError_t launch_fill(uint32_t *color, float *depth, size_t n, uint32_t px, float z,
                        uint32_t flags, int nsm, cudaStream_t s);
// Object culling of the draws with RF_DRAW_CULL_BBOX (sets DrawDev::culled
// and counts into stats[draw.job]).
cudaError_t launch_cull(DrawDev *draws, uint32_t nd, StatsDev *stats, int nsm, cudaStream_t s);
// Line primitives (rf_lines.cu): setup + tile raster of one line draw
// (draws[0], jobs[0]; mask zeroed, queue zeroed).
cudaError_t launch_lines(const DrawDev *draws, const JobDev *jobs, uint32_t nl, const float4 *cpos,
                         const uint8_t *coc, LineRec *recs, uint32_t *mask, uint32_t ntiles,
                         uint32_t *queue, StatsDev *stats, int nsm, cudaStream_t s);
// Depth sort (render.rs:180-182, 209-219; rf_sort.cu).  launch_dsort: the
// key of every clipped triangle -- its draw, then Render::depth (the mean
// clip-space z, prim.rs:21-23) in f32::total_cmp order, ascending or
// descending per its job's depth_sort (0 for jobs without) -- sorted stably,
// so perm[r] is the clipped-order index of the r-th triangle; ptri[p] is the
// input triangle of clipped triangle p.  np = the frame's clipped
// triangles (host-known); scan_scratch holds
// scan_scratch_words(dsort_scan_items(np)) words.
size_t dsort_scratch_bytes(uint32_t np);
uint32_t dsort_scan_items(uint32_t np);
cudaError_t launch_dsort(const DrawDev *draws, uint32_t nd, const JobDev *jobs, uint32_t nt,
                         uint32_t np, const float4 *cpos, const uint32_t *tcnt, const uint32_t *toff,
                         const uint32_t *tpoly, const PolyVert *pool, const uint32_t *counters,
                         uint32_t *perm, uint32_t *ptri, void *scratch, uint32_t *scan_scratch,
                         cudaStream_t s);
// Per-draw clipped-triangle counts only (nout[d]), before np is known.
cudaError_t launch_draw_counts(const DrawDev *draws, uint32_t nd, uint32_t nt, const uint32_t *toff,
                               const uint32_t *counters, uint32_t *nout, cudaStream_t s);
// toff[i] = i, tcnt[i] = 1 for i < n: the raster's view of a sorted frame,
// where every clipped triangle is one unit of the tile masks.
cudaError_t launch_iota(uint32_t *toff, uint32_t *tcnt, uint32_t n, cudaStream_t s);
// Writes the GPU's global timer (ns) into *dst when the stream reaches it
// (dst: device memory or page-locked host memory).
cudaError_t launch_stamp(unsigned long long *dst, cudaStream_t s);
// Adds the n per-job stats slots js[0..n) into *total (one block).
cudaError_t launch_stats_fold(const StatsDev *js, uint32_t n, StatsDev *total, cudaStream_t s);
}  // namespace rfk

#endif
