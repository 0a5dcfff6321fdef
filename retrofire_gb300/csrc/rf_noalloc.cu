// rf_noalloc.cu — rf_render_noalloc: one render() call that allocates no
// device memory.
//
// Who needs it: callers that may not call cudaMalloc at render time — a
// frame loop running under a fixed, pre-reserved device-memory budget, or a
// plugin living inside a host application that owns every allocation and
// hands the plugin only the buffers it is to fill.  They own their input and
// output buffers; the library supplies the scratch space from a fixed area
// compiled into it.
//
// The scratch is one file-scope __device__ array of RF_NOALLOC_SCRATCH_BYTES
// (8 MiB).  Every GPU that loads the library keeps that area until the
// process exits.  Host code only sees a host-side stand-in for the array's
// name, so the device address is looked up with cudaGetSymbolAddress, once
// per device, with that device current, on the first call made on it.  That
// first call should therefore happen before any stream capture begins.  The
// address is kept for the life of the process: after cudaDeviceReset on a
// device it is stale, so the call must not be used on a device that was
// reset since its first call.
//
// All calls share the one area and each call overwrites what the previous
// one left there; the parts that must start at zero are cleared by every
// call.  Two calls whose GPU work overlaps (different streams, or different
// host threads on one device) race on the area and give wrong results:
// order such calls on one stream.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/rfgpu.h"
#include "rf_internal.cuh"
#include "rf_kernels.cuh"

namespace {

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr uint32_t TILE_W = 32;
constexpr uint32_t WARPS = 4;
constexpr uint32_t MAX_TILES = ((RF_NOALLOC_MAX_W + TILE_W - 1) / TILE_W) *
                               ((RF_NOALLOC_MAX_H + RF_TILE_H - 1) / RF_TILE_H);
constexpr uint32_t MASK_WORDS = (RF_NOALLOC_MAX_TRIS + 31) / 32;
constexpr uint32_t SUM_WORDS = (MASK_WORDS + 31) / 32;

// Layout of the scratch area (byte offsets, 256-byte aligned).
constexpr size_t OFF_DRAW = 0;
constexpr size_t OFF_JOB = al(OFF_DRAW + sizeof(DrawDev));
constexpr size_t OFF_STATS = al(OFF_JOB + sizeof(JobDev));
constexpr size_t OFF_CNT = al(OFF_STATS + sizeof(StatsDev));
constexpr size_t OFF_CPOS = al(OFF_CNT + RF_CNT_N * 4);
constexpr size_t OFF_COC = al(OFF_CPOS + (size_t)RF_NOALLOC_MAX_VERTS * 16);
constexpr size_t OFF_TCNT = al(OFF_COC + RF_NOALLOC_MAX_VERTS);
constexpr size_t OFF_TOFF = al(OFF_TCNT + (size_t)RF_NOALLOC_MAX_TRIS * 4);
constexpr size_t OFF_TPOLY = al(OFF_TOFF + (size_t)RF_NOALLOC_MAX_TRIS * 4);
constexpr size_t OFF_SCAN = al(OFF_TPOLY + (size_t)RF_NOALLOC_MAX_TRIS * 4);
constexpr size_t OFF_POOL = al(OFF_SCAN + 64 * 4);
constexpr size_t OFF_PRIMS =
    al(OFF_POOL + (size_t)RF_NOALLOC_MAX_TRIS * RF_POLY_STORE * sizeof(PolyVert));
constexpr size_t OFF_MASK = al(OFF_PRIMS + (size_t)RF_NOALLOC_MAX_TRIS * RF_MAX_FAN * sizeof(PrimRec));
constexpr size_t OFF_ROWTOT = al(OFF_MASK + (size_t)MAX_TILES * (MASK_WORDS + SUM_WORDS) * 4);
constexpr size_t OFF_RPRIMS = al(OFF_ROWTOT + 8);
constexpr size_t OFF_LIVE =
    al(OFF_RPRIMS + (size_t)RF_NOALLOC_MAX_TRIS * RF_MAX_FAN * sizeof(RasterPrim));
constexpr size_t OFF_MARKS = al(OFF_LIVE + (size_t)RF_NOALLOC_MAX_TRIS * RF_MAX_FAN * 12);
constexpr size_t OFF_ITEMS = al(OFF_MARKS + 16);
constexpr size_t OFF_ROWS = al(OFF_ITEMS + (size_t)MAX_TILES * (RF_SPLIT_K + 1) * 4);
// The rest of the area holds row records; triangles whose records do not
// fit are rasterised from their setup records instead (same results).
constexpr size_t ROWS_WORDS = (RF_NOALLOC_SCRATCH_BYTES - OFF_ROWS) / 4;
static_assert(OFF_ROWS + (1u << 20) <= RF_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds its stated size");

constexpr int MAX_DEVICES = 64;
void *g_addr[MAX_DEVICES];
std::mutex g_mu;

uint32_t nattr_of(int32_t shader) {
    switch (shader) {
        case RF_SHADER_FLAT: return 0;
        case RF_SHADER_TEXTURED: return 2;
        case RF_SHADER_TEX_GOURAUD: return 5;
        default: return 3;
    }
}

uint32_t pack(uint32_t c, int32_t fmt) {
    const uint32_t r = c & 0xFFu, g = (c >> 8) & 0xFFu, b = (c >> 16) & 0xFFu, a = c >> 24;
    switch (fmt) {
        case RF_ARGB8888: return (a << 24) | (r << 16) | (g << 8) | b;
        case RF_XRGB8888: return (r << 16) | (g << 8) | b;
        case RF_RGBA8888: return (r << 24) | (g << 16) | (b << 8) | a;
        default: return (b << 24) | (g << 16) | (r << 8) | a;
    }
}

}  // namespace

// The scratch area itself; its device address is only ever taken through
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_rf_noalloc_scratch[RF_NOALLOC_SCRATCH_BYTES];

// The one draw's and the one job's descriptors, passed by value as kernel
// parameters and written into the scratch area on the stream (no host
// buffer has to outlive the call).
__global__ void k_na_put(DrawDev d, JobDev J, DrawDev *dd, JobDev *jd) {
    if (threadIdx.x == 0) {
        *dd = d;
        *jd = J;
    }
}

// On failure the runtime's last-error state is cleared too, so the
// launches of a later call do not report this error as theirs.
#define NA_CK(call)                              \
    do {                                         \
        if ((call) != cudaSuccess) {             \
            cudaGetLastError();                  \
            return RF_ERR_CUDA;                  \
        }                                        \
    } while (0)

extern "C" rf_status rf_render_noalloc(const float *verts, uint32_t nverts, uint32_t pos_dim,
                                       uint32_t nattr, const uint32_t *idx, uint32_t ntri,
                                       int32_t shader, const float mvp[16], uint32_t flat_rgba,
                                       const uint32_t *tex, uint32_t tw, uint32_t th,
                                       uint32_t sampler, const float viewport[16],
                                       uint32_t *color, float *depth, uint32_t w, uint32_t h,
                                       int32_t pixfmt, const rf_context_flags *flags,
                                       const uint32_t *clear_rgba, const float *depth_clear,
                                       void *cuda_stream, rf_stats *stats) {
    // ---- arguments and limits
    if (!mvp || !viewport || !flags || !color || !w || !h) return RF_ERR_BAD_ARG;
    if (pos_dim != 3 && pos_dim != 4) return RF_ERR_BAD_ARG;
    if (shader < RF_SHADER_FLAT || shader > RF_SHADER_GOURAUD_SRGB) return RF_ERR_BAD_ARG;
    if (nattr != nattr_of(shader)) return RF_ERR_BAD_ARG;
    if (pixfmt < RF_ARGB8888 || pixfmt > RF_BGRA8888) return RF_ERR_BAD_ARG;
    if (flags->depth_test < RF_DEPTH_NONE || flags->depth_test > RF_DEPTH_GREATER ||
        flags->face_cull < RF_CULL_NONE || flags->face_cull > RF_CULL_FRONT ||
        flags->depth_sort != RF_SORT_NONE)  // depth sorting needs scratch this area lacks
        return RF_ERR_BAD_ARG;
    if ((ntri && (!idx || !verts)) || (nverts && !verts)) return RF_ERR_BAD_ARG;
    // Triangles without vertices: every index would be out of range (the
    // reference panics on `vs[i]`, prim.rs:17-19).
    if (ntri && !nverts) return RF_ERR_BAD_ARG;
    if (ntri > RF_NOALLOC_MAX_TRIS || nverts > RF_NOALLOC_MAX_VERTS || w > RF_NOALLOC_MAX_W ||
        h > RF_NOALLOC_MAX_H)
        return RF_ERR_OVER_BUDGET;  // beyond the fixed scratch area
    const bool textured = shader == RF_SHADER_TEXTURED || shader == RF_SHADER_TEX_GOURAUD;
    if (textured) {
        if (!tex || !tw || !th || sampler > RF_SAMPLER_ONCE) return RF_ERR_BAD_ARG;
        if (sampler == RF_SAMPLER_REPEAT_POT && ((tw & (tw - 1)) || (th & (th - 1))))
            return RF_ERR_NON_POT_TEXTURE;
    }

    // ---- per-device set-up: the scratch area's device address
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return RF_ERR_NO_DEVICE;
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_rf_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return RF_ERR_CUDA;
            }
            g_addr[dev] = p;
        }
        base = static_cast<unsigned char *>(g_addr[dev]);
    }
    int nsm = 1;
    NA_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = (cudaStream_t)cuda_stream;

    // ---- descriptors of the one draw and the one job
    DrawDev d{};
    d.verts = verts;
    d.idx = idx;
    d.tex = textured ? tex : nullptr;
    d.nverts = nverts;
    d.ntri = ntri;
    d.pos_dim = pos_dim;
    d.nattr = nattr;
    d.stride = pos_dim + nattr;
    d.shader = shader;
    d.sampler = (int32_t)sampler;
    d.tw = tw;
    d.th = th;
    d.flat_rgba = flat_rgba;
    memcpy(d.mvp, mvp, sizeof d.mvp);
    JobDev J{};
    J.color = color;
    J.depth = depth;
    J.w = w;
    J.h = h;
    J.pixfmt = pixfmt;
    J.depth_test = flags->depth_test;
    J.color_write = flags->color_write;
    J.depth_write = flags->depth_write;
    J.face_cull = flags->face_cull;
    J.tiles_x = (w + TILE_W - 1) / TILE_W;
    J.tiles_y = (h + RF_TILE_H - 1) / RF_TILE_H;
    J.ntri = ntri;
    J.mask_words = (ntri + 31) / 32;
    J.mask_base = 0;
    J.sum_words = (J.mask_words + 31) / 32;
    J.sum_base = (uint64_t)J.tiles_x * J.tiles_y * J.mask_words;  // summaries after the masks
    if (clear_rgba) {
        J.clear_flags |= 1u;
        J.clear_px = pack(*clear_rgba, pixfmt);
    }
    if (depth_clear && depth) {
        J.clear_flags |= 2u;
        volatile float one = 1.0f;
        J.clear_z = one / *depth_clear;  // f32::recip
    }
    memcpy(J.vp, viewport, sizeof J.vp);
    const uint32_t ntiles = J.tiles_x * J.tiles_y;

    DrawDev *dd = reinterpret_cast<DrawDev *>(base + OFF_DRAW);
    JobDev *jd = reinterpret_cast<JobDev *>(base + OFF_JOB);
    StatsDev *sd = reinterpret_cast<StatsDev *>(base + OFF_STATS);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(base + OFF_CNT);
    float4 *cpos = reinterpret_cast<float4 *>(base + OFF_CPOS);
    uint8_t *coc = base + OFF_COC;
    uint32_t *tcnt = reinterpret_cast<uint32_t *>(base + OFF_TCNT);
    uint32_t *toff = reinterpret_cast<uint32_t *>(base + OFF_TOFF);
    uint32_t *tpoly = reinterpret_cast<uint32_t *>(base + OFF_TPOLY);
    uint32_t *scan = reinterpret_cast<uint32_t *>(base + OFF_SCAN);
    PolyVert *pool = reinterpret_cast<PolyVert *>(base + OFF_POOL);
    PrimRec *prims = reinterpret_cast<PrimRec *>(base + OFF_PRIMS);
    uint32_t *mask = reinterpret_cast<uint32_t *>(base + OFF_MASK);
    unsigned long long *rowtot = reinterpret_cast<unsigned long long *>(base + OFF_ROWTOT);
    RasterPrim *rprims = reinterpret_cast<RasterPrim *>(base + OFF_RPRIMS);
    uint32_t *live = reinterpret_cast<uint32_t *>(base + OFF_LIVE);
    unsigned long long *marks = reinterpret_cast<unsigned long long *>(base + OFF_MARKS);
    uint32_t *items = reinterpret_cast<uint32_t *>(base + OFF_ITEMS);
    uint32_t *rows = reinterpret_cast<uint32_t *>(base + OFF_ROWS);

    // ---- zero what the kernels accumulate into, then the pass itself
    NA_CK(cudaMemsetAsync(sd, 0, sizeof(StatsDev), s));
    NA_CK(cudaMemsetAsync(cnt, 0, RF_CNT_N * 4, s));
    if (ntri == 0) {
        if (J.clear_flags)
            NA_CK(rfk::launch_fill(color, depth, (size_t)w * h, J.clear_px, J.clear_z,
                                   J.clear_flags, nsm, s));
    } else {
        k_na_put<<<1, 32, 0, s>>>(d, J, dd, jd);
        NA_CK(cudaGetLastError());
        NA_CK(cudaMemsetAsync(mask, 0, (size_t)ntiles * (J.mask_words + J.sum_words) * 4, s));
        NA_CK(rfk::launch_vertex(dd, 1, nverts, cpos, coc, cnt, marks, nsm, s));
        NA_CK(rfk::launch_clip(dd, 1, ntri, cpos, coc, tcnt, tpoly, toff, pool, RF_NOALLOC_MAX_TRIS,
                               cnt, nsm, s, toff, false));  // (the scan places the outputs)
        NA_CK(rfk::launch_scan(tcnt, toff, ntri, scan, cnt + RF_CNT_PRIMS, s));
        NA_CK(rfk::launch_setup(dd, 1, jd, ntri, TILE_W, cpos, tcnt, toff, tpoly, pool, prims,
                                rowtot, rows, ROWS_WORDS, rprims, mask, live,
                                marks, sd, cnt, nsm, s, nullptr, nullptr, shader));
        NA_CK(rfk::launch_items(jd, 1, mask, ntiles, marks, (uint32_t)nsm * 16u, items, cnt, s));
        const bool fast = depth && flags->depth_test == RF_DEPTH_LESS && flags->color_write &&
                          flags->depth_write;
        NA_CK(rfk::launch_raster(TILE_W, shader, fast, jd, 1, dd, prims, rprims, rows, tcnt, toff,
                                 mask, ntiles, items, cnt + RF_CNT_ITEMS,
                                 cnt + RF_CNT_QUEUE, sd, WARPS, nsm, s));
    }
    if (stats) {
        StatsDev hs{};
        uint32_t hc[RF_CNT_N] = {0};
        NA_CK(cudaMemcpyAsync(&hs, sd, sizeof hs, cudaMemcpyDeviceToHost, s));
        NA_CK(cudaMemcpyAsync(hc, cnt, sizeof hc, cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        rf_stats o{};
        o.calls = 1;
        o.prims_i = ntri;
        o.verts_i = nverts;
        o.prims_o = hs.prims_o;
        o.verts_o = hs.verts_o;
        o.frags_i = hs.frags_i;
        o.frags_o = hs.frags_o;
        o.oob = hs.oob + hc[RF_CNT_POOLOVF] + hc[RF_CNT_POLYOVF] + hc[RF_CNT_BADIDX];
        *stats = o;
    }
    return RF_OK;
}
