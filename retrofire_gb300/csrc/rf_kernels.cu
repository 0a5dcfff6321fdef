// rf_kernels.cu — CUDA kernels of the triangle render path (sm_103a).
//
// Stage map (reference call stack: core/src/render.rs:134-207):
//   k_vertex     vertex shader + ClipVert::new         render.rs:157-165
//   k_clip       status; the crossing triangles queue  clip.rs:245-267
//   k_clip_poly  Sutherland-Hodgman on the queue       clip.rs:283-301,350-400
//   k_scan_*     order-preserving compaction offsets   (submission order)
//   k_setup      to_screen, face cull, tri_fill/scan   prim.rs:62-88, raster.rs:185-302
//                setup, the live list
//   k_bin        scanline walk: stats (frags.i, oob),  raster.rs:80-114, target.rs:259-264
//                row records, tile binning, one warp
//                per live triangle
//   k_tile_items the rasteriser's work list            (scheduling only)
//   k_raster     per-tile span fill, depth test,       raster.rs:60-69, target.rs:163-198
//                fragment shading, pixel packing       (rf_raster.cuh)
//   k_fill       Frame::clear without a later render   front/src/lib.rs:103-120
#include <cuda_runtime.h>

#include "rf_exact.cuh"
#include "rf_internal.cuh"
#include "rf_kernels.cuh"
#include "rf_device.cuh"

using namespace rfx;
using namespace rfd;

namespace {

__constant__ float c_planes[6][4] = {
    {0.0f, 0.0f, -1.0f, -1.0f},  // near   (clip.rs:215-222)
    {0.0f, 0.0f, 1.0f, -1.0f},   // far
    {-1.0f, 0.0f, 0.0f, -1.0f},  // left
    {1.0f, 0.0f, 0.0f, -1.0f},   // right
    {0.0f, -1.0f, 0.0f, -1.0f},  // bottom
    {0.0f, 1.0f, 0.0f, -1.0f},   // top
};

__device__ __forceinline__ uint32_t outcode(const float *p) {
    uint32_t oc = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) oc |= (dot4(c_planes[i], p) > 0.0f) ? (1u << i) : 0u;
    return oc;
}

__device__ __forceinline__ uint32_t nattr_of(int32_t shader) {
    switch (shader) {
        case RF_K_FLAT: return 0;
        case RF_K_TEXTURED: return 2;
        case RF_K_TEX_GOURAUD: return 5;
        default: return 3;
    }
}
// Attributes that ZDiv divides (TexCoord, vec.rs:666-677); colours do not
// (color.rs:628).
__device__ __forceinline__ uint32_t zdiv_mask_of(int32_t shader) {
    return shader == RF_K_TEXTURED ? 0x3u : (shader == RF_K_TEX_GOURAUD ? 0x18u : 0u);
}

}  // namespace

// ---------------------------------------------------------------------------
// K1: vertex shader (mvp.apply, mat.rs:952-973, or clip-space passthrough)
// and outcode (clip.rs:240-242, 303-309).
// ---------------------------------------------------------------------------
__global__ void k_vertex(const DrawDev *__restrict__ draws, uint32_t nd, uint32_t nv_total,
                         float4 *__restrict__ cpos, uint8_t *__restrict__ coc,
                         uint32_t *__restrict__ counters, unsigned long long *__restrict__ marks) {
    if (blockIdx.x == 0) {  // the frame's counters, for the kernels after this one
        if (counters && threadIdx.x == 0) {
            counters[RF_CNT_POOL] = 0;
            counters[RF_CNT_QUEUE] = 0;
            counters[RF_CNT_LIVE] = 0;
            counters[RF_CNT_LIVE_SMALL] = 0;
            counters[RF_CNT_LIVE_MID] = 0;
            counters[RF_CNT_PRIMS] = 0;
            counters[RF_CNT_CLIPQ] = 0;
            *marks = 0;
        }
    }
    // Warp-uniform loop (the draw lookup is shared by the warp's lanes).
    for (uint32_t wbase = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wbase < nv_total;
         wbase += gridDim.x * blockDim.x) {
        const uint32_t gv = wbase + (threadIdx.x & 31u);
        const uint32_t di = warp_upper_index(nd, gv < nv_total ? gv : nv_total - 1,
                                             [&](uint32_t i) { return draws[i].vert_base; });
        if (gv >= nv_total) continue;
        const DrawDev &d = draws[di];
        if (d.culled) continue;  // a render() call that is not made
        const float *src = d.verts + (size_t)(gv - d.vert_base) * d.stride;
        float p[4];
        if (d.pos_dim == 4) {
            p[0] = src[0]; p[1] = src[1]; p[2] = src[2]; p[3] = src[3];
        } else {
            const float h[4] = {src[0], src[1], src[2], 1.0f};  // Point3::to_hom
#pragma unroll
            for (int r = 0; r < 4; ++r) p[r] = dot4(d.mvp + 4 * r, h);
        }
        cpos[gv] = make_float4(p[0], p[1], p[2], p[3]);
        coc[gv] = (uint8_t)outcode(p);
    }
}

// ---------------------------------------------------------------------------
// A mesh's BBox::of (render/scene.rs:37-46: BBox::extend over every
// position, f32::min / f32::max) on the device, after each upload: block b
// folds vertices b, b + nb, ... into part[b]; one block then folds the
// parts into out.  min/max ignore a NaN operand and their result does not
// depend on the order (up to the sign of a zero, which no cull test sees).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bbox_part(const float *__restrict__ verts, uint32_t nverts,
                                                   uint32_t stride, float *__restrict__ part) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nverts; i += gridDim.x * blockDim.x) {
        const float *v = verts + (size_t)i * stride;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], v[k]);
            hi[k] = fmaxf(hi[k], v[k]);
        }
    }
    __shared__ float red[6][8];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], o));
        }
        if (lane == 0) {
            red[k][w] = lo[k];
            red[3 + k][w] = hi[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        float r = red[threadIdx.x][0];
        for (uint32_t j = 1; j < blockDim.x / 32; ++j)
            r = threadIdx.x < 3 ? fminf(r, red[threadIdx.x][j]) : fmaxf(r, red[threadIdx.x][j]);
        part[blockIdx.x * 6 + threadIdx.x] = r;
    }
}
__global__ void k_bbox_fold(const float *__restrict__ part, uint32_t nb, float *__restrict__ out) {
    if (threadIdx.x < 6) {
        float r = threadIdx.x < 3 ? INFINITY : -INFINITY;
        for (uint32_t b = 0; b < nb; ++b)
            r = threadIdx.x < 3 ? fminf(r, part[b * 6 + threadIdx.x]) : fmaxf(r, part[b * 6 + threadIdx.x]);
        out[threadIdx.x] = r;
    }
}

// ---------------------------------------------------------------------------
// K0: object-level frustum culling (render/scene.rs:80-87 BBox::visibility
// as the per-object loop of demos/src/bin/crates.rs:114-133 uses it): one
// thread per draw with RF_DRAW_CULL_BBOX.  The bbox corners in BBox::verts
// order go through the draw's vertex transform; all eight outside one plane
// (view_frustum::status == Hidden, clip.rs:245-267) culls the draw.
// ---------------------------------------------------------------------------
__global__ void k_cull(DrawDev *__restrict__ draws, uint32_t nd, StatsDev *__restrict__ stats) {
    for (uint32_t di = blockIdx.x * blockDim.x + threadIdx.x; di < nd; di += gridDim.x * blockDim.x) {
        DrawDev &d = draws[di];
        d.culled = 0;
        if (!(d.flags & RF_K_DRAW_CULL_BBOX) || d.pos_dim != 3) continue;
        uint32_t all = 0x3Fu;
        for (int c = 0; c < 8; ++c) {
            const float h[4] = {d.bbox[(c & 4) ? 3 : 0], d.bbox[(c & 2) ? 4 : 1], d.bbox[(c & 1) ? 5 : 2], 1.0f};
            float p[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) p[r] = dot4(d.mvp + 4 * r, h);
            all &= outcode(p);
        }
        StatsDev &S = stats[d.job];
        atomicAdd(&S.objs_i, 1ull);
        if (all) {
            d.culled = 1;
            atomicAdd(&S.cull_calls, 1ull);
            atomicAdd(&S.cull_prims, (unsigned long long)d.ntri);
            atomicAdd(&S.cull_verts, (unsigned long long)d.nverts);
        } else {
            atomicAdd(&S.objs_o, 1ull);
        }
    }
}

// ---------------------------------------------------------------------------
// K2: per input triangle, frustum status and (for Clipped) the
// Sutherland-Hodgman polygon (clip.rs:167-193, 283-301), stored in the pool.
// tcnt[t] = number of fan triangles; tpoly[t] = pool slot or RF_NO_POLY.
// ---------------------------------------------------------------------------
namespace {
struct CV {
    float pos[4];
    float a[RF_MAX_ATTR];
    uint32_t oc;
};

__device__ int clip_plane(int plane, const CV *in, int nin, CV *out, uint32_t na, bool &ovf) {
    int nout = 0;
    if (nin == 0) return 0;
    const uint32_t bit = 1u << plane;
    for (int i = 0; i < nin; ++i) {
        const CV &v0 = in[i];
        const CV &v1 = in[i + 1 == nin ? 0 : i + 1];
        if ((v0.oc & bit) == 0) {
            if (nout < RF_POLY_CAP) out[nout++] = v0;
            else ovf = true;
        }
        // ClipPlane::intersect (clip.rs:121-145)
        const float d0 = dot4(c_planes[plane], v0.pos);
        const float d1 = dot4(c_planes[plane], v1.pos);
        if (fmul(d0, d1) < 0.0f) {
            const float t = fdiv(-d0, fsub(d1, d0));
            CV v;
#pragma unroll
            for (int c = 0; c < 4; ++c) v.pos[c] = lerp(v0.pos[c], v1.pos[c], t);
            for (uint32_t c = 0; c < na; ++c) v.a[c] = lerp(v0.a[c], v1.a[c], t);
            v.oc = outcode(v.pos);
            if (nout < RF_POLY_CAP) out[nout++] = v;
            else ovf = true;
        }
    }
    return nout;
}
}  // namespace

#define RF_CLIP_THREADS 256u  // k_clip's block
// Classification (clip.rs:245-267 status): one thread per triangle; the
// few that cross a plane go to a queue for k_clip_poly, so the clipping
// loop runs on full warps.
__global__ void k_clip(const DrawDev *__restrict__ draws, uint32_t nd, uint32_t nt_total,
                       const uint8_t *__restrict__ coc, uint32_t *__restrict__ tcnt,
                       uint32_t *__restrict__ tpoly, uint32_t *__restrict__ queue,
                       uint32_t *__restrict__ counters, uint32_t *__restrict__ toff,
                       uint32_t *__restrict__ prim_total) {
    // Block-uniform loop (the draw lookup is shared by a warp's lanes, the
    // output slots are taken once per block).
    __shared__ uint32_t wslot[2][RF_CLIP_THREADS / 32];
    uint32_t buf = 0;
    for (uint32_t bbase = blockIdx.x * blockDim.x; bbase < nt_total; bbase += gridDim.x * blockDim.x) {
        const uint32_t gt = bbase + threadIdx.x;
        const uint32_t di = warp_upper_index(nd, gt < nt_total ? gt : nt_total - 1,
                                             [&](uint32_t i) { return draws[i].tri_base; });
        bool clipped = false;
        uint32_t cnt = 0;
        if (gt < nt_total) {
            const DrawDev &d = draws[di];
            if (!d.culled) {  // (a culled draw is a render() call that is not made: no output)
                const uint32_t t = gt - d.tri_base;
                uint32_t vi[3];
                bool bad = false;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    vi[k] = d.idx[3 * (size_t)t + k];
                    bad |= vi[k] >= d.nverts;
                }
                if (bad) {
                    atomicAdd(&counters[RF_CNT_BADIDX], 1u);  // index out of range (render.rs:170 panics)
                } else {
                    const uint32_t o0 = coc[vi[0] + d.vert_base], o1 = coc[vi[1] + d.vert_base],
                                   o2 = coc[vi[2] + d.vert_base];
                    if ((o0 & o1 & o2) != 0u) cnt = 0;       // Hidden
                    else if ((o0 | o1 | o2) == 0u) cnt = 1;  // Visible
                    else clipped = true;
                }
            }
            tcnt[gt] = cnt;
            tpoly[gt] = clipped ? di : RF_NO_POLY;  // (a queued triangle's draw, for k_clip_poly)
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, clipped);
        if (bal) {
            const uint32_t lane = threadIdx.x & 31u, lead = __ffs(bal) - 1;
            uint32_t at = 0;
            if (lane == lead) at = atomicAdd(&counters[RF_CNT_CLIPQ], (uint32_t)__popc(bal));
            at = __shfl_sync(0xFFFFFFFFu, at, lead);
            if (clipped) queue[at + __popc(bal & ((1u << lane) - 1u))] = gt;
        }
        if (prim_total) {
            // The triangle's output slots: one for a visible triangle, a
            // whole fan's worth (RF_MAX_FAN, of which k_clip_poly fills the
            // first tcnt) for one that crosses a plane, consecutive over the
            // block and taken from the frame's running total with one atomic
            // per block (one per warp contends on the counter in frames of
            // millions of triangles).
            const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
            const uint32_t vis = __ballot_sync(0xFFFFFFFFu, cnt != 0u);
            const uint32_t lt = (1u << lane) - 1u;
            if (lane == 0) wslot[buf][w] = __popc(vis) + RF_MAX_FAN * __popc(bal);
            __syncthreads();
            if (w == 0) {
                const uint32_t v = lane < RF_CLIP_THREADS / 32 ? wslot[buf][lane] : 0u;
                uint32_t incl = v;
#pragma unroll
                for (uint32_t o = 1; o < RF_CLIP_THREADS / 32; o <<= 1) {
                    const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= o) incl += x;
                }
                const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, RF_CLIP_THREADS / 32 - 1);
                uint32_t at = 0;
                if (lane == 0 && total) at = atomicAdd(prim_total, total);
                at = __shfl_sync(0xFFFFFFFFu, at, 0);
                if (lane < RF_CLIP_THREADS / 32) wslot[buf][lane] = at + incl - v;
            }
            __syncthreads();
            if (cnt || clipped)
                toff[gt] = wslot[buf][w] + __popc(vis & lt) + RF_MAX_FAN * __popc(bal & lt);
            buf ^= 1u;  // (the other buffer next: no third barrier)
        }
    }
}

// Sutherland-Hodgman for the queued triangles (clip.rs:283-301, 350-400):
// sixteen lanes per triangle, two triangles per warp, lane j holding polygon
// vertex j.  Per plane each lane tests its vertex and its edge to vertex
// j + 1 (the same operations as ClipPlane::clip_simple_polygon), a prefix
// count over the group gives every output vertex its slot, and each lane
// fetches its new vertex -- the kept vertex or the edge's intersection --
// from the lane that produced it.  The output order is the reference's:
// per edge in order, the kept start vertex, then the intersection.
__device__ __forceinline__ void clip_groups(const DrawDev *__restrict__ draws, const float4 *__restrict__ cpos,
                                            const uint8_t *__restrict__ coc, uint32_t *__restrict__ tcnt,
                                            uint32_t *__restrict__ tpoly, const uint32_t *__restrict__ queue,
                                            PolyVert *__restrict__ pool, uint32_t pool_cap,
                                            uint32_t *__restrict__ counters, uint32_t nq) {
    constexpr uint32_t FULL = 0xFFFFFFFFu;
    static_assert(RF_POLY_CAP == 16, "one 16-lane group holds a polygon");
    const uint32_t lane = threadIdx.x & 31u, j = lane & 15u, gb = lane & 16u;
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t qb = wid * 2u; qb < nq; qb += nw * 2u) {  // warp-uniform
        const uint32_t qi = qb + (gb >> 4);
        const bool have = qi < nq;
        const uint32_t gt = have ? queue[qi] : 0u;
        const uint32_t di = have ? tpoly[gt] : 0u;  // k_clip left the draw index there
        const DrawDev &d = draws[di];
        const uint32_t na = have ? (d.nattr < RF_MAX_ATTR ? d.nattr : RF_MAX_ATTR) : 0u;
        float pos[4] = {0.0f, 0.0f, 0.0f, 1.0f}, a[RF_MAX_ATTR];
#pragma unroll
        for (int c = 0; c < RF_MAX_ATTR; ++c) a[c] = 0.0f;
        uint32_t oc = 0;
        if (have && j < 3u) {
            const uint32_t vi = d.idx[3 * (size_t)(gt - d.tri_base) + j] + d.vert_base;
            const float4 p = cpos[vi];
            pos[0] = p.x; pos[1] = p.y; pos[2] = p.z; pos[3] = p.w;
            const float *src = d.verts + (size_t)(vi - d.vert_base) * d.stride + d.pos_dim;
#pragma unroll
            for (int c = 0; c < RF_MAX_ATTR; ++c)
                if ((uint32_t)c < na) a[c] = src[c];
            oc = coc[vi];
        }
        uint32_t n = have ? 3u : 0u;
        bool ovf = false;
        for (int pl = 0; pl < 6; ++pl) {
            const bool act = j < n;
            const float dd = act ? dot4(c_planes[pl], pos) : 0.0f;
            const bool in = act && (oc & (1u << pl)) == 0u;
            // The edge to the next vertex (the first one closes the polygon).
            const uint32_t nb = gb + (j + 1u < n ? j + 1u : 0u);
            const float d1 = __shfl_sync(FULL, dd, nb);
            float p1[4], a1[RF_MAX_ATTR];
#pragma unroll
            for (int c = 0; c < 4; ++c) p1[c] = __shfl_sync(FULL, pos[c], nb);
#pragma unroll
            for (int c = 0; c < RF_MAX_ATTR; ++c) a1[c] = __shfl_sync(FULL, a[c], nb);
            const bool cross = act && fmul(dd, d1) < 0.0f;  // ClipPlane::intersect (clip.rs:121-145)
            float xp[4] = {0.0f, 0.0f, 0.0f, 0.0f}, xa[RF_MAX_ATTR];
#pragma unroll
            for (int c = 0; c < RF_MAX_ATTR; ++c) xa[c] = 0.0f;
            uint32_t xoc = 0;
            if (cross) {
                const float t = fdiv(-dd, fsub(d1, dd));
#pragma unroll
                for (int c = 0; c < 4; ++c) xp[c] = lerp(pos[c], p1[c], t);
#pragma unroll
                for (int c = 0; c < RF_MAX_ATTR; ++c)
                    if ((uint32_t)c < na) xa[c] = lerp(a[c], a1[c], t);
                xoc = outcode(xp);
            }
            // Slots: an inclusive count over the group, then each output slot
            // k = j finds the first lane whose count exceeds k.
            const uint32_t cnt = (in ? 1u : 0u) + (cross ? 1u : 0u);
            uint32_t incl = cnt;
#pragma unroll
            for (uint32_t o = 1; o < 16u; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, o, 16);
                if (j >= o) incl += y;
            }
            const uint32_t total = __shfl_sync(FULL, incl, gb + 15u);
            uint32_t sl = 0;
#pragma unroll
            for (uint32_t step = 8; step >= 1; step >>= 1) {
                const uint32_t v = __shfl_sync(FULL, incl, gb + sl + step - 1u);
                if (v <= j) sl += step;
            }
            const uint32_t src = gb + sl;
            const uint32_t ex = __shfl_sync(FULL, incl - cnt, src);
            const bool keep0 = __shfl_sync(FULL, in ? 1u : 0u, src) != 0u && j == ex;
            float np_[4], na_[RF_MAX_ATTR];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float kv = __shfl_sync(FULL, pos[c], src), xv = __shfl_sync(FULL, xp[c], src);
                np_[c] = keep0 ? kv : xv;
            }
#pragma unroll
            for (int c = 0; c < RF_MAX_ATTR; ++c) {
                const float kv = __shfl_sync(FULL, a[c], src), xv = __shfl_sync(FULL, xa[c], src);
                na_[c] = keep0 ? kv : xv;
            }
            const uint32_t ko = __shfl_sync(FULL, oc, src), xo = __shfl_sync(FULL, xoc, src);
            oc = keep0 ? ko : xo;
#pragma unroll
            for (int c = 0; c < 4; ++c) pos[c] = np_[c];
#pragma unroll
            for (int c = 0; c < RF_MAX_ATTR; ++c) a[c] = na_[c];
            if (total > RF_POLY_CAP) ovf = true;  // more vertices than the working buffer keeps
            n = total < RF_POLY_CAP ? total : RF_POLY_CAP;
        }
        if (n > RF_POLY_STORE) ovf = true;
        if (ovf) n = 0;  // only float pathologies get here; counted in stats.oob, dropped
        uint32_t cntf = n >= 3u ? n - 2u : 0u, slot = RF_NO_POLY;
        if (j == 0u && have) {
            if (ovf) atomicAdd(&counters[RF_CNT_POLYOVF], 1u);
            if (cntf) {
                slot = atomicAdd(&counters[RF_CNT_POOL], 1u);
                if (slot >= pool_cap) {
                    atomicAdd(&counters[RF_CNT_POOLOVF], 1u);
                    slot = RF_NO_POLY;
                }
            }
        }
        slot = __shfl_sync(FULL, slot, gb);
        if (slot == RF_NO_POLY) cntf = 0;
        if (have && slot != RF_NO_POLY && j < n) {
            PolyVert *dst = pool + (size_t)slot * RF_POLY_STORE + j;
#pragma unroll
            for (int c = 0; c < 4; ++c) dst->pos[c] = pos[c];
#pragma unroll
            for (int c = 0; c < RF_MAX_ATTR; ++c)
                if ((uint32_t)c < na) dst->a[c] = a[c];
        }
        if (have && j == 0u) {
            tcnt[gt] = cntf;
            tpoly[gt] = slot;
        }
    }
}

// The same, one thread per triangle: for long queues, where whole warps of
// triangles keep the SMs busy and the per-lane work of the groups would
// cost more issue slots than it saves latency.
__device__ __forceinline__ void clip_threads(const DrawDev *__restrict__ draws, const float4 *__restrict__ cpos,
                                             const uint8_t *__restrict__ coc, uint32_t *__restrict__ tcnt,
                                             uint32_t *__restrict__ tpoly, const uint32_t *__restrict__ queue,
                                             PolyVert *__restrict__ pool, uint32_t pool_cap,
                                             uint32_t *__restrict__ counters, uint32_t nq) {
    for (uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x; qi < nq; qi += gridDim.x * blockDim.x) {
        const uint32_t gt = queue[qi];
        const DrawDev &d = draws[tpoly[gt]];  // k_clip left the draw index there
        const uint32_t t = gt - d.tri_base;
        uint32_t vi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) vi[k] = d.idx[3 * (size_t)t + k] + d.vert_base;
        CV A[RF_POLY_CAP], B[RF_POLY_CAP];
        const uint32_t na = d.nattr < RF_MAX_ATTR ? d.nattr : RF_MAX_ATTR;
        for (int k = 0; k < 3; ++k) {
            const float4 p = cpos[vi[k]];
            A[k].pos[0] = p.x; A[k].pos[1] = p.y; A[k].pos[2] = p.z; A[k].pos[3] = p.w;
            const float *src = d.verts + (size_t)(vi[k] - d.vert_base) * d.stride + d.pos_dim;
            for (uint32_t c = 0; c < na; ++c) A[k].a[c] = src[c];
            A[k].oc = coc[vi[k]];
        }
        CV *vin = A, *vout = B;
        int nin = 3, nout = 0;
        bool ovf = false;
        for (int pl = 0; pl < 6; ++pl) {
            nout = clip_plane(pl, vin, nin, vout, na, ovf);
            nin = 0;
            if (nout == 0) break;
            if (pl < 5) {
                CV *tmp = vin; vin = vout; vout = tmp;
                nin = nout; nout = 0;
            }
        }
        if (nout > RF_POLY_STORE) ovf = true;
        if (ovf) {
            // Only reachable through float pathologies (a convex triangle
            // gains at most one vertex per plane); counted in stats.oob and
            // dropped.
            atomicAdd(&counters[RF_CNT_POLYOVF], 1u);
            nout = 0;
        }
        uint32_t cnt = nout >= 3 ? (uint32_t)(nout - 2) : 0u, slot = RF_NO_POLY;
        if (cnt) {
            slot = atomicAdd(&counters[RF_CNT_POOL], 1u);
            if (slot < pool_cap) {
                PolyVert *dst = pool + (size_t)slot * RF_POLY_STORE;
                for (int k = 0; k < nout; ++k) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) dst[k].pos[c] = vout[k].pos[c];
                    for (uint32_t c = 0; c < na; ++c) dst[k].a[c] = vout[k].a[c];
                }
            } else {
                atomicAdd(&counters[RF_CNT_POOLOVF], 1u);
                cnt = 0;
                slot = RF_NO_POLY;
            }
        }
        tcnt[gt] = cnt;
        tpoly[gt] = slot;
    }
}

#define RF_CLIP_GROUP_MAX 32768u  // queues up to this long are clipped by lane groups
__global__ void __launch_bounds__(256)
k_clip_poly(const DrawDev *__restrict__ draws, const float4 *__restrict__ cpos,
            const uint8_t *__restrict__ coc, uint32_t *__restrict__ tcnt,
            uint32_t *__restrict__ tpoly, const uint32_t *__restrict__ queue,
            PolyVert *__restrict__ pool, uint32_t pool_cap, uint32_t *__restrict__ counters) {
    const uint32_t nq = counters[RF_CNT_CLIPQ];
    if (nq <= RF_CLIP_GROUP_MAX) clip_groups(draws, cpos, coc, tcnt, tpoly, queue, pool, pool_cap, counters, nq);
    else clip_threads(draws, cpos, coc, tcnt, tpoly, queue, pool, pool_cap, counters, nq);
}

// ---------------------------------------------------------------------------
// Exclusive scan of tcnt (order-preserving compaction of the clipped
// triangles: output prim order == clipped order of render.rs:184-205).
// ---------------------------------------------------------------------------
#define SCAN_THREADS 1024
#define SCAN_ITEMS 4
static_assert(SCAN_THREADS * SCAN_ITEMS == RF_SCAN_BLOCK_ITEMS, "scan block size");
// Exclusive scan of each block's SCAN_THREADS * SCAN_ITEMS values; the block
// totals go to block_sums, and with a single block the total to *total.
__global__ void k_scan_blocks(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                              uint32_t n, uint32_t *__restrict__ block_sums,
                              uint32_t *__restrict__ total) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t base = blockIdx.x * (SCAN_THREADS * SCAN_ITEMS) + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = base + i < n ? in[base + i] : 0u;
        s += v[i];
    }
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t ws = warp_sums[lane], wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= (uint32_t)o) wi += y;
        }
        warp_sums[lane] = wi - ws;
        if (lane == 31) {
            block_sums[blockIdx.x] = wi;
            if (gridDim.x == 1) *total = wi;
        }
    }
    __syncthreads();
    uint32_t run = warp_sums[wid] + incl - s;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

// Single block: exclusive scan of the block sums in place; total -> *total.
__global__ void k_scan_sums(uint32_t *__restrict__ sums, uint32_t nb, uint32_t *__restrict__ total) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nb; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t s = i < nb ? sums[i] : 0u;
        uint32_t incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t ws = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0u, wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
                if (lane >= (uint32_t)o) wi += y;
            }
            warp_sums[lane] = wi - ws;
        }
        __syncthreads();
        const uint32_t excl = carry + warp_sums[wid] + incl - s;
        if (i < nb) sums[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + s;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(uint32_t *__restrict__ out, uint32_t n, const uint32_t *__restrict__ sums) {
    const uint32_t base = blockIdx.x * (SCAN_THREADS * SCAN_ITEMS) + threadIdx.x * SCAN_ITEMS;
    const uint32_t add = sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i)
        if (base + i < n) out[base + i] += add;
}

// ---------------------------------------------------------------------------
// K3: triangle setup.
// ---------------------------------------------------------------------------
namespace {
struct SV {  // screen-space vertex: (ScreenPt, V) without the unused y step
    float x, y;
    float c[RF_NC];  // c[0] = screen z (1/w), c[1..] = attributes
};

// raster.rs:248-302 scan(): fills one HalfRec.
__device__ void scan_setup(float y0, float y1, const SV &l0, const SV &l1, const SV &r0,
                           const SV &r1, uint32_t nc, HalfRec &h) {
    const float recip_dy = fdiv(1.0f, fsub(y1, y0));
    const float dlx = fmul(fsub(l1.x, l0.x), recip_dy);
    const float drx = fmul(fsub(r1.x, r0.x), recip_dy);
    const float dx = fsub(fadd(r0.x, drx), fadd(l0.x, dlx));
    const float rdx = fdiv(1.0f, dx);
    const float y0r = round_up_to_half(y0);
    const float y1r = round_up_to_half(y1);
    const float yt = fsub(y0r, y0);
    h.y0r = y0r;
    h.n = as_u32(fsub(y1r, y0r));
    float st[RF_NR];
    h.d[RF_R_LX] = dlx;
    h.d[RF_R_RX] = drx;
    st[RF_R_LX] = fadd(l0.x, fmul(fsub(fadd(l0.x, dlx), l0.x), yt));
    st[RF_R_RX] = fadd(r0.x, fmul(drx, yt));
    for (uint32_t c = 0; c < RF_NC; ++c) {
        if (c < nc) {
            const float dl = fmul(fsub(l1.c[c], l0.c[c]), recip_dy);
            const float dr = fmul(fsub(r1.c[c], r0.c[c]), recip_dy);
            const float l0s = fadd(l0.c[c], dl), r0s = fadd(r0.c[c], dr);
            h.d[RF_R_C + c] = dl;
            h.dvdx[c] = fmul(fsub(r0s, l0s), rdx);
            st[RF_R_C + c] = fadd(l0.c[c], fmul(fsub(fadd(l0.c[c], dl), l0.c[c]), yt));
        } else {
            h.d[RF_R_C + c] = 0.0f;
            h.dvdx[c] = 0.0f;
            st[RF_R_C + c] = 0.0f;
        }
    }
    for (uint32_t r = 0; r < RF_NR; ++r) h.b0[r] = f2u(st[r]);
}

// The two binade runs of row quantity r of a half whose start (b0) and
// step (d) are set: run 0 from the first row, run 1 after one explicit
// addition (rfd::row_value reads them).  Needed only by triangles
// rasterised without row records.
__device__ void half_runs(const HalfRec &h, HalfRuns &u, uint32_t r) {
    uint32_t k0, k1;
    int32_t i0, i1;
    fast_params(u2f(h.b0[r]), h.d[r], i0, k0);
    u.i0[r] = i0;
    u.e0[r] = k0;
    if (k0 == 0xFFFFFFFFu) {  // fixed point: run 0 covers every row
        u.b1[r] = h.b0[r];
        u.i1[r] = 0;
        u.e1[r] = k0;
        return;
    }
    const float v1 = fadd(u2f(h.b0[r] + k0 * (uint32_t)i0), h.d[r]);
    fast_params(v1, h.d[r], i1, k1);
    u.i1[r] = i1;
    u.b1[r] = f2u(v1);
    const uint64_t e1 = (uint64_t)k0 + 1u + k1;
    u.e1[r] = e1 > 0xFFFFFFFEull ? 0xFFFFFFFEu : (uint32_t)e1;
}

}  // namespace

#define RF_SETUP_THREADS 64
__global__ void __launch_bounds__(RF_SETUP_THREADS)
k_setup(const DrawDev *__restrict__ draws, uint32_t nd,
                        const JobDev *__restrict__ jobs, uint32_t nt_total,
                        const float4 *__restrict__ cpos, const uint32_t *__restrict__ tcnt,
                        const uint32_t *__restrict__ toff, const uint32_t *__restrict__ tpoly,
                        const PolyVert *__restrict__ pool, PrimRec *__restrict__ prims,
                        unsigned long long *__restrict__ rows_total, RasterPrim *__restrict__ rprims,
                        uint32_t *__restrict__ live, uint32_t *__restrict__ live_n,
                        uint32_t *__restrict__ live_small, uint32_t *__restrict__ live_small_n,
                        uint32_t *__restrict__ live_mid, uint32_t *__restrict__ live_mid_n,
                        uint32_t *__restrict__ extra, StatsDev *__restrict__ stats,
                        const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ptri) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *extra = 0;  // the work list's counter
    // Each thread builds its record in shared memory; the warp then writes
    // the records out with coalesced 16-byte stores.  Only triangles that
    // pass the face-cull test get a record, and their indices are appended
    // to the live list the binning pass walks.
    // (the record's first RF_PRIM_CORE_BYTES only: the binade runs, needed
    // by few triangles, go straight to global memory)
    __shared__ __align__(16) uint4 sbuf[RF_SETUP_THREADS][RF_PRIM_CORE_BYTES / 16];
    const uint32_t lane = threadIdx.x & 31, wbase = threadIdx.x & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    // Depth-sorted frames (perm != nullptr): thread gt is the gt-th clipped
    // triangle in sorted order, perm[gt] its index in clipped order, ptri
    // the input triangle it came from; the draws' tri_base / ntri count
    // clipped triangles then, and src_tri_base locates the input ones.
    for (uint32_t base = blockIdx.x * blockDim.x; base < nt_total; base += stride) {
        const uint32_t gt = base + threadIdx.x;
        const bool active = gt < nt_total;
        const uint32_t cnt = active ? (perm ? 1u : tcnt[gt]) : 0u;
        uint32_t job = 0xFFFFFFFFu;
        unsigned long long prims_o = 0;
        uint32_t di = 0, t = 0, nc = 0, na = 0, zm = 0, slot = RF_NO_POLY, p0 = 0, fan0 = 0;
        const uint32_t dwarp = warp_upper_index(nd, active ? gt : nt_total - 1,
                                                [&](uint32_t i) { return draws[i].tri_base; });
        if (cnt) {
            di = dwarp;
            job = draws[di].job;
            nc = 1 + nattr_of(draws[di].shader);
            na = nc - 1;
            zm = zdiv_mask_of(draws[di].shader);
            if (perm) {
                const uint32_t pc = perm[gt], tin = ptri[pc];
                t = tin - draws[di].src_tri_base;
                slot = tpoly[tin];
                fan0 = pc - toff[tin];
                p0 = gt;
            } else {
                t = gt - draws[di].tri_base;
                slot = tpoly[gt];
                p0 = toff[gt];
            }
        }
        const uint32_t maxc = __reduce_max_sync(0xFFFFFFFFu, cnt);
        for (uint32_t c = 0; c < maxc; ++c) {
            const bool have = c < cnt;
            bool keep = false;  // passes the face-cull test
            uint32_t list = 0;  // ... and its binning list: 0 k_bin, 1 / 2 k_bin_small (8 / 16 lanes)
            if (have) {
                const DrawDev &d = draws[di];
                const JobDev &J = jobs[job];
                // Gather the three clip-space vertices of this (fan) triangle.
                float pos[3][4], at[3][RF_MAX_ATTR];
                for (int k = 0; k < 3; ++k) {
                    if (slot == RF_NO_POLY) {
                        const uint32_t li = d.idx[3 * (size_t)t + k];
                        const float4 p = cpos[d.vert_base + li];
                        pos[k][0] = p.x; pos[k][1] = p.y; pos[k][2] = p.z; pos[k][3] = p.w;
                        const float *src = d.verts + (size_t)li * d.stride + d.pos_dim;
                        for (uint32_t a = 0; a < na; ++a) at[k][a] = src[a];
                    } else {
                        const PolyVert &v = pool[(size_t)slot * RF_POLY_STORE + (k == 0 ? 0 : fan0 + c + k)];
#pragma unroll
                        for (int q = 0; q < 4; ++q) pos[k][q] = v.pos[q];
                        for (uint32_t a = 0; a < na; ++a) at[k][a] = v.a[a];
                    }
                }
                // prim.rs:62-88 to_screen + viewport (mat.rs:945-949).
                SV sv[3];
                for (int k = 0; k < 3; ++k) {
                    const float w = pos[k][3];
                    const float ndc[4] = {fdiv(pos[k][0], w), fdiv(pos[k][1], w), fdiv(1.0f, w), 1.0f};
                    sv[k].x = dot4(J.vp + 0, ndc);
                    sv[k].y = dot4(J.vp + 4, ndc);
                    sv[k].c[0] = dot4(J.vp + 8, ndc);
                    for (uint32_t a = 0; a < RF_MAX_ATTR; ++a)
                        sv[k].c[1 + a] = a < na ? (((zm >> a) & 1u) ? fdiv(at[k][a], w) : at[k][a]) : 0.0f;
                }
                // Winding (geom/prim.rs:152-156, 288-294) and face_cull (ctx.rs:95-101).
                const float ux = fsub(sv[1].x, sv[0].x), uy = fsub(sv[1].y, sv[0].y);
                const float vx = fsub(sv[2].x, sv[0].x), vy = fsub(sv[2].y, sv[0].y);
                const float wz = fadd(fadd(0.0f, fmul(-uy, vx)), fmul(ux, vy));
                const bool backface = wz < 0.0f;
                const bool culled = (J.face_cull == RF_K_CULL_BACK && backface) ||
                                    (J.face_cull == RF_K_CULL_FRONT && !backface);
                keep = !culled;
                if (culled && cnt > 1) {
                    // A piece of a clipped triangle: the rasteriser walks
                    // every piece of a triangle it meets and skips this one.
                    RasterPrim *R = rprims + p0 + c;
                    R->draw = di;
                    R->flags = 0u;
                    R->kind = d.shader;
                    R->zmax = __int_as_float(0x7F800000);
                }
                if (!culled) {
                // This thread's slot: the fields before `runs` only.
                PrimRec &P = *reinterpret_cast<PrimRec *>(sbuf[threadIdx.x]);
                P.draw = di;
                P.live = 1u;
                P.tri = gt;
                P.kind = d.shader;
                P.rloc = 0;
                P.rwords = 0;
                P.job = job;
                prims_o += 1;
                // raster.rs:185-224 tri_fill: stable sort by y (total_cmp).
                SV v0 = sv[0], v1 = sv[1], v2 = sv[2], tmp;
                if (total_key(v0.y) > total_key(v1.y)) { tmp = v0; v0 = v1; v1 = tmp; }
                if (total_key(v1.y) > total_key(v2.y)) { tmp = v1; v1 = v2; v2 = tmp; }
                if (total_key(v0.y) > total_key(v1.y)) { tmp = v0; v0 = v1; v1 = tmp; }
                const float tt = fdiv(fsub(v1.y, v0.y), fsub(v2.y, v0.y));
                SV mid1;
                mid1.x = lerp(v0.x, v2.x, tt);
                mid1.y = v1.y;
                for (uint32_t q = 0; q < RF_NC; ++q) mid1.c[q] = lerp(v0.c[q], v2.c[q], tt);
                const bool mid0_left = v1.x < mid1.x;
                const SV &left = mid0_left ? v1 : mid1;
                const SV &right = mid0_left ? mid1 : v1;
                scan_setup(v0.y, v1.y, v0, left, v0, right, nc, P.half[0]);
                scan_setup(v1.y, v2.y, left, v2, right, v2, nc, P.half[1]);
                // Row records for the scanlines that land on the target's
                // rows, unless a half starts above the buffer (its rows map
                // onto row 0 several times: rasterised from this record).
                uint32_t rows = 0;
                bool regular = true;
                for (int hh = 0; hh < 2; ++hh) {
                    const HalfRec &H = P.half[hh];
                    if (H.n == 0 || !(fabsf(H.y0r) < RF_MAX_COORD)) continue;
                    const int32_t Y = (int32_t)fsub(H.y0r, 0.5f);
                    if (Y < 0) regular = false;
                    const int64_t in = min((int64_t)H.n, max((int64_t)0, (int64_t)J.h - Y));
                    rows += (uint32_t)in;
                }
                const uint64_t w = regular ? (uint64_t)rows * (1u + 2u * nc) : 0u;
                if (w < 0x40000000ull) P.rwords = (uint32_t)w;
                if (P.rwords != 0u) list = rows <= 8u ? 1u : rows <= 16u ? 2u : 0u;
                if (P.rwords == 0u) {  // rasterised from this record: it needs the runs
                    PrimRec *G = prims + p0 + c;
                    for (int hh = 0; hh < 2; ++hh)
                        for (uint32_t r = 0; r < RF_NR; ++r) half_runs(P.half[hh], G->runs[hh], r);
                }
                }
            }
            __syncwarp();
            // Room for this step's row records: one atomic per warp on the
            // frame's running total, each lane's block after the lower
            // lanes' (the records' place in the buffer is free; each
            // triangle's own records stay contiguous).  An offset past 32
            // bits is clamped, so the binning pass finds no room for it.
            {
                PrimRec &P = *reinterpret_cast<PrimRec *>(sbuf[threadIdx.x]);
                const unsigned long long w = keep ? P.rwords : 0u;
                unsigned long long incl = w;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= (uint32_t)o) incl += y;
                }
                const unsigned long long total = __shfl_sync(0xFFFFFFFFu, incl, 31);
                unsigned long long at = 0;
                if (total && lane == 0) at = atomicAdd(rows_total, total);
                at = __shfl_sync(0xFFFFFFFFu, at, 0) + (incl - w);
                if (w) P.rloc = at < 0xFFFFFFFFull ? (uint32_t)at : 0xFFFFFFFFu;
            }
            __syncwarp();
            uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
            const uint32_t dst = p0 + c;
            // Append this step's live triangles to their lists.
            for (uint32_t which = 0; which < 3; ++which) {
                const uint32_t b = __ballot_sync(0xFFFFFFFFu, keep && list == which);
                if (!b) continue;
                uint32_t *cnt_w = which == 0 ? live_n : which == 1 ? live_small_n : live_mid_n;
                uint32_t *list_w = which == 0 ? live : which == 1 ? live_small : live_mid;
                const uint32_t lead = __ffs(b) - 1;
                uint32_t at = 0;
                if (lane == lead) at = atomicAdd(cnt_w, (uint32_t)__popc(b));
                at = __shfl_sync(0xFFFFFFFFu, at, lead);
                if ((b >> lane) & 1u) list_w[at + __popc(b & ((1u << lane) - 1u))] = dst;
            }
            // Write out the records built in this step, one per pass.
            while (bal) {
                const uint32_t l = __ffs(bal) - 1;
                bal &= bal - 1;
                const uint32_t dl = __shfl_sync(0xFFFFFFFFu, dst, l);
                const uint4 *src = sbuf[wbase + l];
                uint4 *out = reinterpret_cast<uint4 *>(prims + dl);
                if (lane < RF_PRIM_CORE_BYTES / 16) out[lane] = src[lane];
            }
            __syncwarp();
        }
        // Stats, aggregated per warp when all lanes share one job.
        const uint32_t hasjob = __ballot_sync(0xFFFFFFFFu, job != 0xFFFFFFFFu);
        if (hasjob) {
            const uint32_t j0 = __shfl_sync(0xFFFFFFFFu, job, __ffs(hasjob) - 1);
            const bool same = __all_sync(0xFFFFFFFFu, job == j0 || job == 0xFFFFFFFFu);
            if (same || job != 0xFFFFFFFFu) {
                StatsDev *S = stats + (same ? j0 : job);
                warp_add_u64(&S->prims_o, prims_o, same);
                warp_add_u64(&S->verts_o, 3ull * prims_o, same);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// K3b: scanline statistics and tile binning, one warp per triangle.
// For every scanline of both halves (ScanlineIter::next, raster.rs:80-114)
// the lane owning that row computes the exact edge values (closed-form run or
// the general loop), then frags.i / oob as rasterize_fb counts them
// (target.rs:259-264) and the pixel columns it covers; a warp reduction per
// 32-row band gives the tiles to mark in the job's bitmask.
// ---------------------------------------------------------------------------
namespace {

// k steps of Iter::next on the first N components, side by side.
template <int N>
__device__ __forceinline__ void step_k(float *v, const float *d, uint32_t k) {
    uint32_t i = 0;
    for (; i + 4u <= k; i += 4u) {  // four additions per trip, the same sequence
#pragma unroll
        for (int c = 0; c < N; ++c) v[c] = fadd(fadd(fadd(fadd(v[c], d[c]), d[c]), d[c]), d[c]);
    }
    for (; i < k; ++i) {
#pragma unroll
        for (int c = 0; c < N; ++c) v[c] = fadd(v[c], d[c]);
    }
}

struct RowOut {
    unsigned long long frags_i;
    uint32_t oob;
    uint32_t px0, px1;  // covered pixel columns [px0, px1), px0 >= px1 if none
};

// Scanline j of half H landing on row y (< h).
__device__ __forceinline__ void row_stats(const HalfRec *__restrict__ H, const HalfRuns *__restrict__ U,
                                          uint32_t j, uint32_t w, RowOut &o) {
    const float lx = row_value(H, U, RF_R_LX, j);
    const float rx = row_value(H, U, RF_R_RX, j);
    const float x0r = round_up_to_half(lx), x1r = round_up_to_half(rx);
    const uint64_t xs = as_usize(x0r);
    uint64_t xe = as_usize(x1r);
    if (xe < xs) xe = xs;
    o.frags_i += xe - xs;
    if (xe > w) o.oob += 1;
    uint64_t nfr = xe - xs;
    const uint32_t cnt = as_u32(fsub(x1r, x0r));
    if (cnt < nfr) nfr = cnt;
    if (nfr && xs < w) {
        o.px0 = min(o.px0, (uint32_t)xs);
        o.px1 = max(o.px1, (uint32_t)(xs + nfr < w ? xs + nfr : w));
    }
}

// An upper bound of every running sum z_k = z_{k-1} + dz (k < n) of a
// span starting at z_0 (raster.rs:60-69 / vary.rs:142-155): with dz <= 0
// the sums never rise, so z_0 itself; with dz > 0, z_0 >= 1e-30 and n <=
// 2^20 every sum is within (1 + 2^-24)^k of z_0 + k dz and the computed
// e = fl(z_0 + fl((n - 1) dz)) within (1 - 2^-24)^2 of it, so e times
// 1 + (n + 5) 2^-23 (exact in f32), rounded, bounds them all.  Otherwise
// +inf (no bound); NaN inputs give +inf too.
__device__ __forceinline__ float span_depth_bound(float z0, float dz, uint32_t n) {
    const float inf = __int_as_float(0x7F800000);
    if (n == 0) return -inf;
    if (!(fabsf(z0) < inf) || dz != dz) return inf;
    if (dz <= 0.0f) return z0;
    if (!(z0 >= 1e-30f) || n > (1u << 20) || !(dz < inf)) return inf;
    const float e = fadd(z0, fmul((float)(n - 1u), dz));
    const float f = fadd(1.0f, fmul((float)(n + 5u), 1.1920928955078125e-07f));  // 1 + (n+5) 2^-23
    const float b = fmul(e, f);
    return b == b ? b : inf;
}

// One scanline of a regular triangle (raster.rs:84-113): its span from the
// row's edge values lx, rx (target.rs:259-264 for frags.i / oob), its row
// record at rec -- w0 = first | end << 16 of the covered columns, the
// varyings at the first fragment, then at the span's first tile boundary
// -- and the bound of its depths into zhi.  cv[c * cs] is component c of
// the row's interpolated values; dvh the half's per-pixel steps.
template <int NCT>
__device__ __forceinline__ void row_record(float lx, float rx, const float *cv, uint32_t cs,
                                           const float *dvh, uint32_t nc, uint32_t w, uint32_t tile_w,
                                           uint32_t *rec, RowOut &o, float &zhi) {
    const float x0r = round_up_to_half(lx), x1r = round_up_to_half(rx);
    const uint64_t xs = as_usize(x0r);
    uint64_t xe = as_usize(x1r);
    if (xe < xs) xe = xs;
    o.frags_i = xe - xs;
    if (xe > w) o.oob = 1;
    uint64_t nfr = xe - xs;
    const uint32_t cnt = as_u32(fsub(x1r, x0r));
    if (cnt < nfr) nfr = cnt;
    uint32_t w0 = 0;
    if (nfr && xs < w) {
        o.px0 = (uint32_t)xs;
        o.px1 = (uint32_t)(xs + nfr < w ? xs + nfr : w);
        w0 = o.px0 | (o.px1 << 16);
    }
    rec[0] = w0;
    // v0.lerp(v0.step(dv_dx), x0 - v0.x)  (raster.rs:102), and the
    // varyings at the span's first tile boundary.
    const float tshift = fsub(x0r, lx);
    const uint32_t kb = w0 ? tile_w - (o.px0 & (tile_w - 1u)) : 0u;
    const bool crosses = w0 && o.px0 + kb < o.px1;
    const uint32_t ksteps = crosses ? kb : 0u;  // <= tile width
    // The components step side by side (independent chains), each exactly
    // like Iter::next.
    constexpr uint32_t NCL = NCT ? (uint32_t)NCT : RF_NC;
    float vb[NCL], dvc[NCL];
#pragma unroll
    for (uint32_t c = 0; c < NCL; ++c) {
        if (c < nc) {
            const float v = cv[c * cs];
            dvc[c] = dvh[c];
            vb[c] = fadd(v, fmul(fsub(fadd(v, dvc[c]), v), tshift));
            rec[1 + c] = f2u(vb[c]);
        } else {
            dvc[c] = 0.0f;
            vb[c] = 0.0f;
        }
    }
    if (w0) zhi = fmaxf(zhi, span_depth_bound(vb[0], dvc[0], o.px1 - o.px0));
    if constexpr (NCT != 0) {
        step_k<NCT>(vb, dvc, ksteps);
    } else {
        switch (nc) {  // only the kind's components step
            case 1: step_k<1>(vb, dvc, ksteps); break;
            case 2: step_k<2>(vb, dvc, ksteps); break;
            case 3: step_k<3>(vb, dvc, ksteps); break;
            case 4: step_k<4>(vb, dvc, ksteps); break;
            case 5: step_k<5>(vb, dvc, ksteps); break;
            default: step_k<6>(vb, dvc, ksteps); break;
        }
    }
#pragma unroll
    for (uint32_t c = 0; c < NCL; ++c)
        if (c < nc) rec[1 + nc + c] = f2u(vb[c]);
}

}  // namespace

// NCT: the components (1 + attributes) of every triangle of the launch, or
// 0 when its draws mix shader kinds (taken per triangle).
template <int NCT>
__global__ void __launch_bounds__(256, 4)
k_bin(const DrawDev *__restrict__ draws, const JobDev *__restrict__ jobs,
      PrimRec *__restrict__ prims, const uint32_t *__restrict__ live, uint32_t tile_w,
      uint32_t *__restrict__ rows, unsigned long long rows_cap, RasterPrim *__restrict__ rprims,
      uint32_t *__restrict__ mask, StatsDev *__restrict__ stats, uint32_t *__restrict__ counters,
      unsigned long long *__restrict__ marks) {
    const uint32_t lane = threadIdx.x & 31, wib = (threadIdx.x >> 5) & 7;
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t tw_log2 = __ffs(tile_w) - 1;  // tile widths are powers of two
    // Only the triangles that passed the face-cull test (the live list, in
    // no particular order: every output below depends on the triangle alone).
    const uint32_t nl = counters[RF_CNT_LIVE];
    // Two record slots per warp of the 256-thread block: the next triangle's
    // record is copied (cp.async) while the current one is walked.
    __shared__ __align__(16) uint4 sbuf[8][2][RF_PRIM_CORE_BYTES / 16];  // records' first parts
    __shared__ __align__(16) RasterPrim srp[8];
    // Scanline values of one band: quantity q of the band's row i at
    // [q][i] (rows 16-byte aligned: the walk stores four rows at once).
    __shared__ __align__(16) float stab[8][RF_NR][RF_TILE_H + 4];
    auto fetch = [&](uint4 *dst, uint32_t p, bool ok) {
        if (ok) {
            const char *src = reinterpret_cast<const char *>(prims + p);
            for (uint32_t q = lane; q < RF_PRIM_CORE_BYTES / 16; q += 32) {
                const uint32_t sa = (uint32_t)__cvta_generic_to_shared(reinterpret_cast<char *>(dst) + q * 16);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + q * 16)
                             : "memory");
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    uint32_t cur = 0;
    // Live-list entries: this warp's current and next triangle (the one
    // after that is loaded one iteration ahead).
    uint32_t pc = wid < nl ? __ldg(live + wid) : 0u;
    uint32_t pn = wid + nw < nl ? __ldg(live + wid + nw) : 0u;
    fetch(sbuf[wib][0], pc, wid < nl);
    RasterPrim *R = &srp[wib];
    float (*T)[RF_TILE_H + 4] = stab[wib];
    uint32_t cur_job = 0xFFFFFFFFu;
    unsigned long long acc_fi = 0, acc_oob = 0;  // per-lane, for cur_job
    float zhi_tri = -__int_as_float(0x7F800000);  // per-lane bound of this triangle's depths
    uint32_t acc_marks = 0;                        // (triangle, tile) bits set by this lane
    auto flush = [&]() {
        if (cur_job != 0xFFFFFFFFu) {
            warp_add_u64(&stats[cur_job].frags_i, acc_fi, true);
            warp_add_u64(&stats[cur_job].oob, acc_oob, true);
        }
        acc_fi = acc_oob = 0;
    };
    // One band of the target: reduce the lanes' covered columns and mark the
    // band's tiles with this triangle's bit.
    auto mark_band = [&](int64_t band, RowOut &o, const JobDev &J, uint32_t word, uint32_t bit) {
        const uint32_t lo = __reduce_min_sync(0xFFFFFFFFu, o.px0 < o.px1 ? o.px0 : 0xFFFFFFFFu);
        const uint32_t hi = __reduce_max_sync(0xFFFFFFFFu, o.px0 < o.px1 ? o.px1 : 0u);
        if (lo < hi) {
            const uint32_t t0 = lo >> tw_log2, t1 = (hi - 1) >> tw_log2;
            uint32_t *row = mask + J.mask_base + (size_t)band * J.tiles_x * J.mask_words + word;
            // ... and the summary bit of that mask word
            uint32_t *srow = mask + J.sum_base + (size_t)band * J.tiles_x * J.sum_words + (word >> 5);
            const uint32_t sbit = 1u << (word & 31u);
            for (uint32_t t = t0 + lane; t <= t1; t += 32) {
                atomicOr(row + (size_t)t * J.mask_words, bit);
                atomicOr(srow + (size_t)t * J.sum_words, sbit);
                ++acc_marks;
            }
        }
    };
    for (uint32_t i = wid; i < nl; i += nw) {
        const uint32_t pnn = i + 2 * nw < nl ? __ldg(live + i + 2 * nw) : 0u;
        __syncwarp();  // the other slot's previous triangle is done
        fetch(sbuf[wib][cur ^ 1u], pn, i + nw < nl);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncwarp();
        const uint32_t p = pc;
        pc = pn;
        pn = pnn;
        PrimRec *sP = reinterpret_cast<PrimRec *>(sbuf[wib][cur]);  // fields before `runs` only
        cur ^= 1u;
        if (lane == 0) {
            R->draw = sP->draw;
            R->flags = sP->live ? RF_RP_LIVE : 0u;
            R->kind = sP->kind;
            R->base = 0;
            R->stride = 0;
            R->y0 = R->c0 = R->y1 = R->c1 = 0;
            R->zmax = __int_as_float(0x7F800000);  // +inf: no bound (only row records give one)
        }
        __syncwarp();
        const PrimRec *P = sP;
        if (P->live) {
            const uint32_t job = P->job;
            if (job != cur_job) {
                flush();
                cur_job = job;
            }
            const JobDev &J = jobs[job];
            const uint32_t tl = P->tri - J.tri_base;
            const uint32_t word = tl >> 5, bit = 1u << (tl & 31);
            const uint32_t nc = NCT ? (uint32_t)NCT : 1 + nattr_of(P->kind);
            const uint32_t nr = RF_R_C + nc;
            const uint32_t stride = 1 + 2 * nc;
            bool regular = P->rwords != 0;
            unsigned long long base = 0;
            if (regular) {
                base = P->rloc;
                if (base + P->rwords > rows_cap) {  // no room: rasterise from the PrimRec
                    regular = false;
                    if (lane == 0) atomicAdd(&counters[RF_CNT_ROWSOVF], 1u);
                    // ... which then needs its binade runs (lane r: quantity r).
                    if (lane < RF_NR) {
                        half_runs(sP->half[0], prims[p].runs[0], lane);
                        half_runs(sP->half[1], prims[p].runs[1], lane);
                    }
                    __syncwarp();
                }
            }
            if (lane == 0 && regular) {
                R->flags |= RF_RP_ROWS;
                R->base = (uint32_t)base;
                R->stride = stride;
            }
            // Both halves' rows, records and dv/dx; a regular triangle's
            // rows are all on the buffer (row >= 0).
            int64_t Yh[2] = {0, 0};
            uint32_t inh[2] = {0u, 0u};
            for (int hh = 0; hh < 2; ++hh) {
                const HalfRec *H = &P->half[hh];
                const uint32_t n = H->n;
                if (lane < RF_NC) R->dvdx[hh][lane] = H->dvdx[lane];
                if (n == 0) continue;
                const float y0r = H->y0r;
                if (!(fabsf(y0r) < RF_MAX_COORD)) {  // outside the supported range
                    if (lane == 0) acc_oob += 1;
                    continue;
                }
                // row(j) = max(0, Y + j); |y0r| < 2^22, so the 32-bit convert
                const int64_t Y = (int32_t)fsub(y0r, 0.5f);
                // Scanlines at or below the buffer's last row count only in oob.
                const int64_t in_rows = min((int64_t)n, max((int64_t)0, (int64_t)J.h - Y));
                if (lane == 0) acc_oob += (unsigned long long)((int64_t)n - in_rows);
                if (in_rows <= 0) continue;
                Yh[hh] = Y;
                inh[hh] = (uint32_t)in_rows;
            }
            if (regular) {
                // Scanlines y: half 0's rows Yh[0] .., then half 1's (the
                // halves meet at the middle vertex's row), walked in one pass
                // so a band holding both is visited once.  One lane per row
                // quantity runs each half's own running sums
                // (ScanlineIter::next), then one lane per row for the span,
                // stats and row record (half 1's records follow half 0's).
                if (lane == 0) {
                    R->y0 = (uint32_t)Yh[0];
                    R->c0 = inh[0];
                    R->y1 = (uint32_t)Yh[1];
                    R->c1 = inh[1];
                }
                // (32-bit rows: a regular triangle's rows are on the target)
                const int32_t lo0 = (int32_t)Yh[0], hi0 = lo0 + (int32_t)inh[0] - 1;
                const int32_t lo1 = (int32_t)Yh[1], hi1 = lo1 + (int32_t)inh[1] - 1;
                const int32_t ylo = inh[0] ? lo0 : lo1, yhi = inh[1] ? hi1 : hi0;
                // Lane q (< nr) runs the upper half's quantity q, lane 16 + q
                // the lower half's, so a band holding both walks them at once.
                const uint32_t wq = lane & 15u, wh = lane >> 4;
                const bool wlane = wq < nr && (wh ? inh[1] : inh[0]) != 0u;
                float wv = wlane ? u2f(P->half[wh].b0[wq]) : 0.0f;
                const float wd = wlane ? P->half[wh].d[wq] : 0.0f;
                const int32_t wlo = wh ? lo1 : lo0, whi = wh ? hi1 : hi0;
                // Rows a..b of the band starting at row bs from running value wv.
                auto walk = [&](float &wv, float wd, int32_t a, int32_t b, int32_t bs) {
                    if (a > b) return;
                    float *col = T[wq];
                    uint32_t i = (uint32_t)(a - bs);
                    const uint32_t e = (uint32_t)(b - bs) + 1u;
                    for (; (i & 3u) && i < e; ++i) {
                        col[i] = wv;
                        wv = fadd(wv, wd);
                    }
                    for (; i + 4u <= e; i += 4u) {  // four rows per trip, one store
                        const float w1 = fadd(wv, wd), w2 = fadd(w1, wd), w3 = fadd(w2, wd);
                        *reinterpret_cast<float4 *>(col + i) = make_float4(wv, w1, w2, w3);
                        wv = fadd(w3, wd);
                    }
                    for (; i < e; ++i) {
                        col[i] = wv;
                        wv = fadd(wv, wd);
                    }
                };
                for (int32_t band = (inh[0] | inh[1]) ? ylo / RF_TILE_H : 1; band * RF_TILE_H <= yhi; ++band) {
                    const int32_t ys = max(ylo, band * RF_TILE_H);
                    const int32_t ye = min(yhi, band * RF_TILE_H + RF_TILE_H - 1);
                    const int32_t bs = band * RF_TILE_H;
                    if (wlane) walk(wv, wd, max(ys, wlo), min(ye, whi), bs);
                    __syncwarp();
                    const int32_t y = band * RF_TILE_H + (int32_t)lane;
                    const bool in0 = inh[0] && y >= lo0 && y <= hi0;
                    const bool in1 = inh[1] && y >= lo1 && y <= hi1;
                    RowOut o{0, 0, 0xFFFFFFFFu, 0};
                    if (in0 || in1) {
                        const uint32_t hh = in0 ? 0u : 1u;
                        const uint32_t i = (uint32_t)(y - bs);
                        const uint32_t ridx = in0 ? (uint32_t)(y - lo0) : inh[0] + (uint32_t)(y - lo1);
                        row_record<NCT>(T[RF_R_LX][i], T[RF_R_RX][i], &T[RF_R_C][i], RF_TILE_H + 4,
                                        P->half[hh].dvdx, nc, J.w, tile_w, rows + base + (size_t)ridx * stride,
                                        o, zhi_tri);
                    }
                    acc_fi += o.frags_i;
                    acc_oob += o.oob;
                    mark_band(band, o, J, word, bit);
                    __syncwarp();
                }
                // The triangle's depth bound: the largest of its rows'.
#pragma unroll
                for (int sft = 16; sft > 0; sft >>= 1)
                    zhi_tri = fmaxf(zhi_tri, __shfl_xor_sync(0xFFFFFFFFu, zhi_tri, sft));
                if (lane == 0) R->zmax = zhi_tri;
                zhi_tri = -__int_as_float(0x7F800000);
            }
            for (int hh = 0; hh < 2 && !regular; ++hh) {
                const HalfRec *H = &P->half[hh];
                if (inh[hh] == 0) continue;
                const int64_t Y = Yh[hh];
                const int64_t in_rows = (int64_t)inh[hh];
                // Rows above the buffer all land on row 0: walked by lane 0.
                RowOut o0{0, 0, 0xFFFFFFFFu, 0};
                int64_t jfirst = 0;
                if (Y < 0) {
                    jfirst = min(in_rows, (int64_t)1 - Y);
                    if (lane == 0)
                        for (int64_t j = 0; j < jfirst; ++j)
                            row_stats(H, &prims[p].runs[hh], (uint32_t)j, J.w, o0);
                }
                // Remaining rows y = Y + j > 0 (or all rows when Y >= 0), by band.
                const int64_t ylo = Y + jfirst, yhi = Y + in_rows - 1;
                for (int64_t band = (ylo > 0 ? ylo : 0) / RF_TILE_H; band * RF_TILE_H <= yhi; ++band) {
                    const int64_t y = band * RF_TILE_H + lane;
                    RowOut o{0, 0, 0xFFFFFFFFu, 0};
                    if (y >= ylo && y <= yhi) row_stats(H, &prims[p].runs[hh], (uint32_t)(y - Y), J.w, o);
                    if (band == 0) {  // fold the rows above the buffer into band 0
                        o.frags_i += o0.frags_i;
                        o.oob += o0.oob;
                        o.px0 = min(o.px0, o0.px0);
                        o.px1 = max(o.px1, o0.px1);
                        o0 = RowOut{0, 0, 0xFFFFFFFFu, 0};
                    }
                    acc_fi += o.frags_i;
                    acc_oob += o.oob;
                    mark_band(band, o, J, word, bit);
                }
                // Band 0 not visited (no row y > 0): flush the row-0 walk of
                // lane 0.  The test is made warp-uniform before the shuffles.
                const bool pend0 =
                    __shfl_sync(0xFFFFFFFFu, (o0.frags_i || o0.oob || o0.px0 < o0.px1) ? 1 : 0, 0) != 0;
                if (pend0) {
                    acc_fi += o0.frags_i;
                    acc_oob += o0.oob;
                    RowOut z{0, 0, __shfl_sync(0xFFFFFFFFu, o0.px0, 0), __shfl_sync(0xFFFFFFFFu, o0.px1, 0)};
                    if (lane != 0) z = RowOut{0, 0, 0xFFFFFFFFu, 0};
                    mark_band(0, z, J, word, bit);
                }
            }
        }
        __syncwarp();
        {
            const uint4 *src = reinterpret_cast<const uint4 *>(R);
            uint4 *dst = reinterpret_cast<uint4 *>(rprims + p);
            if (lane < sizeof(RasterPrim) / 16) dst[lane] = src[lane];
        }
    }
    flush();
    warp_add_u64(marks, acc_marks, true);
}

// ---------------------------------------------------------------------------
// K3c: the same work for small triangles, G = 8 or 16 lanes per triangle.
// A regular triangle with at most G rows on the target (k_setup puts it on
// that group size's list) would leave most of a warp idle in k_bin, so
// here a group of G lanes takes it -- 32 / G triangles per warp (its
// reductions over its own lanes, the warp reconverging between phases):
// one lane per row quantity walks the rows (both halves, ScanlineIter::next
// in the reference's order), then one lane per row does the span, stats,
// record and depth bound exactly as k_bin, and the group marks the (at most
// two) bands' tiles.  A triangle whose records do not fit goes onto k_bin's
// live list instead (k_bin runs after this kernel and takes it with the
// rest).
// ---------------------------------------------------------------------------
static_assert(sizeof(RasterPrim) / 16 <= 8, "a group of eight lanes stores a RasterPrim in one pass");
// G: lanes per triangle (8 or 16: the list of triangles with at most G rows).
template <int NCT, uint32_t G>
__global__ void __launch_bounds__(256, 4)
k_bin_small(const JobDev *__restrict__ jobs, PrimRec *__restrict__ prims,
            const uint32_t *__restrict__ live_small, uint32_t *__restrict__ live, uint32_t tile_w,
            uint32_t *__restrict__ rows, unsigned long long rows_cap, RasterPrim *__restrict__ rprims, uint32_t *__restrict__ mask,
            StatsDev *__restrict__ stats, uint32_t *__restrict__ counters,
            unsigned long long *__restrict__ marks, uint32_t count_slot) {
    static_assert(G == 8 || G == 16, "group sizes");
    constexpr uint32_t NG = 32 / G;  // groups per warp
    constexpr uint32_t NONE = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31, wib = (threadIdx.x >> 5) & 7;
    const uint32_t g = lane / G, gl = lane & (G - 1);  // group of the warp, lane in the group
    const uint32_t gmask = (G == 16 ? 0xFFFFu : 0xFFu) << (G * g);
    const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint32_t ng = (gridDim.x * blockDim.x) / G;
    const uint32_t tw_log2 = __ffs(tile_w) - 1;
    const uint32_t nl = counters[count_slot];
    __shared__ __align__(16) uint4 sbuf[8][NG][RF_PRIM_CORE_BYTES / 16];  // records' first parts
    __shared__ __align__(16) RasterPrim srp[8][NG];
    __shared__ float stab[8][NG][RF_NR][G];  // quantity q of row r at [q][r]
    const PrimRec *P = reinterpret_cast<const PrimRec *>(sbuf[wib][g]);
    RasterPrim *R = &srp[wib][g];
    float (*T)[G] = stab[wib][g];
    uint32_t cur_job = NONE;
    unsigned long long acc_fi = 0, acc_oob = 0;  // per lane, for cur_job
    uint32_t acc_marks = 0;
    auto gsum = [&](unsigned long long v) {
        for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o);
        return v;
    };
    auto flush = [&]() {
        if (cur_job != NONE) {
            const unsigned long long fi = gsum(acc_fi), oob = gsum(acc_oob);
            if (gl == 0 && fi) atomicAdd(&stats[cur_job].frags_i, fi);
            if (gl == 0 && oob) atomicAdd(&stats[cur_job].oob, oob);
        }
        acc_fi = acc_oob = 0;
    };
    // Warp-uniform trips: the four groups of a warp take four consecutive
    // list entries each trip, and the warp reconverges between the phases
    // (groups left to drift apart would issue their instructions apart).
    for (uint32_t w4 = gid - g; w4 < nl; w4 += ng) {
        const uint32_t i = w4 + g;
        const bool act = i < nl;
        uint32_t e = 0;  // the output triangle
        if (act) {
            e = __ldg(live_small + i);
            const uint4 *src = reinterpret_cast<const uint4 *>(prims + e);
            for (uint32_t q = gl; q < RF_PRIM_CORE_BYTES / 16; q += G) sbuf[wib][g][q] = src[q];
        }
        __syncwarp();
        bool run = act;
        unsigned long long base = 0;
        uint32_t word = 0, bit = 0, nc = 0, nr = 0, stride = 0, nrows = 0;
        int64_t Yh[2] = {0, 0};
        uint32_t inh[2] = {0u, 0u};
        const JobDev *J = nullptr;
        if (act) {
            const uint32_t job = P->job;
            if (job != cur_job) {
                flush();
                cur_job = job;
            }
            J = &jobs[job];
            base = P->rloc;
            if (base + P->rwords > rows_cap) {  // no room for its records: k_bin's path
                if (gl == 0) live[atomicAdd(&counters[RF_CNT_LIVE], 1u)] = e;
                run = false;
            }
        }
        if (run) {
            const uint32_t tl = P->tri - J->tri_base;
            word = tl >> 5;
            bit = 1u << (tl & 31);
            nc = NCT ? (uint32_t)NCT : 1 + nattr_of(P->kind);
            nr = RF_R_C + nc;
            stride = 1 + 2 * nc;
            // Both halves' rows on the target (as in k_bin).
            for (int hh = 0; hh < 2; ++hh) {
                const HalfRec *H = &P->half[hh];
                const uint32_t n = H->n;
                if (n == 0) continue;
                const float y0r = H->y0r;
                if (!(fabsf(y0r) < RF_MAX_COORD)) {
                    if (gl == 0) acc_oob += 1;
                    continue;
                }
                const int64_t Y = (int32_t)fsub(y0r, 0.5f);
                const int64_t in_rows = min((int64_t)n, max((int64_t)0, (int64_t)J->h - Y));
                if (gl == 0) acc_oob += (unsigned long long)((int64_t)n - in_rows);
                if (in_rows <= 0) continue;
                Yh[hh] = Y;
                inh[hh] = (uint32_t)in_rows;
            }
            nrows = inh[0] + inh[1];  // <= G (the list's rule)
            if (gl == 0) {
                R->draw = P->draw;
                R->flags = RF_RP_LIVE | RF_RP_ROWS;
                R->kind = P->kind;
                R->base = (uint32_t)base;
                R->stride = stride;
                R->y0 = (uint32_t)Yh[0];
                R->c0 = inh[0];
                R->y1 = (uint32_t)Yh[1];
                R->c1 = inh[1];
            }
            if (gl < RF_NC) {
                R->dvdx[0][gl] = P->half[0].dvdx[gl];
                R->dvdx[1][gl] = P->half[1].dvdx[gl];
            }
            // Row quantity gl of both halves' rows, half 0's first.
            if (gl < nr) {
                for (int hh = 0; hh < 2; ++hh) {
                    float v = u2f(P->half[hh].b0[gl]);
                    const float d = P->half[hh].d[gl];
                    const uint32_t r1 = hh ? nrows : inh[0];
                    for (uint32_t r = hh ? inh[0] : 0u; r < r1; ++r) {
                        T[gl][r] = v;
                        v = fadd(v, d);
                    }
                }
            }
        }
        __syncwarp();
        // Row gl: its span, stats, record and depth bound.
        RowOut o{0, 0, 0xFFFFFFFFu, 0};
        float zhi = -__int_as_float(0x7F800000);
        uint32_t yb = NONE;  // the row's band
        if (run && gl < nrows) {
            const uint32_t hh = gl < inh[0] ? 0u : 1u;
            const int64_t y = hh ? Yh[1] + (gl - inh[0]) : Yh[0] + gl;
            yb = (uint32_t)(y / RF_TILE_H);
            row_record<NCT>(T[RF_R_LX][gl], T[RF_R_RX][gl], &T[RF_R_C][gl], G,
                            P->half[hh].dvdx, nc, J->w, tile_w, rows + base + (size_t)gl * stride, o, zhi);
        }
        __syncwarp();
        acc_fi += o.frags_i;
        acc_oob += o.oob;
        if (run) {
            // The bands' tiles: the group's covered columns per band.
            const uint32_t b_lo = __reduce_min_sync(gmask, yb);
            const uint32_t b_hi = __reduce_max_sync(gmask, yb == NONE ? 0u : yb);
            for (uint32_t b = b_lo; b_lo != NONE && b <= b_hi; ++b) {
                const bool inb = yb == b && o.px0 < o.px1;
                const uint32_t lo = __reduce_min_sync(gmask, inb ? o.px0 : NONE);
                const uint32_t hi = __reduce_max_sync(gmask, inb ? o.px1 : 0u);
                if (lo < hi) {
                    const uint32_t t0 = lo >> tw_log2, t1 = (hi - 1) >> tw_log2;
                    uint32_t *mrow = mask + J->mask_base + (size_t)b * J->tiles_x * J->mask_words + word;
                    uint32_t *srow = mask + J->sum_base + (size_t)b * J->tiles_x * J->sum_words + (word >> 5);
                    const uint32_t sbit = 1u << (word & 31u);
                    for (uint32_t t = t0 + gl; t <= t1; t += G) {
                        atomicOr(mrow + (size_t)t * J->mask_words, bit);
                        atomicOr(srow + (size_t)t * J->sum_words, sbit);
                        ++acc_marks;
                    }
                }
            }
            // The triangle's depth bound: the largest of its rows'.
            for (int o2 = G / 2; o2 > 0; o2 >>= 1) zhi = fmaxf(zhi, __shfl_xor_sync(gmask, zhi, o2));
            if (gl == 0) R->zmax = zhi;
            __syncwarp(gmask);
            const uint4 *rs = reinterpret_cast<const uint4 *>(R);
            uint4 *dst = reinterpret_cast<uint4 *>(rprims + e);
            if (gl < sizeof(RasterPrim) / 16) dst[gl] = rs[gl];
        }
        __syncwarp();
    }
    // The stats left over, one atomic per warp when its groups ended on the
    // same job (the usual case: a frame of one target), else per group.
    const uint32_t has = __ballot_sync(0xFFFFFFFFu, cur_job != NONE);
    const uint32_t j0 = has ? __shfl_sync(0xFFFFFFFFu, cur_job, __ffs(has) - 1) : NONE;
    if (has && __all_sync(0xFFFFFFFFu, cur_job == j0 || cur_job == NONE)) {
        warp_add_u64(&stats[j0].frags_i, acc_fi, true);
        warp_add_u64(&stats[j0].oob, acc_oob, true);
    } else {
        flush();
    }
    __syncwarp();
    warp_add_u64(marks, acc_marks, true);
}

// The rasteriser's work list.  A tile walks its triangles serially, so the
// tiles that take longest should start first, and a tile far more crowded
// than the rest (the horizon of a scene of many small objects) would close
// the pass alone: such a tile is split into RF_SPLIT_K items, one per slice
// of RF_TILE_H / RF_SPLIT_K rows, walked by different warps (each pixel
// still sees its triangles in order: a row belongs to one slice).  The list
// is items[ntiles ..) -- the heavy tiles and the slices of the crowded ones,
// in no particular order -- then items[0 .. ntiles) -- every tile in index
// order, RF_ITEM_SKIP where the tile went to the first part.
//
// k_tile_items: one warp per tile.  Its nonzero mask words (the set bits
// of its summary words) stand for its triangle count: at most the count,
// about it where the tile's triangles are scattered through the submission
// order; where most words are nonzero the bits are counted instead.  A
// crowded tile is one whose count exceeds twice the frame's marks per
// resident warp: its walk alone would outlast two warps' fair shares of
// the pass, so splitting it shortens the pass.
#define RF_SPLIT_MIN 64u  // a tile with fewer binned triangles is never split
#define RF_HEAVY_MIN 16u  // ... nor taken early
__global__ void __launch_bounds__(256)
k_tile_items(const JobDev *__restrict__ jobs, uint32_t nj, const uint32_t *__restrict__ mask,
             uint32_t ntiles, const unsigned long long *__restrict__ marks, uint32_t slots,
             uint32_t *__restrict__ items, uint32_t *__restrict__ extra) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (tile >= ntiles) return;
    const uint32_t ji = upper_index(nj, tile, [&](uint32_t i) { return jobs[i].tile_base; });
    const JobDev &J = jobs[ji];
    const uint32_t lt = tile - J.tile_base;
    const uint32_t *sw = mask + J.sum_base + (size_t)lt * J.sum_words;
    uint32_t c = 0;
    for (uint32_t i = lane; i < J.sum_words; i += 32) c += __popc(sw[i]);
    c = __reduce_add_sync(0xFFFFFFFFu, c);
    if (2u * c >= J.mask_words) {
        // Half the mask words or more are nonzero: they say little about
        // the count, so count the bits (a few small busy scenes do this).
        const uint32_t *mw = mask + J.mask_base + (size_t)lt * J.mask_words;
        c = 0;
        for (uint32_t i = lane; i < J.mask_words; i += 32) c += __popc(mw[i]);
        c = __reduce_add_sync(0xFFFFFFFFu, c);
    }
    if (lane == 0) {
        const unsigned long long share2 = 2ull * *marks / slots;
        const uint32_t thr = (uint32_t)min(max((unsigned long long)RF_SPLIT_MIN, share2), 0xFFFFFFFFull);
        const bool crowded = c > thr;
        // Heavy: more than twice the frame's mean; taken before the rest.
        const bool heavy = crowded || (c > RF_HEAVY_MIN && c > 2ull * *marks / ntiles);
        items[tile] = heavy ? RF_ITEM_SKIP : tile << RF_ITEM_SHIFT;
        if (crowded) {
            const uint32_t at = ntiles + atomicAdd(extra, RF_SPLIT_K);
            for (uint32_t k = 1; k <= RF_SPLIT_K; ++k) items[at + k - 1] = (tile << RF_ITEM_SHIFT) | k;
        } else if (heavy) {
            items[ntiles + atomicAdd(extra, 1u)] = tile << RF_ITEM_SHIFT;
        }
    }
}

// Frame::clear applied directly (when no render follows before a read).
__global__ void k_fill(uint32_t *__restrict__ color, float *__restrict__ depth, size_t n,
                       uint32_t px, float z, uint32_t flags) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        if (flags & 1u) color[i] = px;
        if ((flags & 2u) && depth) depth[i] = z;
    }
}

// ---------------------------------------------------------------------------
// Launch helpers (host side).
// ---------------------------------------------------------------------------
namespace rfk {

cudaError_t launch_vertex(const DrawDev *draws, uint32_t nd, uint32_t nv, float4 *cpos,
                          uint8_t *coc, uint32_t *counters, unsigned long long *marks,
                          int nsm, cudaStream_t s) {
    if (nv == 0) return cudaSuccess;
    uint32_t blocks = min((nv + 255) / 256, (uint32_t)nsm * 16);
    k_vertex<<<blocks, 256, 0, s>>>(draws, nd, nv, cpos, coc, counters, marks);
    return cudaGetLastError();
}

cudaError_t launch_clip(const DrawDev *draws, uint32_t nd, uint32_t nt, const float4 *cpos,
                        const uint8_t *coc, uint32_t *tcnt, uint32_t *tpoly, uint32_t *queue,
                        PolyVert *pool, uint32_t pool_cap, uint32_t *counters, int nsm, cudaStream_t s,
                        uint32_t *toff, bool place) {
    if (nt == 0) return cudaSuccess;
    uint32_t *prim_total = place ? counters + RF_CNT_PRIMS : nullptr;
    const uint32_t blocks = min((nt + RF_CLIP_THREADS - 1) / RF_CLIP_THREADS, (uint32_t)nsm * 16);
    k_clip<<<blocks, RF_CLIP_THREADS, 0, s>>>(draws, nd, nt, coc, tcnt, tpoly, queue, counters, toff, prim_total);
    // The queue's length is known on the device only: a grid for all of it
    // at the worst case, each thread striding over what is there.
    const uint32_t pblocks = min((nt + 15) / 16, (uint32_t)nsm * 8);  // 16 triangles per block
    k_clip_poly<<<pblocks, 256, 0, s>>>(draws, cpos, coc, tcnt, tpoly, queue, pool, pool_cap, counters);
    return cudaGetLastError();
}

size_t scan_scratch_words(uint32_t n) {
    return (n + SCAN_THREADS * SCAN_ITEMS - 1) / (SCAN_THREADS * SCAN_ITEMS) + 1;
}

cudaError_t launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *scratch,
                        uint32_t *total, cudaStream_t s) {
    if (n == 0) return cudaMemsetAsync(total, 0, 4, s);
    const uint32_t nb = (n + SCAN_THREADS * SCAN_ITEMS - 1) / (SCAN_THREADS * SCAN_ITEMS);
    k_scan_blocks<<<nb, SCAN_THREADS, 0, s>>>(in, out, n, scratch, total);
    if (nb > 1) {  // one block: its scan is the whole scan
        k_scan_sums<<<1, 1024, 0, s>>>(scratch, nb, total);
        k_scan_add<<<nb, SCAN_THREADS, 0, s>>>(out, n, scratch);
    }
    return cudaGetLastError();
}

cudaError_t launch_mesh_bbox(const float *verts, uint32_t nverts, uint32_t stride, float *bbox,
                             cudaStream_t s) {
    const uint32_t nb = max(1u, min(RF_MESH_BBOX_BLOCKS, (nverts + 255) / 256));
    k_bbox_part<<<nb, 256, 0, s>>>(verts, nverts, stride, bbox + 6);
    k_bbox_fold<<<1, 32, 0, s>>>(bbox + 6, nb, bbox);
    return cudaGetLastError();
}

cudaError_t launch_setup(const DrawDev *draws, uint32_t nd, const JobDev *jobs, uint32_t nt,
                         uint32_t tile_w, const float4 *cpos, const uint32_t *tcnt,
                         const uint32_t *toff, const uint32_t *tpoly, const PolyVert *pool,
                         PrimRec *prims, unsigned long long *rows_total, uint32_t *rows,
                         unsigned long long rows_cap,
                         RasterPrim *rprims, uint32_t *mask, uint32_t *live, unsigned long long *marks,
                         StatsDev *stats, uint32_t *counters, int nsm, cudaStream_t s,
                         const uint32_t *perm, const uint32_t *ptri, int kind) {
    cudaError_t e = cudaMemsetAsync(rows_total, 0, 8, s);  // the frame's row-record words
    if (e != cudaSuccess) return e;
    if (nt == 0)  // no setup pass to zero the work-list counter
        return cudaMemsetAsync(counters + RF_CNT_ITEMS, 0, 4, s);
    uint32_t blocks = min((nt + RF_SETUP_THREADS - 1) / RF_SETUP_THREADS, (uint32_t)nsm * 32);
    // The live list has room for every output triangle three times over:
    // the triangles for k_bin from the start, those with at most 8 rows from
    // a third of the way, those with 9 to 16 rows from two thirds.  (A
    // depth-sorted frame's triangles are single clipped pieces.)
    const size_t live_cap = perm ? (size_t)nt : (size_t)nt * RF_MAX_FAN;
    uint32_t *live_small = live + live_cap, *live_mid = live + 2 * live_cap;
    k_setup<<<blocks, RF_SETUP_THREADS, 0, s>>>(draws, nd, jobs, nt, cpos, tcnt, toff, tpoly, pool,
                                                prims, rows_total, rprims, live,
                                                counters + RF_CNT_LIVE, live_small,
                                                counters + RF_CNT_LIVE_SMALL, live_mid,
                                                counters + RF_CNT_LIVE_MID, counters + RF_CNT_ITEMS,
                                                stats, perm, ptri);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // The small triangles, eight lanes each, then one warp per other live
    // output triangle (with the small ones that found no room for their
    // records); the counts are only known on the device.
    auto bin = k_bin<0>;
    auto bin8 = k_bin_small<0, 8>;
    auto bin16 = k_bin_small<0, 16>;
    switch (kind) {  // components per triangle: 1 + the kind's attributes
        case RF_K_FLAT: bin = k_bin<1>; bin8 = k_bin_small<1, 8>; bin16 = k_bin_small<1, 16>; break;
        case RF_K_TEXTURED: bin = k_bin<3>; bin8 = k_bin_small<3, 8>; bin16 = k_bin_small<3, 16>; break;
        case RF_K_GOURAUD:
        case RF_K_GOURAUD_SRGB: bin = k_bin<4>; bin8 = k_bin_small<4, 8>; bin16 = k_bin_small<4, 16>; break;
        case RF_K_TEX_GOURAUD: bin = k_bin<6>; bin8 = k_bin_small<6, 8>; bin16 = k_bin_small<6, 16>; break;
        default: break;
    }
    const uint32_t sblocks = min((nt + 31) / 32, (uint32_t)nsm * 4);
    bin8<<<sblocks, 256, 0, s>>>(jobs, prims, live_small, live, tile_w, rows, rows_cap, rprims, mask, stats,
                                 counters, marks, RF_CNT_LIVE_SMALL);
    bin16<<<sblocks, 256, 0, s>>>(jobs, prims, live_mid, live, tile_w, rows, rows_cap, rprims, mask, stats,
                                  counters, marks, RF_CNT_LIVE_MID);
    const uint32_t wblocks = min((nt * 2 + 7) / 8, (uint32_t)nsm * 16);
    bin<<<wblocks, 256, 0, s>>>(draws, jobs, prims, live, tile_w, rows, rows_cap, rprims, mask, stats,
                                counters, marks);
    return cudaGetLastError();
}

cudaError_t launch_items(const JobDev *jobs, uint32_t nj, const uint32_t *mask, uint32_t ntiles,
                         const unsigned long long *marks, uint32_t slots, uint32_t *items,
                         uint32_t *counters, cudaStream_t s) {
    if (ntiles == 0) return cudaSuccess;
    k_tile_items<<<(uint32_t)(((uint64_t)ntiles * 32 + 255) / 256), 256, 0, s>>>(
        jobs, nj, mask, ntiles, marks, slots ? slots : 1u, items, counters + RF_CNT_ITEMS);
    return cudaGetLastError();
}

cudaError_t launch_raster(uint32_t tile_w, int kind, bool fast, const JobDev *jobs, uint32_t nj,
                          const DrawDev *draws, const PrimRec *prims, const RasterPrim *rprims,
                          const uint32_t *rows, const uint32_t *tcnt, const uint32_t *toff,
                          const uint32_t *mask, uint32_t ntiles, const uint32_t *items, const uint32_t *nitems,
                          uint32_t *queue,
                          StatsDev *stats, uint32_t warps, int nsm, cudaStream_t s) {
    if (ntiles == 0) return cudaSuccess;
    switch (tile_w) {
        case 8: return launch_raster_tw8(kind, fast, jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        case 16: return launch_raster_tw16(kind, fast, jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        case 64: return launch_raster_tw64(kind, fast, jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        default: return launch_raster_tw32(kind, fast, jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
    }
}

cudaError_t launch_cull(DrawDev *draws, uint32_t nd, StatsDev *stats, int nsm, cudaStream_t s) {
    if (nd == 0) return cudaSuccess;
    const uint32_t blocks = min((nd + 127) / 128, (uint32_t)nsm * 8);
    k_cull<<<blocks, 128, 0, s>>>(draws, nd, stats);
    return cudaGetLastError();
}

// Per-job stats of a batch folded into the context's running total.  One
// block; stream order makes the plain read-modify-write of *total safe.
__global__ void __launch_bounds__(256) k_stats_fold(const StatsDev *__restrict__ js, uint32_t n,
                                                    StatsDev *__restrict__ total) {
    constexpr int NF = (int)(sizeof(StatsDev) / sizeof(unsigned long long));
    static_assert(sizeof(StatsDev) == NF * sizeof(unsigned long long), "StatsDev is all counters");
    __shared__ unsigned long long part[NF][8];
    unsigned long long a[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) a[f] = 0;
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
        const unsigned long long *c = reinterpret_cast<const unsigned long long *>(js + j);
#pragma unroll
        for (int f = 0; f < NF; ++f) a[f] += c[f];
    }
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[f] += __shfl_xor_sync(0xFFFFFFFFu, a[f], o);
        if (lane == 0) part[f][w] = a[f];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long *t = reinterpret_cast<unsigned long long *>(total);
        for (int f = 0; f < NF; ++f) {
            unsigned long long sum = 0;
            for (uint32_t i = 0; i < blockDim.x / 32; ++i) sum += part[f][i];
            t[f] += sum;
        }
    }
}

// The GPU's global nanosecond timer at this point of the stream.
__global__ void k_stamp(unsigned long long *dst) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *dst = t;
}

cudaError_t launch_stamp(unsigned long long *dst, cudaStream_t s) {
    k_stamp<<<1, 1, 0, s>>>(dst);
    return cudaGetLastError();
}

cudaError_t launch_stats_fold(const StatsDev *js, uint32_t n, StatsDev *total, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_stats_fold<<<1, 256, 0, s>>>(js, n, total);
    return cudaGetLastError();
}

cudaError_t launch_fill(uint32_t *color, float *depth, size_t n, uint32_t px, float z,
                        uint32_t flags, int nsm, cudaStream_t s) {
    if (n == 0 || flags == 0) return cudaSuccess;
    uint32_t blocks = (uint32_t)min((n + 255) / 256, (size_t)nsm * 8);
    k_fill<<<blocks, 256, 0, s>>>(color, depth, n, px, z, flags);
    return cudaGetLastError();
}

}  // namespace rfk
