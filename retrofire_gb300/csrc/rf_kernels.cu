// rf_kernels.cu — CUDA kernels of the triangle render path (sm_103a).
//
// Stage map (reference call stack: core/src/render.rs:134-207):
//   k_vertex   vertex shader + ClipVert::new         render.rs:157-165
//   k_clip     status + Sutherland-Hodgman count      clip.rs:245-301,350-400
//   k_scan_*   order-preserving compaction offsets    (submission order)
//   k_setup    to_screen, face cull, tri_fill/scan    prim.rs:62-88, raster.rs:185-302
//              setup, row walk (stats), tile binning
//   k_raster   per-tile scan conversion, depth test,  raster.rs:80-114, target.rs:163-198
//              fragment shading, pixel packing
//   k_fill     Frame::clear without a later render    front/src/lib.rs:103-120
#include <cuda_runtime.h>

#include "rf_exact.cuh"
#include "rf_internal.cuh"
#include "rf_kernels.cuh"

using namespace rfx;

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

// Largest i with key(i) <= x over a sorted array of n records.
template <class F>
__device__ __forceinline__ uint32_t upper_index(uint32_t n, uint32_t x, F key) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (key(mid) <= x) lo = mid;
        else hi = mid;
    }
    return lo;
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

// Warp-aggregated 64-bit counter add (all 32 lanes must call).
__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, unsigned long long v,
                                             bool same_dst) {
    if (same_dst) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
    } else if (v) {
        atomicAdd(dst, v);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// K1: vertex shader (mvp.apply, mat.rs:952-973, or clip-space passthrough)
// and outcode (clip.rs:240-242, 303-309).
// ---------------------------------------------------------------------------
__global__ void k_vertex(const DrawDev *__restrict__ draws, uint32_t nd, uint32_t nv_total,
                         float4 *__restrict__ cpos, uint8_t *__restrict__ coc) {
    for (uint32_t gv = blockIdx.x * blockDim.x + threadIdx.x; gv < nv_total;
         gv += gridDim.x * blockDim.x) {
        const uint32_t di = upper_index(nd, gv, [&](uint32_t i) { return draws[i].vert_base; });
        const DrawDev &d = draws[di];
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

__global__ void k_clip(const DrawDev *__restrict__ draws, uint32_t nd, uint32_t nt_total,
                       const float4 *__restrict__ cpos, const uint8_t *__restrict__ coc,
                       uint32_t *__restrict__ tcnt, uint32_t *__restrict__ tpoly,
                       PolyVert *__restrict__ pool, uint32_t pool_cap,
                       uint32_t *__restrict__ counters) {
    for (uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x; gt < nt_total;
         gt += gridDim.x * blockDim.x) {
        const uint32_t di = upper_index(nd, gt, [&](uint32_t i) { return draws[i].tri_base; });
        const DrawDev &d = draws[di];
        const uint32_t t = gt - d.tri_base;
        uint32_t vi[3], oc[3];
        bool bad = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            vi[k] = d.idx[3 * (size_t)t + k];
            bad |= vi[k] >= d.nverts;
            vi[k] = bad ? 0u : vi[k] + d.vert_base;
        }
        uint32_t cnt = 0, slot = RF_NO_POLY;
        if (bad) {
            atomicAdd(&counters[RF_CNT_BADIDX], 1u);  // index out of range (render.rs:170 panics)
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) oc[k] = coc[vi[k]];
            if ((oc[0] & oc[1] & oc[2]) != 0u) {
                cnt = 0;  // Hidden
            } else if ((oc[0] | oc[1] | oc[2]) == 0u) {
                cnt = 1;  // Visible
            } else {
                CV A[RF_POLY_CAP], B[RF_POLY_CAP];
                const uint32_t na = d.nattr < RF_MAX_ATTR ? d.nattr : RF_MAX_ATTR;
                for (int k = 0; k < 3; ++k) {
                    const float4 p = cpos[vi[k]];
                    A[k].pos[0] = p.x; A[k].pos[1] = p.y; A[k].pos[2] = p.z; A[k].pos[3] = p.w;
                    const float *src = d.verts + (size_t)(vi[k] - d.vert_base) * d.stride + d.pos_dim;
                    for (uint32_t c = 0; c < na; ++c) A[k].a[c] = src[c];
                    A[k].oc = oc[k];
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
                    // Only reachable through float pathologies (a convex
                    // triangle gains at most one vertex per plane); counted
                    // in stats.oob and dropped.
                    atomicAdd(&counters[RF_CNT_POLYOVF], 1u);
                    nout = 0;
                }
                cnt = nout >= 3 ? (uint32_t)(nout - 2) : 0u;
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
            }
        }
        tcnt[gt] = cnt;
        tpoly[gt] = slot;
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan of tcnt (order-preserving compaction of the clipped
// triangles: output prim order == clipped order of render.rs:184-205).
// ---------------------------------------------------------------------------
#define SCAN_THREADS 1024
#define SCAN_ITEMS 4
__global__ void k_scan_blocks(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                              uint32_t n, uint32_t *__restrict__ block_sums) {
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
        if (lane == 31) block_sums[blockIdx.x] = wi;
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
    h.dlx = dlx;
    h.drx = drx;
    h.lx = fadd(l0.x, fmul(fsub(fadd(l0.x, dlx), l0.x), yt));
    h.rx = fadd(r0.x, fmul(drx, yt));
    for (uint32_t c = 0; c < RF_NC; ++c) {
        if (c < nc) {
            const float dl = fmul(fsub(l1.c[c], l0.c[c]), recip_dy);
            const float dr = fmul(fsub(r1.c[c], r0.c[c]), recip_dy);
            const float l0s = fadd(l0.c[c], dl), r0s = fadd(r0.c[c], dr);
            h.dc[c] = dl;
            h.dvdx[c] = fmul(fsub(r0s, l0s), rdx);
            h.c[c] = fadd(l0.c[c], fmul(fsub(fadd(l0.c[c], dl), l0.c[c]), yt));
        } else {
            h.dc[c] = 0.0f;
            h.dvdx[c] = 0.0f;
            h.c[c] = 0.0f;
        }
    }
}

struct WalkAcc {
    unsigned long long frags_i, oob;
};

// Walks the scanlines of one half exactly like ScanlineIter::next
// (raster.rs:80-114) for the frags.i / oob counters of rasterize_fb
// (target.rs:259-264), and marks the tiles its pixels touch.
__device__ void walk_half(const HalfRec &h, const JobDev &J, uint32_t tw, uint32_t tl,
                          uint32_t *__restrict__ mask, WalkAcc &acc) {
    if (h.n == 0) return;
    if (!(fabsf(h.y0r) < RF_MAX_COORD)) {  // outside the supported coordinate range
        acc.oob += 1;
        return;
    }
    float lx = h.lx, rx = h.rx, yf = h.y0r;
    uint32_t band = 0xFFFFFFFFu, bx0 = 0, bx1 = 0;
    const uint32_t word = tl >> 5, bit = 1u << (tl & 31);
    auto flush = [&]() {
        if (band != 0xFFFFFFFFu && bx1 > bx0) {
            const uint32_t t0 = bx0 / tw, t1 = (bx1 - 1) / tw;
            uint32_t *row = mask + J.mask_base + (size_t)band * J.tiles_x * J.mask_words + word;
            for (uint32_t t = t0; t <= t1; ++t) atomicOr(row + (size_t)t * J.mask_words, bit);
        }
    };
    for (uint32_t j = 0; j < h.n; ++j) {
        const uint64_t y = as_usize(yf);
        if (y >= J.h) {  // every later row is at least as low: all out of bounds
            acc.oob += h.n - j;
            break;
        }
        const float x0r = round_up_to_half(lx), x1r = round_up_to_half(rx);
        const uint64_t xs = as_usize(x0r);
        uint64_t xe = as_usize(x1r);
        if (xe < xs) xe = xs;
        acc.frags_i += xe - xs;
        if (xe > J.w) acc.oob += 1;
        uint64_t nfr = xe - xs;
        const uint32_t cnt = as_u32(fsub(x1r, x0r));
        if (cnt < nfr) nfr = cnt;
        if (nfr && xs < J.w) {
            const uint32_t px0 = (uint32_t)xs;
            const uint32_t px1 = (uint32_t)(xs + nfr < J.w ? xs + nfr : J.w);
            const uint32_t b = (uint32_t)y / RF_TILE_H;
            if (b != band) {
                flush();
                band = b;
                bx0 = px0;
                bx1 = px1;
            } else {
                bx0 = min(bx0, px0);
                bx1 = max(bx1, px1);
            }
        }
        lx = fadd(lx, h.dlx);
        rx = fadd(rx, h.drx);
        yf = fadd(yf, 1.0f);
    }
    flush();
}
}  // namespace

__global__ void k_setup(const DrawDev *__restrict__ draws, uint32_t nd,
                        const JobDev *__restrict__ jobs, uint32_t nt_total, uint32_t tile_w,
                        const float4 *__restrict__ cpos, const uint32_t *__restrict__ tcnt,
                        const uint32_t *__restrict__ toff, const uint32_t *__restrict__ tpoly,
                        const PolyVert *__restrict__ pool, PrimRec *__restrict__ prims,
                        uint32_t *__restrict__ mask, StatsDev *__restrict__ stats) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < nt_total; base += stride) {
        const uint32_t gt = base + threadIdx.x;
        const bool active = gt < nt_total;
        const uint32_t cnt = active ? tcnt[gt] : 0u;
        uint32_t job = 0xFFFFFFFFu;
        unsigned long long prims_o = 0, frags_i = 0, oob = 0;
        if (cnt) {
            const uint32_t di = upper_index(nd, gt, [&](uint32_t i) { return draws[i].tri_base; });
            const DrawDev &d = draws[di];
            job = d.job;
            const JobDev &J = jobs[job];
            const uint32_t t = gt - d.tri_base;
            const uint32_t nc = 1 + nattr_of(d.shader);
            const uint32_t na = nc - 1;
            const uint32_t zm = zdiv_mask_of(d.shader);
            const uint32_t slot = tpoly[gt];
            const uint32_t p0 = toff[gt];
            WalkAcc acc{0, 0};
            for (uint32_t c = 0; c < cnt; ++c) {
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
                        const PolyVert &v = pool[(size_t)slot * RF_POLY_STORE + (k == 0 ? 0 : c + k)];
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
                PrimRec &P = prims[p0 + c];
                P.draw = di;
                P.live = culled ? 0u : 1u;
                if (culled) continue;
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
                HalfRec h0, h1;
                scan_setup(v0.y, v1.y, v0, left, v0, right, nc, h0);
                scan_setup(v1.y, v2.y, left, v2, right, v2, nc, h1);
                P.half[0] = h0;
                P.half[1] = h1;
                const uint32_t tl = gt - J.tri_base;
                walk_half(h0, J, tile_w, tl, mask, acc);
                walk_half(h1, J, tile_w, tl, mask, acc);
            }
            frags_i = acc.frags_i;
            oob = acc.oob;
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
                warp_add_u64(&S->frags_i, frags_i, same);
                warp_add_u64(&S->oob, oob, same);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// K4: tile rasteriser.
// A warp owns one tile of RF_TILE_H rows x TW columns at a time; lane r owns
// row r of the tile for the whole tile, so per-pixel submission order is the
// order in which the lane walks the triangle list — no atomics, no sorting.
// Colour and depth sit in shared memory column-major (word x*32 + r): the
// bank of every access is the lane id, whatever x each lane is at.
// Each lane enters its row with exact jump-aheads (rfx::seq_add_n) from the
// triangle setup: the scanline's edge values after j rows, then the span's
// varyings after k pixels, then steps pixel by pixel like Iter::next.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ uint32_t pack_px(uint32_t c, int32_t fmt) {
    const uint32_t r = c & 0xFFu, g = (c >> 8) & 0xFFu, b = (c >> 16) & 0xFFu, a = c >> 24;
    switch (fmt) {  // pixfmt.rs:76-103
        case RF_K_ARGB8888: return (a << 24) | (r << 16) | (g << 8) | b;
        case RF_K_XRGB8888: return (r << 16) | (g << 8) | b;
        case RF_K_RGBA8888: return (r << 24) | (g << 16) | (b << 8) | a;
        default: return (b << 24) | (g << 16) | (r << 8) | a;
    }
}

__device__ __forceinline__ uint32_t to_color4(float r, float g, float b) {
    // color.rs:253-263: (256 * c) as u8, alpha 0xFF.
    return as_u8(fmul(256.0f, r)) | (as_u8(fmul(256.0f, g)) << 8) | (as_u8(fmul(256.0f, b)) << 16) |
           0xFF000000u;
}

__device__ __forceinline__ uint32_t sample_tex(const DrawDev &d, float tu, float tv) {
    const float w = (float)d.tw, h = (float)d.th;
    uint32_t u, v;
    if (d.sampler == RF_K_REPEAT_POT) {  // tex.rs:240-266
        u = (uint32_t)as_i32(ffloor(fmul(w, tu))) & (d.tw - 1u);
        v = (uint32_t)as_i32(ffloor(fmul(h, tv))) & (d.th - 1u);
    } else if (d.sampler == RF_K_CLAMP) {  // tex.rs:272-304
        float su = fmul(tu, w), sv = fmul(tv, h);
        const float wm = fsub(w, 1.0f), hm = fsub(h, 1.0f);
        su = su < 0.0f ? 0.0f : (su > wm ? wm : su);
        sv = sv < 0.0f ? 0.0f : (sv > hm ? hm : sv);
        u = as_u32(ffloor(su));
        v = as_u32(ffloor(sv));
    } else {  // SamplerOnce (tex.rs:313-357), index clamped instead of panicking
        u = min(as_u32(fmul(w, tu)), d.tw - 1u);
        v = min(as_u32(fmul(h, tv)), d.th - 1u);
    }
    return __ldg(d.tex + (size_t)v * d.tw + u);
}

template <int KIND>
struct Kind {
    static constexpr int NC = KIND == RF_K_FLAT ? 1
                            : KIND == RF_K_TEXTURED ? 3
                            : KIND == RF_K_TEX_GOURAUD ? 6 : 4;
    __device__ static __forceinline__ uint32_t shade(const DrawDev &d, const float *v) {
        if constexpr (KIND == RF_K_FLAT) {
            return d.flat_rgba;
        } else if constexpr (KIND == RF_K_GOURAUD) {
            return to_color4(v[1], v[2], v[3]);
        } else if constexpr (KIND == RF_K_TEXTURED) {
            // Scanline::fragments: var.z_div(pos.z) (raster.rs:60-69)
            return sample_tex(d, fdiv(v[1], v[0]), fdiv(v[2], v[0]));
        } else if constexpr (KIND == RF_K_TEX_GOURAUD) {
            const uint32_t t = sample_tex(d, fdiv(v[4], v[0]), fdiv(v[5], v[0]));
            const float tr = fdiv((float)(t & 0xFFu), 256.0f);
            const float tg = fdiv((float)((t >> 8) & 0xFFu), 256.0f);
            const float tb = fdiv((float)((t >> 16) & 0xFFu), 256.0f);
            return to_color4(fmul(tr, v[1]), fmul(tg, v[2]), fmul(tb, v[3]));
        } else {  // GOURAUD_SRGB: Color3f<LinRgb>::to_srgb (color.rs:383-392)
            const float ig = fdiv(1.0f, 2.2f);
            return to_color4(powf(v[1], ig), powf(v[2], ig), powf(v[3], ig));
        }
    }
};

struct TileCtx {
    uint32_t *scol;
    float *sdep;
    uint32_t lane;
    uint32_t y;       // this lane's row
    uint32_t tx0;     // first column of the tile
    uint32_t ncols;   // columns of the tile inside the target
    bool row_ok;
    bool has_depth;
    int32_t depth_test;
    bool color_write, depth_write;
    int32_t fmt;
    uint32_t w;
    unsigned long long frags_o;
};

// One scanline segment: the lane's row j of half h, clipped to the tile.
template <int KIND>
__device__ __forceinline__ void span(TileCtx &T, const DrawDev &d, const HalfRec &h, uint32_t j) {
    constexpr int NC = Kind<KIND>::NC;
    const float lx = seq_add_n(h.lx, h.dlx, j);
    const float rx = seq_add_n(h.rx, h.drx, j);
    const float x0r = round_up_to_half(lx), x1r = round_up_to_half(rx);
    const uint64_t xs = as_usize(x0r);
    uint64_t xe = as_usize(x1r);
    if (xe < xs) xe = xs;
    if (xs >= T.tx0 + T.ncols) return;
    uint64_t nfr = xe - xs;
    const uint32_t cnt = as_u32(fsub(x1r, x0r));
    if (cnt < nfr) nfr = cnt;
    const uint64_t send = xs + nfr;  // xs < 2^32 here, no overflow
    const uint32_t a = (uint32_t)(xs > T.tx0 ? xs : T.tx0);
    const uint32_t b = (uint32_t)(send < (uint64_t)(T.tx0 + T.ncols) ? send : (uint64_t)(T.tx0 + T.ncols));
    if (a >= b) return;
    // v0 = left.next(); v0 = v0.lerp(v0.step(dv_dx), x0 - v0.x)  (raster.rs:88-102)
    const float tshift = fsub(x0r, lx);
    const uint32_t k0 = a - (uint32_t)xs;
    float v[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const float c0 = seq_add_n(h.c[c], h.dc[c], j);
        const float adj = fadd(c0, fmul(fsub(fadd(c0, h.dvdx[c]), c0), tshift));
        v[c] = seq_add_n(adj, h.dvdx[c], k0);
    }
    float dv[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) dv[c] = h.dvdx[c];
    uint32_t idx = (a - T.tx0) * RF_TILE_H + T.lane;
    for (uint32_t x = a; x < b; ++x, idx += RF_TILE_H) {
        const float z = v[0];
        bool pass = true;
        if (T.has_depth) {
            const float cur = T.sdep[idx];
            switch (T.depth_test) {  // ctx.rs:86-89
                case RF_K_DEPTH_NONE: pass = true; break;
                case RF_K_DEPTH_LESS: pass = cur < z; break;
                case RF_K_DEPTH_EQUAL: pass = cur == z; break;
                default: pass = cur > z; break;
            }
        }
        if (pass) {
            if (T.color_write) {
                T.scol[idx] = pack_px(Kind<KIND>::shade(d, v), T.fmt);
                T.frags_o += 1;
            }
            if (T.has_depth && T.depth_write) T.sdep[idx] = z;
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) v[c] = fadd(v[c], dv[c]);
    }
}

template <int KIND>
__device__ __forceinline__ void raster_half(TileCtx &T, const DrawDev &d, const HalfRec &h) {
    if (h.n == 0 || !T.row_ok) return;
    if (!(fabsf(h.y0r) < RF_MAX_COORD)) return;
    // Row of scanline j is (y0r + j) as usize = max(0, Y + j), Y = y0r - 0.5.
    const int32_t Y = (int32_t)fsub(h.y0r, 0.5f);
    if (T.y > 0 || Y >= 0) {
        const int64_t j = (int64_t)T.y - Y;
        if (j >= 0 && j < (int64_t)h.n) span<KIND>(T, d, h, (uint32_t)j);
    } else {
        const int64_t jn = min((int64_t)h.n, (int64_t)1 - Y);
        for (int64_t j = 0; j < jn; ++j) span<KIND>(T, d, h, (uint32_t)j);
    }
}

__device__ __forceinline__ void raster_prim(TileCtx &T, const DrawDev *__restrict__ draws,
                                            const PrimRec *__restrict__ P) {
    if (!P->live) return;
    const DrawDev &d = draws[P->draw];
    const HalfRec h0 = P->half[0];
    const HalfRec h1 = P->half[1];
    switch (d.shader) {
        case RF_K_FLAT: raster_half<RF_K_FLAT>(T, d, h0); raster_half<RF_K_FLAT>(T, d, h1); break;
        case RF_K_GOURAUD: raster_half<RF_K_GOURAUD>(T, d, h0); raster_half<RF_K_GOURAUD>(T, d, h1); break;
        case RF_K_TEXTURED: raster_half<RF_K_TEXTURED>(T, d, h0); raster_half<RF_K_TEXTURED>(T, d, h1); break;
        case RF_K_TEX_GOURAUD:
            raster_half<RF_K_TEX_GOURAUD>(T, d, h0);
            raster_half<RF_K_TEX_GOURAUD>(T, d, h1);
            break;
        default:
            raster_half<RF_K_GOURAUD_SRGB>(T, d, h0);
            raster_half<RF_K_GOURAUD_SRGB>(T, d, h1);
            break;
    }
}

}  // namespace

template <int TW>
__global__ void __launch_bounds__(RF_RASTER_MAX_THREADS)
k_raster(const JobDev *__restrict__ jobs, uint32_t nj, const DrawDev *__restrict__ draws,
         const PrimRec *__restrict__ prims, const uint32_t *__restrict__ tcnt,
         const uint32_t *__restrict__ toff, const uint32_t *__restrict__ mask,
         uint32_t ntiles_total, uint32_t *__restrict__ tile_queue, StatsDev *__restrict__ stats) {
    extern __shared__ uint32_t smem[];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *scol = smem + warp * (2 * TW * RF_TILE_H);
    float *sdep = reinterpret_cast<float *>(scol + TW * RF_TILE_H);
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(tile_queue, 1u);
        tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
        if (tile >= ntiles_total) break;
        const uint32_t ji = upper_index(nj, tile, [&](uint32_t i) { return jobs[i].tile_base; });
        const JobDev &J = jobs[ji];
        const uint32_t lt = tile - J.tile_base;
        const uint32_t tyi = lt / J.tiles_x, txi = lt - tyi * J.tiles_x;
        TileCtx T;
        T.scol = scol;
        T.sdep = sdep;
        T.lane = lane;
        T.tx0 = txi * TW;
        T.y = tyi * RF_TILE_H + lane;
        T.ncols = min((uint32_t)TW, J.w - T.tx0);
        T.row_ok = T.y < J.h;
        T.has_depth = J.depth != nullptr;
        T.depth_test = J.depth_test;
        T.color_write = J.color_write != 0;
        T.depth_write = J.depth_write != 0;
        T.fmt = J.pixfmt;
        T.w = J.w;
        T.frags_o = 0;
        const size_t row_off = (size_t)T.y * J.w + T.tx0;
        bool loaded = false;
        auto load_tile = [&]() {
            // Lane r loads row r; colour/depth come from the target or from
            // a pending clear (the clear is fused into this load).
            for (uint32_t x = 0; x < (uint32_t)TW; ++x) {
                const uint32_t i = x * RF_TILE_H + lane;
                const bool in = T.row_ok && x < T.ncols;
                scol[i] = (J.clear_flags & 1u) ? J.clear_px : (in ? J.color[row_off + x] : 0u);
                if (T.has_depth)
                    sdep[i] = (J.clear_flags & 2u) ? J.clear_z : (in ? J.depth[row_off + x] : 0.0f);
            }
        };
        const uint32_t *tmask = mask + J.mask_base + (size_t)lt * J.mask_words;
        for (uint32_t wb = 0; wb < J.mask_words; wb += 32) {
            const uint32_t word = wb + lane < J.mask_words ? tmask[wb + lane] : 0u;
            uint32_t bal = __ballot_sync(0xFFFFFFFFu, word != 0u);
            if (bal && !loaded) {
                load_tile();
                loaded = true;
            }
            while (bal) {
                const uint32_t src = __ffs(bal) - 1;
                bal &= bal - 1;
                uint32_t wv = __shfl_sync(0xFFFFFFFFu, word, src);
                while (wv) {
                    const uint32_t b = __ffs(wv) - 1;
                    wv &= wv - 1;
                    const uint32_t gt = J.tri_base + (wb + src) * 32 + b;
                    const uint32_t p0 = toff[gt], pc = tcnt[gt];
                    for (uint32_t p = p0; p < p0 + pc; ++p) raster_prim(T, draws, prims + p);
                }
            }
        }
        if (!loaded && J.clear_flags) {
            load_tile();
            loaded = true;
        }
        if (loaded && T.row_ok) {
            for (uint32_t x = 0; x < T.ncols; ++x) {
                const uint32_t i = x * RF_TILE_H + lane;
                J.color[row_off + x] = scol[i];
                if (T.has_depth) J.depth[row_off + x] = sdep[i];
            }
        }
        __syncwarp();
        const uint32_t j0 = __shfl_sync(0xFFFFFFFFu, ji, 0);
        warp_add_u64(&stats[j0].frags_o, T.frags_o, true);
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
                          uint8_t *coc, int nsm, cudaStream_t s) {
    if (nv == 0) return cudaSuccess;
    uint32_t blocks = min((nv + 255) / 256, (uint32_t)nsm * 16);
    k_vertex<<<blocks, 256, 0, s>>>(draws, nd, nv, cpos, coc);
    return cudaGetLastError();
}

cudaError_t launch_clip(const DrawDev *draws, uint32_t nd, uint32_t nt, const float4 *cpos,
                        const uint8_t *coc, uint32_t *tcnt, uint32_t *tpoly, PolyVert *pool,
                        uint32_t pool_cap, uint32_t *counters, int nsm, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    uint32_t blocks = min((nt + 127) / 128, (uint32_t)nsm * 16);
    k_clip<<<blocks, 128, 0, s>>>(draws, nd, nt, cpos, coc, tcnt, tpoly, pool, pool_cap, counters);
    return cudaGetLastError();
}

size_t scan_scratch_words(uint32_t n) {
    return (n + SCAN_THREADS * SCAN_ITEMS - 1) / (SCAN_THREADS * SCAN_ITEMS) + 1;
}

cudaError_t launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *scratch,
                        uint32_t *total, cudaStream_t s) {
    if (n == 0) return cudaMemsetAsync(total, 0, 4, s);
    const uint32_t nb = (n + SCAN_THREADS * SCAN_ITEMS - 1) / (SCAN_THREADS * SCAN_ITEMS);
    k_scan_blocks<<<nb, SCAN_THREADS, 0, s>>>(in, out, n, scratch);
    k_scan_sums<<<1, 1024, 0, s>>>(scratch, nb, total);
    k_scan_add<<<nb, SCAN_THREADS, 0, s>>>(out, n, scratch);
    return cudaGetLastError();
}

cudaError_t launch_setup(const DrawDev *draws, uint32_t nd, const JobDev *jobs, uint32_t nt,
                         uint32_t tile_w, const float4 *cpos, const uint32_t *tcnt,
                         const uint32_t *toff, const uint32_t *tpoly, const PolyVert *pool,
                         PrimRec *prims, uint32_t *mask, StatsDev *stats, int nsm, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    uint32_t blocks = min((nt + 127) / 128, (uint32_t)nsm * 16);
    k_setup<<<blocks, 128, 0, s>>>(draws, nd, jobs, nt, tile_w, cpos, tcnt, toff, tpoly, pool,
                                   prims, mask, stats);
    return cudaGetLastError();
}

template <int TW>
static cudaError_t launch_raster_tw(const JobDev *jobs, uint32_t nj, const DrawDev *draws,
                                    const PrimRec *prims, const uint32_t *tcnt,
                                    const uint32_t *toff, const uint32_t *mask, uint32_t ntiles,
                                    uint32_t *queue, StatsDev *stats, uint32_t warps, int nsm,
                                    cudaStream_t s) {
    const size_t smem = (size_t)warps * 2 * TW * RF_TILE_H * 4;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_raster<TW>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raster<TW>, warps * 32, smem);
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)per_sm * (uint32_t)nsm;
    const uint32_t need = (ntiles + warps - 1) / warps;
    if (blocks > need) blocks = need;
    if (blocks == 0) blocks = 1;
    k_raster<TW><<<blocks, warps * 32, smem, s>>>(jobs, nj, draws, prims, tcnt, toff, mask, ntiles,
                                                 queue, stats);
    return cudaGetLastError();
}

cudaError_t launch_raster(uint32_t tile_w, const JobDev *jobs, uint32_t nj, const DrawDev *draws,
                          const PrimRec *prims, const uint32_t *tcnt, const uint32_t *toff,
                          const uint32_t *mask, uint32_t ntiles, uint32_t *queue,
                          StatsDev *stats, uint32_t warps, int nsm, cudaStream_t s) {
    if (ntiles == 0) return cudaSuccess;
    switch (tile_w) {
        case 8: return launch_raster_tw<8>(jobs, nj, draws, prims, tcnt, toff, mask, ntiles, queue, stats, warps, nsm, s);
        case 16: return launch_raster_tw<16>(jobs, nj, draws, prims, tcnt, toff, mask, ntiles, queue, stats, warps, nsm, s);
        case 64: return launch_raster_tw<64>(jobs, nj, draws, prims, tcnt, toff, mask, ntiles, queue, stats, warps, nsm, s);
        default: return launch_raster_tw<32>(jobs, nj, draws, prims, tcnt, toff, mask, ntiles, queue, stats, warps, nsm, s);
    }
}

cudaError_t launch_fill(uint32_t *color, float *depth, size_t n, uint32_t px, float z,
                        uint32_t flags, int nsm, cudaStream_t s) {
    if (n == 0 || flags == 0) return cudaSuccess;
    uint32_t blocks = (uint32_t)min((n + 255) / 256, (size_t)nsm * 8);
    k_fill<<<blocks, 256, 0, s>>>(color, depth, n, px, z, flags);
    return cudaGetLastError();
}

}  // namespace rfk
