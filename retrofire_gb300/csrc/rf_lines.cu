// rf_lines.cu — line primitives: render() for Edge<usize> (core/src/render/
// prim.rs:41-60): the vertex stage (k_vertex), line clipping (clip.rs:
// 311-348), to_screen, face culling (is_backface is false for an edge), and
// line() (raster.rs:115-173), each pixel a one-pixel scanline into the
// target (target.rs:163-198) with the first vertex's position and varyings.
//
// k_line_setup: one thread per line; clips it, walks its pixels with the
// reference's running sum (stats, and the tiles it touches: a per-tile
// bitmask over the lines, bit order = submission order).
// k_line_raster: a warp per 32x32 tile takes the tile's lines in order; a
// line that steps along x gives each column (lane) at most one pixel, one
// that steps along y each row (lane): the lane's pixel comes from the exact
// k-step running sum (rfx::jump), so lanes of one line never collide and
// pixels see the lines in submission order.
#include "rf_raster.cuh"

using namespace rfx;
using namespace rfd;

namespace {

__constant__ float l_planes[6][4] = {
    {0.0f, 0.0f, -1.0f, -1.0f},  // near   (clip.rs:215-222)
    {0.0f, 0.0f, 1.0f, -1.0f},   // far
    {-1.0f, 0.0f, 0.0f, -1.0f},  // left
    {1.0f, 0.0f, 0.0f, -1.0f},   // right
    {0.0f, -1.0f, 0.0f, -1.0f},  // bottom
    {0.0f, 1.0f, 0.0f, -1.0f},   // top
};

__device__ __forceinline__ uint32_t loutcode(const float *p) {
    uint32_t oc = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) oc |= (dot4(l_planes[i], p) > 0.0f) ? (1u << i) : 0u;
    return oc;
}

struct LV {
    float pos[4];
    float a[RF_MAX_ATTR];
    uint32_t oc;
};

// ClipPlane::intersect (clip.rs:121-145) on one edge.
__device__ bool lintersect(int p, const LV &a, const LV &b, uint32_t na, LV &out) {
    const float d0 = dot4(l_planes[p], a.pos), d1 = dot4(l_planes[p], b.pos);
    if (!(fmul(d0, d1) < 0.0f)) return false;
    const float t = fdiv(-d0, fsub(d1, d0));
#pragma unroll
    for (int c = 0; c < 4; ++c) out.pos[c] = lerp(a.pos[c], b.pos[c], t);
    for (uint32_t c = 0; c < na; ++c) out.a[c] = lerp(a.a[c], b.a[c], t);
    out.oc = loutcode(out.pos);
    return true;
}

__device__ __forceinline__ uint32_t lzdiv_mask(int32_t shader) {
    return shader == RF_K_TEXTURED ? 0x3u : (shader == RF_K_TEX_GOURAUD ? 0x18u : 0u);
}

// Shaded colour of a fragment with varyings v (v[0] = z, v[1..] attributes
// after to_screen), packed in the target's format.
__device__ uint32_t lshade(const DrawDev &d, const float *v, int32_t fmt) {
    using namespace rfr;
    uint32_t c;
    switch (d.shader) {
        case RF_K_FLAT: c = Kind<RF_K_FLAT>::shade(d, v); break;
        case RF_K_GOURAUD: c = Kind<RF_K_GOURAUD>::shade(d, v); break;
        case RF_K_TEXTURED: c = Kind<RF_K_TEXTURED>::shade(d, v); break;
        case RF_K_TEX_GOURAUD: c = Kind<RF_K_TEX_GOURAUD>::shade(d, v); break;
        default: c = Kind<RF_K_GOURAUD_SRGB>::shade(d, v); break;
    }
    return pack_px(c, pack_selector(fmt));
}

}  // namespace

__global__ void k_line_setup(const DrawDev *__restrict__ draws, const JobDev *__restrict__ jobs,
                             uint32_t nl, const float4 *__restrict__ cpos,
                             const uint8_t *__restrict__ coc, LineRec *__restrict__ recs,
                             uint32_t *__restrict__ mask, StatsDev *__restrict__ stats) {
    const DrawDev &d = draws[0];
    const JobDev &J = jobs[0];
    const uint32_t na = d.nattr, zm = lzdiv_mask(d.shader);
    unsigned long long po = 0, fi = 0, oob = 0;
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) {
        LineRec R{};
        LV e[2];
        for (int k = 0; k < 2; ++k) {
            const uint32_t vi = d.idx[2 * (size_t)l + k];
            const float4 p = cpos[vi];
            e[k].pos[0] = p.x; e[k].pos[1] = p.y; e[k].pos[2] = p.z; e[k].pos[3] = p.w;
            e[k].oc = coc[vi];
            const float *src = d.verts + (size_t)vi * d.stride + d.pos_dim;
            for (uint32_t c = 0; c < RF_MAX_ATTR; ++c) e[k].a[c] = c < na ? src[c] : 0.0f;
        }
        bool keep = (e[0].oc & e[1].oc) == 0;  // both outside one plane: dropped
        if (keep && (e[0].oc | e[1].oc)) {
            for (int p = 0; p < 6; ++p) {
                const bool a_in = (e[0].oc & (1u << p)) == 0, b_in = (e[1].oc & (1u << p)) == 0;
                if (!a_in && !b_in) {
                    keep = false;
                    break;
                }
                LV v;
                if (lintersect(p, e[0], e[1], na, v)) {
                    if (a_in) e[1] = v;
                    else if (b_in) e[0] = v;
                }
            }
        }
        // to_screen (prim.rs:62-88): (x/w, y/w, 1/w) through the viewport,
        // attributes z_div'd where the shader's types divide.
        float s[2][3], at[2][RF_MAX_ATTR];
        if (keep) {
            for (int k = 0; k < 2; ++k) {
                const float w = e[k].pos[3];
                const float ndc[4] = {fdiv(e[k].pos[0], w), fdiv(e[k].pos[1], w), fdiv(1.0f, w), 1.0f};
                s[k][0] = dot4(J.vp + 0, ndc);
                s[k][1] = dot4(J.vp + 4, ndc);
                s[k][2] = dot4(J.vp + 8, ndc);
                for (uint32_t c = 0; c < RF_MAX_ATTR; ++c)
                    at[k][c] = c < na ? (((zm >> c) & 1u) ? fdiv(e[k].a[c], w) : e[k].a[c]) : 0.0f;
            }
            if (J.face_cull == RF_K_CULL_FRONT) keep = false;  // face_cull(false)
        }
        if (keep) {
            po += 1;
            // raster.rs:121-173 line(): v0 the upper end, then for a wide
            // line the left end (dx, dy keep their values).
            int i0 = 0, i1 = 1;
            if (s[0][1] > s[1][1]) { i0 = 1; i1 = 0; }
            const float dx = fsub(s[i1][0], s[i0][0]), dy = fsub(s[i1][1], s[i0][1]);
            const bool wide = fabsf(dx) > dy;
            if (wide && dx < 0.0f) { const int t = i0; i0 = i1; i1 = t; }
            uint64_t b, e2;
            float s0, dd;
            if (wide) {
                const float x0 = round_up_to_half(s[i0][0]), x1 = round_up_to_half(s[i1][0]);
                dd = fdiv(dy, dx);
                s0 = fadd(s[i0][1], fmul(dd, fsub(x0, s[i0][0])));
                b = as_usize(x0);
                e2 = as_usize(x1);
            } else {
                const float y0 = round_up_to_half(s[i0][1]), y1 = round_up_to_half(s[i1][1]);
                dd = fdiv(dx, dy);
                s0 = fadd(s[i0][0], fmul(dd, fsub(y0, s[i0][1])));
                b = as_usize(y0);
                e2 = as_usize(y1);
            }
            const uint64_t n = e2 > b ? e2 - b : 0u;
            if (n > RF_LINE_MAX_SPAN) {
                oob += 1;  // out of the supported range: counted, not drawn
            } else if (n) {
                float v[RF_NC];
                v[0] = s[i0][2];
                for (uint32_t c = 0; c < RF_MAX_ATTR; ++c) v[1 + c] = at[i0][c];
                R.live = 1;
                R.wide = wide ? 1u : 0u;
                R.begin = b;
                R.n = (uint32_t)n;
                R.s0 = s0;
                R.d = dd;
                R.z = v[0];
                R.color = J.color_write ? lshade(d, v, J.pixfmt) : 0u;
                // The pixels with the running sum, for the stats and tiles.
                float val = s0;
                uint32_t last = 0xFFFFFFFFu;
                for (uint64_t k = 0; k < n; ++k) {
                    const uint64_t x = wide ? b + k : as_usize(val);
                    const uint64_t y = wide ? as_usize(val) : b + k;
                    val = fadd(val, dd);
                    if (y >= J.h) {
                        oob += 1;
                        continue;
                    }
                    fi += 1;
                    if (x >= J.w) {
                        oob += 1;
                        continue;
                    }
                    const uint32_t tile = (uint32_t)(y / RF_TILE_H) * J.tiles_x + (uint32_t)(x / RF_TILE_H);
                    if (tile != last) {
                        atomicOr(mask + (size_t)tile * J.mask_words + (l >> 5), 1u << (l & 31));
                        last = tile;
                    }
                }
            }
        }
        recs[l] = R;
    }
    warp_add_u64(&stats->prims_o, po, true);
    warp_add_u64(&stats->verts_o, 3ull * po, true);
    warp_add_u64(&stats->frags_i, fi, true);
    warp_add_u64(&stats->oob, oob, true);
}

__global__ void k_line_raster(const JobDev *__restrict__ jobs, const LineRec *__restrict__ recs,
                              const uint32_t *__restrict__ mask, uint32_t ntiles,
                              uint32_t *__restrict__ queue, StatsDev *__restrict__ stats) {
    const JobDev &J = jobs[0];
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long fo = 0;
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(queue, 1u);
        tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
        if (tile >= ntiles) break;
        const uint32_t ty = tile / J.tiles_x, tx = tile - ty * J.tiles_x;
        const uint64_t tx0 = (uint64_t)tx * RF_TILE_H, ty0 = (uint64_t)ty * RF_TILE_H;
        const uint64_t tx1 = min(tx0 + RF_TILE_H, (uint64_t)J.w);
        const uint32_t *tm = mask + (size_t)tile * J.mask_words;
        for (uint32_t wb = 0; wb < J.mask_words; wb += 32) {
            const uint32_t word = wb + lane < J.mask_words ? tm[wb + lane] : 0u;
            uint32_t bal = __ballot_sync(0xFFFFFFFFu, word != 0u);
            while (bal) {
                const uint32_t src = __ffs(bal) - 1;
                bal &= bal - 1;
                uint32_t w = __shfl_sync(0xFFFFFFFFu, word, src);
                while (w) {
                    const uint32_t l = (wb + src) * 32 + (__ffs(w) - 1);
                    w &= w - 1;
                    const LineRec R = recs[l];
                    uint64_t x = 0, y = 0;
                    bool mine = false;
                    if (R.wide) {  // lane = column
                        x = tx0 + lane;
                        if (x < tx1 && x >= R.begin && x - R.begin < R.n) {
                            y = as_usize(jump(R.s0, R.d, (uint32_t)(x - R.begin)));
                            mine = y >= ty0 && y < ty0 + RF_TILE_H && y < J.h;
                        }
                    } else {  // lane = row
                        y = ty0 + lane;
                        if (y < J.h && y >= R.begin && y - R.begin < R.n) {
                            x = as_usize(jump(R.s0, R.d, (uint32_t)(y - R.begin)));
                            mine = x >= tx0 && x < tx1;
                        }
                    }
                    if (mine) {
                        const size_t i = (size_t)y * J.w + x;
                        bool pass = true;
                        if (J.depth) {
                            const float cur = J.depth[i];
                            switch (J.depth_test) {  // ctx.rs:86-89
                                case RF_K_DEPTH_NONE: pass = true; break;
                                case RF_K_DEPTH_LESS: pass = cur < R.z; break;
                                case RF_K_DEPTH_EQUAL: pass = cur == R.z; break;
                                default: pass = cur > R.z; break;
                            }
                        }
                        if (pass) {
                            if (J.color_write) {
                                J.color[i] = R.color;
                                fo += 1;
                            }
                            if (J.depth && J.depth_write) J.depth[i] = R.z;
                        }
                    }
                    __syncwarp();  // this line's pixels before the next line's tests
                }
            }
        }
    }
    warp_add_u64(&stats->frags_o, fo, true);
}

namespace rfk {

cudaError_t launch_lines(const DrawDev *draws, const JobDev *jobs, uint32_t nl, const float4 *cpos,
                         const uint8_t *coc, LineRec *recs, uint32_t *mask, uint32_t ntiles,
                         uint32_t *queue, StatsDev *stats, int nsm, cudaStream_t s) {
    if (nl == 0) return cudaSuccess;
    const uint32_t blocks = min((nl + 127) / 128, (uint32_t)nsm * 8);
    k_line_setup<<<blocks, 128, 0, s>>>(draws, jobs, nl, cpos, coc, recs, mask, stats);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const uint32_t rblocks = min((ntiles + 3) / 4, (uint32_t)nsm * 8);
    k_line_raster<<<rblocks, 128, 0, s>>>(jobs, recs, mask, ntiles, queue, stats);
    return cudaGetLastError();
}

}  // namespace rfk
