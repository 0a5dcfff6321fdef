// rf_raster.cuh — the tile rasteriser (k_raster), included by one
// translation unit per tile width (rf_raster_tw*.cu) so the specialised
// kernels compile in parallel.
#ifndef RF_RASTER_CUH
#define RF_RASTER_CUH

#include <cuda_runtime.h>

#include <mutex>

#include "rf_device.cuh"

// ---------------------------------------------------------------------------
// K4: tile rasteriser.
// A warp owns one tile of RF_TILE_H rows x TW columns at a time; lane r owns
// row r of the tile for the whole tile, so per-pixel submission order is the
// order in which the lane walks the triangle list — no atomics, no sorting.
// Colour and depth sit in shared memory column-major (word x*32 + r): the
// bank of every access is the lane id, whatever x each lane is at.
// Each lane reads its row's record (written by the binning pass from the
// reference's own running sums: the clipped span, the varyings at its first
// fragment and at its first tile boundary), enters the tile from one of
// those -- or, in a third or later tile of a long span, with an exact jump
// (rfx::jump) of whole tile widths from the boundary values -- then steps
// pixel by pixel like Iter::next.  Warps take work items (a tile, or a row
// slice of a crowded one) from the list k_tile_items builds; triangle
// headers and row records come in through cp.async rings in shared memory,
// and a tile of whole 32-column blocks goes back to HBM through the copy
// engine (cp.async.bulk, one 128-byte row per lane).
// ---------------------------------------------------------------------------
namespace rfr {
using namespace rfx;
using namespace rfd;

// IntoPixel (pixfmt.rs:76-103) of a Color4 packed r | g << 8 | b << 16 |
// a << 24, as one byte permutation: the selector of each format puts the
// channels where the format wants them (XRGB8888's top byte is zero).
__host__ __device__ constexpr uint32_t pack_selector(int32_t fmt) {
    return fmt == RF_K_ARGB8888 ? 0x3012u : fmt == RF_K_XRGB8888 ? 0x4012u : fmt == RF_K_RGBA8888 ? 0x0123u : 0x2103u;
}
__device__ __forceinline__ uint32_t pack_px(uint32_t c, uint32_t sel) { return __byte_perm(c, 0u, sel); }
// The same pixel straight from the channel bytes r, g, b (each 0..255 in a
// 32-bit word): the byte selector over (r | g << 8, b | 0xFF00) -- byte k of
// the Color4 word is byte {0, 1, 4, 5}[k] there, and byte 2 is a zero.
__host__ __device__ constexpr uint32_t rgb_selector(uint32_t sel) {
    uint32_t out = 0;
    for (int i = 0; i < 4; ++i) {
        const uint32_t n = (sel >> (4 * i)) & 0xFu;
        out |= (n == 0u ? 0u : n == 1u ? 1u : n == 2u ? 4u : n == 3u ? 5u : 2u) << (4 * i);
    }
    return out;
}
static_assert(rgb_selector(0x3012u) == 0x5014u && rgb_selector(0x4012u) == 0x2014u &&
                  rgb_selector(0x0123u) == 0x0145u && rgb_selector(0x2103u) == 0x4105u,
              "pixel selectors over the channel bytes");
__device__ __forceinline__ uint32_t pack_rgb(uint32_t r, uint32_t g, uint32_t b, uint32_t rsel) {
    return __byte_perm(__byte_perm(r, g, 0x1140u), b | 0xFF00u, rsel);
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
    static constexpr bool TEXTURED = KIND == RF_K_TEXTURED || KIND == RF_K_TEX_GOURAUD;
    // The texel a fragment samples (textured kinds; any varyings give an
    // in-range index), then the colour from it: shade() split in two so
    // several fragments' texel loads can be in flight together.
    __device__ static __forceinline__ uint32_t texel(const DrawDev &d, const float *v) {
        if constexpr (KIND == RF_K_TEXTURED) return sample_tex(d, fdiv(v[1], v[0]), fdiv(v[2], v[0]));
        else if constexpr (KIND == RF_K_TEX_GOURAUD) return sample_tex(d, fdiv(v[4], v[0]), fdiv(v[5], v[0]));
        else return 0u;
    }
    __device__ static __forceinline__ uint32_t from_texel(uint32_t t, const float *v) {
        if constexpr (KIND == RF_K_TEX_GOURAUD) {
            const float tr = fdiv((float)(t & 0xFFu), 256.0f);
            const float tg = fdiv((float)((t >> 8) & 0xFFu), 256.0f);
            const float tb = fdiv((float)((t >> 16) & 0xFFu), 256.0f);
            return to_color4(fmul(tr, v[1]), fmul(tg, v[2]), fmul(tb, v[3]));
        } else {
            return t;
        }
    }
    // shade() packed into the target's pixel format (sel: pack_selector,
    // rsel: rgb_selector of it).
    __device__ static __forceinline__ uint32_t shade_px(const DrawDev &d, const float *v, uint32_t sel,
                                                        uint32_t rsel) {
        if constexpr (KIND == RF_K_GOURAUD) {
            // color.rs:253-263 as in to_color4, the bytes permuted at once
            return pack_rgb(as_u8(fmul(256.0f, v[1])), as_u8(fmul(256.0f, v[2])), as_u8(fmul(256.0f, v[3])), rsel);
        } else {
            return pack_px(shade(d, v), sel);
        }
    }
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

// Depth bounds of the FAST path: per lane, the minimum current depth of each
// RF_SEG-pixel segment of its tile row (shared memory, word s*32 + lane).
// Under the Less test with depth writes a pixel's depth only grows, so a
// stored minimum stays a lower bound until it is refreshed.
#define RF_SEG 8

struct TileCtx {
    uint32_t *scol;
    float *sdep;
    float *smin;
    uint32_t lane;
    uint32_t y;       // this lane's row
    uint32_t tx0;     // first column of the tile
    uint32_t tx1;     // one past the last column of the tile inside the target
    uint32_t tw;      // tile width (a power of two)
    bool row_ok;
    bool has_depth;
    int32_t depth_test;
    bool color_write, depth_write;
    uint32_t fmt;     // pack_selector of the target's pixel format
    uint32_t rfmt;    // rgb_selector of fmt
    unsigned long long frags_o;
};

// Fragments a..b-1 of one scanline into the tile (raster.rs:60-69,
// target.rs:163-198): v = varyings of fragment a, stepped by dv per pixel.
template <int KIND, bool FAST>
__device__ __forceinline__ uint32_t pixels(TileCtx &T, const DrawDev &d, float *v, const float *dv,
                                           uint32_t a, uint32_t b) {
    constexpr int NC = Kind<KIND>::NC;
    uint32_t idx = (a - T.tx0) * RF_TILE_H + T.lane;
    const uint32_t end = (b - T.tx0) * RF_TILE_H + T.lane;
    if constexpr (FAST) {
        // Four pixels per iteration: their depths are loaded together (this
        // lane alone writes its row, so they cannot change meanwhile); only
        // the running sums chain from pixel to pixel.
        uint32_t nout = 0;
        for (; idx + 3 * RF_TILE_H < end; idx += 4 * RF_TILE_H) {
            const float c0 = T.sdep[idx], c1 = T.sdep[idx + RF_TILE_H];
            const float c2 = T.sdep[idx + 2 * RF_TILE_H], c3 = T.sdep[idx + 3 * RF_TILE_H];
            float v1[NC], v2[NC], v3[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                v1[c] = fadd(v[c], dv[c]);
                v2[c] = fadd(v1[c], dv[c]);
                v3[c] = fadd(v2[c], dv[c]);
            }
            // ctx.rs:86-89 with Some(Less)
            const bool p0 = c0 < v[0], p1 = c1 < v1[0], p2 = c2 < v2[0], p3 = c3 < v3[0];
            if constexpr (Kind<KIND>::TEXTURED) {
                // The passing fragments' texels are loaded together, then used.
                uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0;
                if (p0) t0 = Kind<KIND>::texel(d, v);
                if (p1) t1 = Kind<KIND>::texel(d, v1);
                if (p2) t2 = Kind<KIND>::texel(d, v2);
                if (p3) t3 = Kind<KIND>::texel(d, v3);
                if (p0) {
                    T.scol[idx] = pack_px(Kind<KIND>::from_texel(t0, v), T.fmt);
                    T.sdep[idx] = v[0];
                    ++nout;
                }
                if (p1) {
                    T.scol[idx + RF_TILE_H] = pack_px(Kind<KIND>::from_texel(t1, v1), T.fmt);
                    T.sdep[idx + RF_TILE_H] = v1[0];
                    ++nout;
                }
                if (p2) {
                    T.scol[idx + 2 * RF_TILE_H] = pack_px(Kind<KIND>::from_texel(t2, v2), T.fmt);
                    T.sdep[idx + 2 * RF_TILE_H] = v2[0];
                    ++nout;
                }
                if (p3) {
                    T.scol[idx + 3 * RF_TILE_H] = pack_px(Kind<KIND>::from_texel(t3, v3), T.fmt);
                    T.sdep[idx + 3 * RF_TILE_H] = v3[0];
                    ++nout;
                }
            } else if constexpr (KIND == RF_K_GOURAUD_SRGB) {
                // Three powf per pixel: only the passing pixels are shaded.
                if (p0) {
                    T.scol[idx] = pack_px(Kind<KIND>::shade(d, v), T.fmt);
                    T.sdep[idx] = v[0];
                }
                if (p1) {
                    T.scol[idx + RF_TILE_H] = pack_px(Kind<KIND>::shade(d, v1), T.fmt);
                    T.sdep[idx + RF_TILE_H] = v1[0];
                }
                if (p2) {
                    T.scol[idx + 2 * RF_TILE_H] = pack_px(Kind<KIND>::shade(d, v2), T.fmt);
                    T.sdep[idx + 2 * RF_TILE_H] = v2[0];
                }
                if (p3) {
                    T.scol[idx + 3 * RF_TILE_H] = pack_px(Kind<KIND>::shade(d, v3), T.fmt);
                    T.sdep[idx + 3 * RF_TILE_H] = v3[0];
                }
                nout += (uint32_t)p0 + (uint32_t)p1 + (uint32_t)p2 + (uint32_t)p3;
            } else {
                // Flat and Gouraud shading are a few instructions and read no
                // memory: every pixel's colour is computed and only the
                // stores depend on the depth test (no branches around the
                // arithmetic).
                const uint32_t k0 = Kind<KIND>::shade_px(d, v, T.fmt, T.rfmt);
                const uint32_t k1 = Kind<KIND>::shade_px(d, v1, T.fmt, T.rfmt);
                const uint32_t k2 = Kind<KIND>::shade_px(d, v2, T.fmt, T.rfmt);
                const uint32_t k3 = Kind<KIND>::shade_px(d, v3, T.fmt, T.rfmt);
                if (p0) {
                    T.scol[idx] = k0;
                    T.sdep[idx] = v[0];
                }
                if (p1) {
                    T.scol[idx + RF_TILE_H] = k1;
                    T.sdep[idx + RF_TILE_H] = v1[0];
                }
                if (p2) {
                    T.scol[idx + 2 * RF_TILE_H] = k2;
                    T.sdep[idx + 2 * RF_TILE_H] = v2[0];
                }
                if (p3) {
                    T.scol[idx + 3 * RF_TILE_H] = k3;
                    T.sdep[idx + 3 * RF_TILE_H] = v3[0];
                }
                nout += (uint32_t)p0 + (uint32_t)p1 + (uint32_t)p2 + (uint32_t)p3;
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = fadd(v3[c], dv[c]);
        }
        for (; idx != end; idx += RF_TILE_H) {
            const float z = v[0];
            if (T.sdep[idx] < z) {
                T.scol[idx] = Kind<KIND>::shade_px(d, v, T.fmt, T.rfmt);
                T.sdep[idx] = z;
                ++nout;
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = fadd(v[c], dv[c]);
        }
        T.frags_o += nout;
        return nout;
    } else {
        for (; idx != end; idx += RF_TILE_H) {
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
                    T.scol[idx] = Kind<KIND>::shade_px(d, v, T.fmt, T.rfmt);
                    T.frags_o += 1;
                }
                if (T.has_depth && T.depth_write) T.sdep[idx] = z;
            }
    #pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = fadd(v[c], dv[c]);
        }
        return 0;
    }
}

// FAST path: the minimum current depth of segment s of the lane's row.
__device__ __forceinline__ void seg_refresh(TileCtx &T, uint32_t s) {
    const uint32_t base = s * RF_SEG * RF_TILE_H + T.lane;
    float m = T.sdep[base];
#pragma unroll
    for (uint32_t x = 1; x < RF_SEG; ++x) m = fminf(m, T.sdep[base + x * RF_TILE_H]);
    T.smin[s * RF_TILE_H + T.lane] = m;
}

// FAST path: true when no fragment a..b-1 can pass Less: an upper bound of
// the span's running z is <= the current depth of every pixel it covers.
// z_k = fl(z_{k-1} + dz) never rises when dz <= 0, so its maximum is za; for
// dz > 0 (all values positive, normal range) k <= 63 rounded additions stay
// within (1+2^-24)^k of za + k dz, and fl(za + k dz) is within (1-2^-24)^2
// of it, so fl(e * (1 + 2^-16)) bounds every z_k.  NaN z or depth never
// skips here (the comparisons are false) and never passes later.
__device__ __forceinline__ bool span_hidden(const TileCtx &T, float za, float dz, uint32_t a,
                                            uint32_t b) {
    float zhi;
    if (dz <= 0.0f) {
        zhi = za;
    } else if (dz > 0.0f && za >= 1e-30f) {
        const float e = fadd(za, fmul((float)(b - a - 1u), dz));
        zhi = fmul(e, 1.0000152587890625f);  // 1 + 2^-16
    } else {
        return false;
    }
    const uint32_t s0 = (a - T.tx0) / RF_SEG, s1 = (b - 1u - T.tx0) / RF_SEG;
    float lo = T.smin[s0 * RF_TILE_H + T.lane];
    for (uint32_t s = s0 + 1; s <= s1; ++s) lo = fminf(lo, T.smin[s * RF_TILE_H + T.lane]);
    return zhi <= lo;
}

// The lane's scanline j of half H (raster.rs:84-113), clipped to the tile,
// then its fragments (raster.rs:60-69) into the tile (target.rs:163-198).
// FAST: the default context (depth test Less, colour and depth writes on).
template <int KIND, bool FAST>
__device__ __forceinline__ void span(TileCtx &T, const DrawDev &d, const HalfRec *__restrict__ H,
                                     const HalfRuns *__restrict__ U, uint32_t j) {
    constexpr int NC = Kind<KIND>::NC;
    const float lx = row_value(H, U, RF_R_LX, j);
    const float rx = row_value(H, U, RF_R_RX, j);
    const float x0r = round_up_to_half(lx), x1r = round_up_to_half(rx);
    // xs..xe as `as usize` (target.rs:259-262), zip-truncated to the
    // fragment count, clipped to the tile.  32-bit saturating casts give the
    // same clipped range as 64-bit ones (tile columns are < 2^16), and keep
    // the conversions off the FP64 pipe.
    const uint32_t xs = as_u32(x0r);
    if (xs >= T.tx1) return;
    uint32_t xe = as_u32(x1r);
    if (xe < xs) xe = xs;
    uint32_t nfr = xe - xs;
    const uint32_t cnt = as_u32(fsub(x1r, x0r));
    if (cnt < nfr) nfr = cnt;
    const uint32_t a = xs > T.tx0 ? xs : T.tx0;
    const uint32_t b = nfr >= T.tx1 - xs ? T.tx1 : xs + nfr;
    if (a >= b) return;
    // v0 = left.next(); v0 = v0.lerp(v0.step(dv_dx), x0 - v0.x)  (raster.rs:88-102),
    // then k0 pixel steps to the tile's first column.
    const float tshift = fsub(x0r, lx);
    const uint32_t k0 = a - xs;
    float v[NC], dv[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        dv[c] = H->dvdx[c];
        const float c0 = row_value(H, U, RF_R_C + c, j);
        const float adj = fadd(c0, fmul(fsub(fadd(c0, dv[c]), c0), tshift));
        v[c] = jump(adj, dv[c], k0);
    }
    pixels<KIND, FAST>(T, d, v, dv, a, b);
}

// Which scanline of a half lands on row y: row(j) = (y0r + j) as usize =
// max(0, Y + j) with Y = y0r - 1/2.  Returns the j range [j0, j1) for row y
// (one scanline for rows below the top edge; row 0 also collects the rows
// above the buffer).
__device__ __forceinline__ void rows_for(const HalfRec *__restrict__ H, uint32_t y, uint32_t &j0,
                                         uint32_t &j1) {
    j0 = j1 = 0;
    const uint32_t n = H->n;
    const float y0r = H->y0r;
    if (n == 0 || !(fabsf(y0r) < RF_MAX_COORD)) return;
    const int32_t Y = (int32_t)fsub(y0r, 0.5f);
    if (y > 0 || Y >= 0) {
        const int64_t j = (int64_t)y - Y;
        if (j >= 0 && j < (int64_t)n) {
            j0 = (uint32_t)j;
            j1 = j0 + 1;
        }
    } else {
        j1 = (uint32_t)min((int64_t)n, (int64_t)1 - Y);
    }
}

template <int KIND, bool FAST>
__device__ __forceinline__ void raster_prim_k(TileCtx &T, const DrawDev &d, const PrimRec *__restrict__ P) {
    if (!T.row_ok) return;
    // The two halves cover disjoint rows, so each lane walks only the half
    // holding its row and both halves run in one pass of the warp.  Only
    // row 0 can take scanlines of both halves (rows above the buffer).
    uint32_t a0, a1, b0, b1;
    rows_for(&P->half[0], T.y, a0, a1);
    rows_for(&P->half[1], T.y, b0, b1);
    const bool start1 = a1 == a0;
    const HalfRec *H = start1 ? &P->half[1] : &P->half[0];
    const HalfRuns *U = start1 ? &P->runs[1] : &P->runs[0];
    uint32_t j = start1 ? b0 : a0, jend = start1 ? b1 : a1;
    bool more = !start1 && b1 > b0;
    for (;;) {
        if (j >= jend) {
            if (!more) break;
            H = &P->half[1];
            U = &P->runs[1];
            j = b0;
            jend = b1;
            more = false;
            continue;
        }
        span<KIND, FAST>(T, d, H, U, j);
        ++j;
    }
}

// Row records in shared memory: per staged triangle one slot of
// RF_ROW_WORDS(NC) words per lane, word w of lane L at w * 32 + L (the bank
// is the lane).  Each lane copies its own row's record (cp.async, 4 bytes a
// word) two triangles ahead of its use; a lane whose row the triangle does
// not cover stores word 0 = 0 (an empty span).
template <int KIND>
struct PreNC {
    static constexpr int NC = KIND == RF_K_ANY ? RF_NC : Kind<KIND == RF_K_ANY ? 0 : KIND>::NC;
};
__host__ __device__ constexpr uint32_t row_words(int nc) { return 1u + 2u * (uint32_t)nc; }

// Word indices of RasterPrim fields.
#define RF_RPW_FLAGS 1
#define RF_RPW_BASE 3
#define RF_RPW_STRIDE 4
#define RF_RPW_Y0 5
#define RF_RPW_C0 6
#define RF_RPW_Y1 7
#define RF_RPW_C1 8
#define RF_RPW_ZMAX (9 + 2 * RF_NC)
static_assert(offsetof(RasterPrim, zmax) == 4 * RF_RPW_ZMAX, "RasterPrim word layout");
static_assert(offsetof(RasterPrim, flags) == 4 * RF_RPW_FLAGS && offsetof(RasterPrim, base) == 4 * RF_RPW_BASE &&
                  offsetof(RasterPrim, stride) == 4 * RF_RPW_STRIDE && offsetof(RasterPrim, y0) == 4 * RF_RPW_Y0 &&
                  offsetof(RasterPrim, c0) == 4 * RF_RPW_C0 && offsetof(RasterPrim, y1) == 4 * RF_RPW_Y1 &&
                  offsetof(RasterPrim, c1) == 4 * RF_RPW_C1,
              "RasterPrim word layout");

// Row records of one triangle whose header H sits in shared memory;
// present = the triangle exists.  Every lane calls this together.
template <int KIND>
__device__ __forceinline__ void stage_rows(const TileCtx &T, uint32_t *slot, bool present,
                                           const RasterPrim *H, const uint32_t *__restrict__ rows) {
    const uint32_t flags = H->flags;
    const uint32_t rbase = H->base;
    const uint32_t stride = H->stride;  // 1 + 2 NC of its own kind
    const uint32_t y0 = H->y0, c0 = H->c0, y1 = H->y1, c1 = H->c1;
    uint32_t *dst = slot + T.lane;
    if (!present || !T.row_ok || (flags & (RF_RP_LIVE | RF_RP_ROWS)) != (RF_RP_LIVE | RF_RP_ROWS)) {
        dst[0] = 0u;
        return;
    }
    const uint32_t y = T.y;
    uint32_t j;
    if (y - y0 < c0) {
        j = y - y0;
    } else if (y - y1 < c1) {
        j = c0 + (y - y1);
    } else {
        dst[0] = 0u;
        return;
    }
    const uint32_t *src = rows + rbase + (size_t)j * stride;
    const uint32_t nw = KIND == RF_K_ANY ? stride : row_words(PreNC<KIND>::NC);
#pragma unroll
    for (uint32_t w = 0; w < row_words(PreNC<KIND>::NC); ++w) {
        if (w < nw) {
            const uint32_t sa = (uint32_t)__cvta_generic_to_shared(dst + w * RF_TILE_H);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(src + w) : "memory");
        }
    }
}

template <int KIND, bool FAST>
__device__ __forceinline__ void raster_rows(TileCtx &T, const DrawDev &d, const RasterPrim *__restrict__ R,
                                            uint32_t *slot) {
    constexpr int NC = Kind<KIND>::NC;
    uint32_t *rs = slot + T.lane;
    const uint32_t w0 = rs[0];
    const uint32_t xs = w0 & 0xFFFFu, xe = w0 >> 16;
    const uint32_t a = xs > T.tx0 ? xs : T.tx0;
    const uint32_t b = xe < T.tx1 ? xe : T.tx1;
    if (a >= b) return;
    const uint32_t hh = T.y - R->y0 < R->c0 ? 0u : 1u;
    // The span starts in this tile (k = 0 from its first pixel) or enters it
    // at a tile boundary at or after its first one (k steps from there).
    const bool first = a == xs;
    const uint32_t k = first ? 0u : a - ((xs & ~(T.tw - 1u)) + T.tw);
    const uint32_t off = first ? 1u : 1u + NC;
    if (k) {
        // A third or later tile of the span: step the boundary values in
        // place (the lane's own slot), one component at a time (a rolled
        // loop keeps the jump's code out of the per-component unrolling).
#pragma unroll 1
        for (int c = 0; c < NC; ++c)
            rs[(off + c) * RF_TILE_H] = f2u(jump(u2f(rs[(off + c) * RF_TILE_H]), R->dvdx[hh][c], k));
    }
    float v[NC], dv[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        dv[c] = R->dvdx[hh][c];
        v[c] = u2f(rs[(off + c) * RF_TILE_H]);
    }
    if constexpr (FAST) {
        if (span_hidden(T, v[0], dv[0], a, b)) return;
        if (pixels<KIND, FAST>(T, d, v, dv, a, b)) {
            const uint32_t s1 = (b - 1u - T.tx0) / RF_SEG;
            for (uint32_t s = (a - T.tx0) / RF_SEG; s <= s1; ++s) seg_refresh(T, s);
        }
    } else {
        pixels<KIND, FAST>(T, d, v, dv, a, b);
    }
}

template <int KIND, bool FAST>
__device__ __forceinline__ void raster_one(TileCtx &T, const DrawDev &d, const RasterPrim *__restrict__ R,
                                           const PrimRec *__restrict__ P, uint32_t *rs) {
    if (R->flags & RF_RP_ROWS) raster_rows<KIND, FAST>(T, d, R, rs);
    else raster_prim_k<KIND, FAST>(T, d, P);
}

// KIND: the shader kind of every draw of the job, or RF_K_ANY (dispatch per
// triangle).
template <int KIND, bool FAST>
__device__ __forceinline__ void raster_prim(TileCtx &T, const DrawDev *__restrict__ draws,
                                            const RasterPrim *__restrict__ R,
                                            const PrimRec *__restrict__ P, uint32_t *rs) {
    if (!(R->flags & RF_RP_LIVE)) return;
    const DrawDev &d = draws[R->draw];
    if constexpr (KIND != RF_K_ANY) {
        raster_one<KIND == RF_K_ANY ? 0 : KIND, FAST>(T, d, R, P, rs);
    } else {
        switch (R->kind) {
            case RF_K_FLAT: raster_one<RF_K_FLAT, FAST>(T, d, R, P, rs); break;
            case RF_K_GOURAUD: raster_one<RF_K_GOURAUD, FAST>(T, d, R, P, rs); break;
            case RF_K_TEXTURED: raster_one<RF_K_TEXTURED, FAST>(T, d, R, P, rs); break;
            case RF_K_TEX_GOURAUD: raster_one<RF_K_TEX_GOURAUD, FAST>(T, d, R, P, rs); break;
            default: raster_one<RF_K_GOURAUD_SRGB, FAST>(T, d, R, P, rs); break;
        }
    }
}

// FAST path: the least current depth over the tile's rows this warp owns
// (a lower bound: the segment minima are), warp-uniform.
template <int TW>
__device__ __forceinline__ float tile_depth_min(const TileCtx &T) {
    float m = __int_as_float(0x7F800000);
    if (T.row_ok)
        for (uint32_t sg = 0; sg < (uint32_t)TW / RF_SEG; ++sg) m = fminf(m, T.smin[sg * RF_TILE_H + T.lane]);
#pragma unroll
    for (int sft = 16; sft > 0; sft >>= 1) m = fminf(m, __shfl_xor_sync(0xFFFFFFFFu, m, sft));
    return m;
}

// FAST path: no fragment of triangle R can pass Less in a tile whose depths
// are all >= tzmin (R->zmax bounds its fragments' depths from above; a NaN
// on either side never skips).
template <bool FAST>
__device__ __forceinline__ bool hidden(const RasterPrim *R, float tzmin) {
    if constexpr (FAST) return R->zmax <= tzmin;
    else return false;
}

// Warp-wide selection of set bits in order: lane L offers the bits b (lane
// order, then bit order within a word); the first `want` of them go to the
// output slots first, first + 1, ...  Lane first + k learns where its bit
// came from (src lane, bit pos).  take = how many were handed out, total =
// how many were offered; end_lane / end_rest: the lane of the last bit taken
// and its bits still left.
struct WarpTake {
    uint32_t take, total, src, pos, end_lane, end_rest;
};
// Position of the r-th set bit of v (r >= 1, at most popc(v)): halving
// search on popcounts.
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t v, uint32_t r) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t w = 16; w >= 1; w >>= 1) {
        const uint32_t c = __popc(v & ((1u << w) - 1u));
        if (c < r) {
            r -= c;
            v >>= w;
            pos += w;
        }
    }
    return pos;
}
// (Out of line: it runs once per 32 triangles, and the kernels that switch
// on the shader kind per triangle are large already.)
static __device__ __noinline__ WarpTake warp_take(uint32_t b, uint32_t want, uint32_t first, uint32_t lane) {
    WarpTake t;
    const uint32_t c = __popc(b);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    t.total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    t.take = min(want, t.total);
    // Slot k = lane - first comes from the first lane whose inclusive count
    // exceeds k.
    const uint32_t k = lane - first;  // huge for lane < first: ignored
    uint32_t L = 0;
#pragma unroll
    for (uint32_t step = 16; step >= 1; step >>= 1) {
        const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, L + step - 1);
        if (v <= k) L += step;
    }
    const uint32_t ex = incl - c;
    const uint32_t exL = __shfl_sync(0xFFFFFFFFu, ex, L);
    const uint32_t bL = __shfl_sync(0xFFFFFFFFu, b, L);
    t.src = L;
    t.pos = nth_set_bit(bL, k - exL + 1u);  // (meaningless on lanes outside the take)
    // Where the take stopped: the source of slot take - 1.
    const uint32_t last = first + (t.take ? t.take : 1u) - 1u;
    t.end_lane = __shfl_sync(0xFFFFFFFFu, L, last & 31u);
    const uint32_t end_ex = __shfl_sync(0xFFFFFFFFu, exL, last & 31u);
    const uint32_t end_b = __shfl_sync(0xFFFFFFFFu, bL, last & 31u);
    const uint32_t used = t.take - end_ex;  // bits of end_lane taken
    const uint32_t lastpos = nth_set_bit(end_b, used ? used : 1u);
    t.end_rest = used ? (end_b & ~((2u << lastpos) - 1u)) : end_b;
    return t;
}

// Walks a tile's bitmask in submission order: set bits of the mask words
// (input triangles), each expanded to its clipped output triangles.  The
// tile's summary words (one bit per nonzero mask word) are read 128 at a
// time; the nonzero mask words they name are then fetched 32 at a time
// (lane e loads entry e), so an empty stretch of the mask costs nothing.
// Both gathers pick their next 32 set bits with one warp-wide prefix count
// (warp_take), not bit by bit.  The next 32 input triangles are gathered at
// once, lane k holding the k-th one's output range (toff, tcnt loaded in
// parallel), so one load latency covers 32 triangles.  Warp-uniform state;
// every lane calls next() together.
struct PrimIter {
    const uint32_t *tmask;  // the tile's mask words
    const uint32_t *tsum;   // the tile's summary words
    const uint32_t *toff;
    const uint32_t *tcnt;
    uint32_t nsum, tri_base, lane;
    // Summary words, 128 at a time: lane L holds words sb + 32 c + L in
    // s[c]; the cursor is chunk sc, lane sl, and srem = the bits of that
    // lane's word not taken yet (words of lower lanes are taken).
    uint32_t sb, s0, s1, s2, s3, sc, sl, srem;
    // Gathered mask words: lane e holds entry e (index widx, value wval),
    // wn of them; the cursor is entry wi with wrem = its bits not taken yet.
    uint32_t widx, wval, wn, wi, wrem;
    uint32_t p, pend;
    uint32_t boff, bcnt, bn;      // the gathered batch (lane k: entry k)
    uint32_t keep;                // entries of the batch still to walk
    float bz;                     // lane k: entry k's depth bound (RasterPrim::zmax; NaN: none)
    float zcut;                   // entries whose bound is <= zcut are passed over (NaN: none)
    const RasterPrim *rprims;
    uint32_t slo, shi;            // rows of a row-slice item (slo >= shi: the whole tile)
    bool started, done;           // a window was loaded; the summary words are all read

    __device__ __forceinline__ uint32_t chunk_word() const {
        return sc == 0 ? s0 : (sc == 1 ? s1 : (sc == 2 ? s2 : s3));
    }
    // The next up to 32 nonzero mask words, in order, into the word batch.
    __device__ __forceinline__ void gather_words() {
        uint32_t n = 0, mine = 0;
        for (;;) {
            if (!started || sc == 4) {  // next window of summary words
                if (started) sb += 128;
                started = true;
                if (sb >= nsum) {
                    done = true;
                    break;
                }
                const uint32_t i0 = sb + lane;
                s0 = i0 < nsum ? tsum[i0] : 0u;
                s1 = i0 + 32 < nsum ? tsum[i0 + 32] : 0u;
                s2 = i0 + 64 < nsum ? tsum[i0 + 64] : 0u;
                s3 = i0 + 96 < nsum ? tsum[i0 + 96] : 0u;
                sc = 0;
                sl = 0;
                srem = __shfl_sync(0xFFFFFFFFu, s0, 0);
            }
            const uint32_t w = chunk_word();
            const uint32_t b = lane < sl ? 0u : (lane == sl ? srem : w);
            if (__ballot_sync(0xFFFFFFFFu, b != 0u) == 0u) {  // nothing left in this chunk
                if (++sc < 4) {
                    sl = 0;
                    srem = __shfl_sync(0xFFFFFFFFu, chunk_word(), 0);
                }
                continue;
            }
            WarpTake t = warp_take(b, 32u - n, n, lane);
            if (lane >= n && lane < n + t.take) mine = (sb + sc * 32u + t.src) * 32u + t.pos;
            n += t.take;
            if (t.take < t.total) {  // stopped inside this chunk
                sl = t.end_lane;
                srem = t.end_rest;
                break;
            }
            ++sc;  // chunk used up
            if (sc < 4) {
                sl = 0;
                srem = __shfl_sync(0xFFFFFFFFu, chunk_word(), 0);
            }
            if (n == 32u) break;
        }
        wn = n;
        wi = 0;
        widx = mine;
        wval = lane < n ? tmask[mine] : 0u;
        wrem = __shfl_sync(0xFFFFFFFFu, wval, 0);
    }
    // The next up to 32 input triangles (set bits), in order: lane k holds
    // the k-th one's global index in mine; returns how many.
    __device__ __forceinline__ uint32_t gather_tris(uint32_t &mine) {
        uint32_t n = 0;
        mine = 0;
        while (n < 32u) {
            if (wi >= wn) {
                if (done) break;  // no summary words left
                gather_words();
                if (wn == 0) break;
            }
            const uint32_t b = (lane < wi || lane >= wn) ? 0u : (lane == wi ? wrem : wval);
            WarpTake t = warp_take(b, 32u - n, n, lane);
            const uint32_t wsrc = __shfl_sync(0xFFFFFFFFu, widx, t.src);
            if (lane >= n && lane < n + t.take) mine = tri_base + wsrc * 32u + t.pos;
            n += t.take;
            if (t.take < t.total) {  // stopped inside this word batch
                wi = t.end_lane;
                wrem = t.end_rest;
            } else {
                wi = wn;  // batch used up
            }
        }
        return n;
    }
    __device__ __forceinline__ void refill() {
        uint32_t mine;
        const uint32_t n = gather_tris(mine);
        bn = n;
        bool take = lane < n;
        bz = __int_as_float(0x7FFFFFFF);
        if (lane < n) {
            boff = __ldg(toff + mine);
            bcnt = __ldg(tcnt + mine);
            if (bcnt == 1u) {
                // An unclipped triangle: its depth bound, for passing it over
                // in a tile whose depths have all risen to it (next()) ...
                const uint32_t *h = reinterpret_cast<const uint32_t *>(rprims + boff);
                bz = __ldg(reinterpret_cast<const float *>(h) + RF_RPW_ZMAX);
                if (slo < shi) {
                    // ... and, in a row slice of a crowded tile, whether its
                    // rows meet the slice.
                    const uint32_t fl = __ldg(h + RF_RPW_FLAGS);
                    const uint32_t y0 = __ldg(h + RF_RPW_Y0), c0 = __ldg(h + RF_RPW_C0);
                    const uint32_t y1 = __ldg(h + RF_RPW_Y1), c1 = __ldg(h + RF_RPW_C1);
                    if (fl & RF_RP_ROWS)
                        take = (c0 && y0 < shi && y0 + c0 > slo) || (c1 && y1 < shi && y1 + c1 > slo);
                }
            }
        }
        // (entries passed over for their depth bound now are tested again
        // against the bound of the moment in next())
        keep = __ballot_sync(0xFFFFFFFFu, take && !(bz <= zcut));
    }
    __device__ __forceinline__ void init() {
        sb = s0 = s1 = s2 = s3 = sc = sl = srem = 0;
        widx = wval = wn = wi = wrem = p = pend = 0;
        boff = bcnt = bn = keep = 0;
        bz = zcut = __int_as_float(0x7FFFFFFF);
        started = done = false;
    }
    __device__ __forceinline__ uint32_t next() {
        while (p >= pend) {
            while (keep == 0u) {
                refill();
                if (bn == 0) return 0xFFFFFFFFu;
            }
            const uint32_t k = __ffs(keep) - 1;
            keep &= keep - 1u;
            // Passed over: triangles no pixel of the tile can take any more
            // (depth bound <= the tile's least depth, which only rises; a
            // NaN on either side never passes over).
            if (__shfl_sync(0xFFFFFFFFu, bz, k) <= zcut) continue;
            p = __shfl_sync(0xFFFFFFFFu, boff, k);
            pend = p + __shfl_sync(0xFFFFFFFFu, bcnt, k);
        }
        return p++;
    }
};

// Asynchronous copy of one triangle header into this warp's staging slot
// (16 bytes per lane, lanes 0..5); committed by commit_stage().
__device__ __forceinline__ void stage_prim(RasterPrim *slot, const RasterPrim *src, uint32_t lane) {
    static_assert(sizeof(RasterPrim) % 16 == 0, "RasterPrim must be a whole number of 16-byte chunks");
    static_assert(sizeof(RasterPrim) <= 64 * 16, "RasterPrim is staged in at most two rounds");
    constexpr uint32_t CHUNKS = sizeof(RasterPrim) / 16;
    if (src) {
#pragma unroll
        for (uint32_t c = lane; c < CHUNKS; c += 32) {
            const uint32_t sa = (uint32_t)__cvta_generic_to_shared(reinterpret_cast<char *>(slot) + c * 16);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa),
                         "l"(reinterpret_cast<const char *>(src) + c * 16)
                         : "memory");
        }
    }
}

// One commit group per call on every lane (copies issued since the last).
__device__ __forceinline__ void commit_stage() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

// All but the N most recent groups of this lane complete, and visible to
// the whole warp.
template <int N>
__device__ __forceinline__ void wait_staged_but() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
    __syncwarp();
}

}  // namespace rfr

// Shared-memory words per warp: colour and depth tiles, the ring of staged
// triangle headers, the ring of staged row records, the depth-segment minima.
// Pipeline distances of the rasteriser: a triangle's header is copied into
// shared memory HA triangles before its turn (a ring of HA + 1 slots), its
// row records RA before (a ring of RA + 1).
// Narrow tiles hold fewer pixels per triangle, so their iterations are
// shorter and the row records are copied further ahead.
#define RF_ROW_AHEAD_NARROW 2  // tile widths 8 and 16
#define RF_ROW_AHEAD_WIDE 2    // tile widths 32 and 64
template <int TW>
struct Pipe {
    static constexpr int RA = TW <= 16 ? RF_ROW_AHEAD_NARROW : RF_ROW_AHEAD_WIDE;
    static constexpr int HA = 2 * RA + 1 > 8 ? 2 * RA + 1 : 8;
    static constexpr uint32_t HS = (uint32_t)HA + 1u;  // header slots
    static constexpr uint32_t RS = (uint32_t)RA + 1u;  // row-record slots
};
// The header and row-record rings double as the row-major staging buffer
// of the coalesced tile load and store (32 rows of min(TW, 32) + 1 words),
// so the region is the larger of the two.
template <int TW, int KIND>
__host__ __device__ constexpr uint32_t raster_ring_words() {
    return Pipe<TW>::HS * (uint32_t)(sizeof(RasterPrim) / 4) +
           Pipe<TW>::RS * rfr::row_words(rfr::PreNC<KIND>::NC) * RF_TILE_H;
}
template <int TW>
__host__ __device__ constexpr uint32_t raster_stage_words() {
    return RF_TILE_H * ((TW < 32 ? (uint32_t)TW : 32u) + 1u);
}
template <int TW, int KIND>
__host__ __device__ constexpr uint32_t raster_warp_words() {
    return 2u * TW * RF_TILE_H +
           (raster_ring_words<TW, KIND>() > raster_stage_words<TW>() ? raster_ring_words<TW, KIND>()
                                                                     : raster_stage_words<TW>()) +
           ((uint32_t)TW / RF_SEG) * RF_TILE_H;
}

namespace rfr {

// Coalesced transfer between a tile's global rows and its column-major
// shared-memory copy (word x * 32 + r): 16-byte accesses with the lanes of a
// row side by side (8 lanes per 128 bytes), through a row-major staging
// buffer of stride CB + 1 (CB = columns per pass, at most 32) whose odd
// stride keeps both sides free of bank conflicts.  Only the rows with bit r
// of `want` set are moved.  Every moved row must hold TW columns inside the
// target and start 16-byte aligned.
template <int TW, bool LOAD>
__device__ __forceinline__ void tile_rows_coalesced(uint32_t *__restrict__ tile, uint32_t *__restrict__ stg,
                                                    uint32_t *__restrict__ g, uint32_t pitch,
                                                    uint32_t want, uint32_t lane) {
    constexpr uint32_t CB = TW < 32 ? TW : 32;   // columns per pass
    constexpr uint32_t LPR = CB / 4;             // lanes per row
    constexpr uint32_t RPI = 32 / LPR;           // rows per instruction
    constexpr uint32_t SS = CB + 1;              // staging stride
    const uint32_t lr = lane / LPR, lc = (lane % LPR) * 4;
#pragma unroll 1
    for (uint32_t x0 = 0; x0 < (uint32_t)TW; x0 += CB) {
        if constexpr (LOAD) {
#pragma unroll
            for (uint32_t r0 = 0; r0 < 32; r0 += RPI) {
                const uint32_t r = r0 + lr;
                if ((want >> r) & 1u) {
                    const uint4 v = *reinterpret_cast<const uint4 *>(g + (size_t)r * pitch + x0 + lc);
                    uint32_t *d = stg + r * SS + lc;
                    d[0] = v.x;
                    d[1] = v.y;
                    d[2] = v.z;
                    d[3] = v.w;
                }
            }
            __syncwarp();
#pragma unroll 4
            for (uint32_t x = 0; x < CB; ++x) tile[(x0 + x) * RF_TILE_H + lane] = stg[lane * SS + x];
            __syncwarp();
        } else {
#pragma unroll 4
            for (uint32_t x = 0; x < CB; ++x) stg[lane * SS + x] = tile[(x0 + x) * RF_TILE_H + lane];
            __syncwarp();
#pragma unroll
            for (uint32_t r0 = 0; r0 < 32; r0 += RPI) {
                const uint32_t r = r0 + lr;
                if ((want >> r) & 1u) {
                    const uint32_t *sp = stg + r * SS + lc;
                    *reinterpret_cast<uint4 *>(g + (size_t)r * pitch + x0 + lc) = make_uint4(sp[0], sp[1], sp[2], sp[3]);
                }
            }
            __syncwarp();
        }
    }
}

// The tile's write-back as bulk copies (cp.async.bulk, the copy engine's
// untiled form), for tiles of whole 32-column blocks whose rows start
// 16-byte aligned.  Each 32 x 32 block of the column-major colour tile,
// then of the depth tile, is transposed into 32 rows of exactly 128 bytes
// -- lane r writes word x of row r at step k = x - r (mod 32), so both the
// column reads and the row writes hit 32 different banks -- and lane r
// hands row r to the copy engine as one 128-byte copy.  The first block
// goes to the staging area, every later one into the block read just
// before it (free once read), so no copy is waited for here: the caller
// waits (bulk_store_drain) before it next writes the tile or the staging
// area.  Rows without bit r of `want` are not copied.
template <int TW>
__device__ __forceinline__ void tile_store_bulk(uint32_t *__restrict__ scol, uint32_t *__restrict__ sdep,
                                                bool has_depth, uint32_t *__restrict__ stg,
                                                uint32_t *__restrict__ gcol, uint32_t *__restrict__ gdep,
                                                uint32_t pitch, uint32_t want, uint32_t lane) {
    static_assert(TW % 32 == 0, "whole 32-column blocks");
    constexpr uint32_t NB = (uint32_t)TW / 32u, BW = 32u * RF_TILE_H;  // blocks per buffer, words per block
    uint32_t *dst = stg;
#pragma unroll 1
    for (uint32_t m = 0; m < (has_depth ? 2u * NB : NB); ++m) {
        const uint32_t bi = m < NB ? m : m - NB;  // block within its buffer
        uint32_t *src = (m < NB ? scol : sdep) + bi * BW;
        uint32_t *g = (m < NB ? gcol : gdep) + bi * 32u;
#pragma unroll 8
        for (uint32_t k = 0; k < 32; ++k) {
            const uint32_t x = (lane + k) & 31u;
            dst[lane * 32 + x] = src[x * RF_TILE_H + lane];
        }
        // (rows written through the generic path, read by the copy engine)
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncwarp();
        if ((want >> lane) & 1u) {
            const uint32_t sa = (uint32_t)__cvta_generic_to_shared(dst + lane * 32);
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], 128;\n" ::"l"(
                             g + (size_t)lane * pitch),
                         "r"(sa)
                         : "memory");
        }
        dst = src;
    }
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}

// Every bulk copy this lane issued has read its shared-memory source (the
// tile and the staging area may be written again once the warp is past it).
__device__ __forceinline__ void bulk_store_drain() {
    asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
    __syncwarp();
}

}  // namespace rfr

// KIND: shader kind of every draw of the job (or RF_K_ANY); FAST: the
// default context (depth test Less, colour and depth writes) on a target
// with depth.
template <int TW, int KIND, bool FAST>
__global__ void __launch_bounds__(RF_RASTER_MAX_THREADS, 2)
k_raster(const JobDev *__restrict__ jobs, uint32_t nj, const DrawDev *__restrict__ draws,
         const PrimRec *__restrict__ prims, const RasterPrim *__restrict__ rprims,
         const uint32_t *__restrict__ rows, const uint32_t *__restrict__ tcnt,
         const uint32_t *__restrict__ toff, const uint32_t *__restrict__ mask,
         uint32_t ntiles_total, const uint32_t *__restrict__ items, const uint32_t *__restrict__ nitems_dev,
         uint32_t *__restrict__ tile_queue, StatsDev *__restrict__ stats) {
    using namespace rfr;
    extern __shared__ __align__(16) uint32_t smem[];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr uint32_t WARP_WORDS = raster_warp_words<TW, KIND>();
    static_assert(WARP_WORDS % 4u == 0u && (2u * TW * RF_TILE_H) % 4u == 0u,
                  "each warp's area and its staging start 16-byte aligned (bulk copies)");
    constexpr uint32_t RW = row_words(PreNC<KIND>::NC) * RF_TILE_H;  // words per row slot
    uint32_t *scol = smem + warp * WARP_WORDS;
    float *sdep = reinterpret_cast<float *>(scol + TW * RF_TILE_H);
    RasterPrim *stage = reinterpret_cast<RasterPrim *>(scol + 2 * TW * RF_TILE_H);
    uint32_t *rslots = scol + 2 * TW * RF_TILE_H + Pipe<TW>::HS * (sizeof(RasterPrim) / 4);
    uint32_t *stg = scol + 2 * TW * RF_TILE_H;  // tile staging (the rings, when idle)
    float *smin = reinterpret_cast<float *>(scol + WARP_WORDS - ((uint32_t)TW / RF_SEG) * RF_TILE_H);
    // Queue position q: the heavy tiles and crowded-tile slices first
    // (items[ntiles + q]), then every other tile in index order.
    const uint32_t nfirst = *nitems_dev;
    const uint32_t nitems = ntiles_total + nfirst;
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) {
            do {
                const uint32_t pos = atomicAdd(tile_queue, 1u);
                item = pos >= nitems ? 0xFFFFFFFFu
                                     : items[pos < nfirst ? ntiles_total + pos : pos - nfirst];
            } while (item == RF_ITEM_SKIP);
        }
        item = __shfl_sync(0xFFFFFFFFu, item, 0);
        if (item == 0xFFFFFFFFu) break;
        const uint32_t tile = item >> RF_ITEM_SHIFT, slice = item & ((1u << RF_ITEM_SHIFT) - 1u);  // 0: the whole tile
        if (tile >= ntiles_total) break;
        if constexpr (TW % 32 == 0) bulk_store_drain();  // (the last tile's write-back)
        const uint32_t ji = upper_index(nj, tile, [&](uint32_t i) { return jobs[i].tile_base; });
        const JobDev &J = jobs[ji];
        const uint32_t lt = tile - J.tile_base;
        const uint32_t tyi = lt / J.tiles_x, txi = lt - tyi * J.tiles_x;
        TileCtx T;
        T.scol = scol;
        T.sdep = sdep;
        T.smin = smin;
        T.lane = lane;
        T.tx0 = txi * TW;
        T.tx1 = min(T.tx0 + (uint32_t)TW, J.w);
        T.tw = TW;
        const uint32_t ty0 = tyi * RF_TILE_H;
        T.y = ty0 + lane;
        constexpr uint32_t SLICE_H = RF_TILE_H / RF_SPLIT_K;
        T.row_ok = T.y < J.h && (slice == 0 || lane / SLICE_H == slice - 1u);
        T.has_depth = J.depth != nullptr;
        T.depth_test = J.depth_test;
        T.color_write = J.color_write != 0;
        T.depth_write = J.depth_write != 0;
        T.fmt = pack_selector(J.pixfmt);
        T.rfmt = rgb_selector(T.fmt);
        T.frags_o = 0;
        const uint32_t ncols = T.tx1 - T.tx0;
        const size_t row_off = (size_t)T.y * J.w + T.tx0;
        const uint32_t rows_ok = __ballot_sync(0xFFFFFFFFu, T.row_ok);
        // Coalesced 16-byte row transfers (tile_rows_coalesced) when the
        // tile's rows hold its full width and start 16-byte aligned.
        const bool vec = ((J.w | T.tx0) & 3u) == 0u && ncols == (uint32_t)TW &&
                         (((uintptr_t)J.color | (uintptr_t)J.depth) & 15u) == 0u;
        uint32_t *gcol = J.color + (size_t)ty0 * J.w + T.tx0;
        uint32_t *gdep = reinterpret_cast<uint32_t *>(J.depth) + (size_t)ty0 * J.w + T.tx0;
        bool loaded = false;
        auto load_tile = [&]() {
            const bool cc = J.clear_flags & 1u, cd = (J.clear_flags & 2u) != 0u;
            if (vec) {
                if (cc) {
                    for (uint32_t x = 0; x < (uint32_t)TW; ++x) scol[x * RF_TILE_H + lane] = J.clear_px;
                } else {
                    tile_rows_coalesced<TW, true>(scol, stg, gcol, J.w, rows_ok, lane);
                }
                if (T.has_depth) {
                    if (cd) {
                        for (uint32_t x = 0; x < (uint32_t)TW; ++x) sdep[x * RF_TILE_H + lane] = J.clear_z;
                    } else {
                        tile_rows_coalesced<TW, true>(reinterpret_cast<uint32_t *>(sdep), stg, gdep, J.w,
                                                      rows_ok, lane);
                    }
                }
            } else {
                for (uint32_t x = 0; x < (uint32_t)TW; ++x) {
                    const uint32_t i = x * RF_TILE_H + lane;
                    const bool in = T.row_ok && x < ncols;
                    scol[i] = cc ? J.clear_px : (in ? J.color[row_off + x] : 0u);
                    if (T.has_depth) sdep[i] = cd ? J.clear_z : (in ? J.depth[row_off + x] : 0.0f);
                }
            }
        };
        // FAST: the tile's least current depth (a lower bound of every pixel
        // a span may write), for skipping whole triangles (RasterPrim::zmax).
        // Columns past the target's edge hold +inf, so they bound nothing
        // (they are never written back).
        float tzmin = 0.0f;
        auto load_tile_and_bounds = [&]() {
            load_tile();
            if constexpr (FAST) {
                for (uint32_t x = ncols; x < (uint32_t)TW; ++x) sdep[x * RF_TILE_H + lane] = __int_as_float(0x7F800000);
                for (uint32_t sg = 0; sg < (uint32_t)TW / RF_SEG; ++sg) seg_refresh(T, sg);
                tzmin = tile_depth_min<TW>(T);
            }
        };
        PrimIter it;
        it.tmask = mask + J.mask_base + (size_t)lt * J.mask_words;
        it.tsum = mask + J.sum_base + (size_t)lt * J.sum_words;
        it.toff = toff;
        it.tcnt = tcnt;
        it.nsum = J.sum_words;
        it.rprims = rprims;
        it.slo = slice ? tyi * RF_TILE_H + (slice - 1u) * SLICE_H : 0u;
        it.shi = slice ? it.slo + SLICE_H : 0u;
        it.tri_base = J.tri_base;
        it.lane = lane;
        it.init();
        // Software pipeline over the tile's triangles t0, t1, ...: iteration
        // i rasterises t_i while the headers of t_{i+1} .. t_{i+HA} and the
        // row records of t_{i+1} .. t_{i+RA} are in flight (cp.async into
        // the shared-memory rings).  Iteration i issues the header of
        // t_{i+HA} and the rows of t_{i+RA} as one commit group G_i, then
        // waits for all but the newest RA groups: the rows of t_i (G_{i-RA})
        // and every header up to t_{i+HA-RA} are then complete.  The rows of
        // t_{i+RA} need its header, from G_{i+RA-HA}, complete by the wait of
        // iteration i-1 since HA >= 2 RA + 1.
        constexpr uint32_t NONE = 0xFFFFFFFFu;
        constexpr int HA = Pipe<TW>::HA, RA = Pipe<TW>::RA;
        constexpr uint32_t HS = Pipe<TW>::HS, RS = Pipe<TW>::RS;
        static_assert(RA >= 1 && HA >= 2 * RA + 1 && HS == (uint32_t)HA + 1u, "pipeline shape");
        uint32_t q[HA + 1];  // t_i .. t_{i+HA}
        q[0] = it.next();
        if (q[0] != NONE) {
            load_tile_and_bounds();
            loaded = true;
            if constexpr (FAST) it.zcut = tzmin;
#pragma unroll
            for (int k = 1; k <= HA; ++k) q[k] = q[k - 1] != NONE ? it.next() : NONE;
            // Headers of t_0 .. t_{HA-1} (t_{HA} comes with G_0), waited
            // for at once before the first row records are staged.
#pragma unroll
            for (int k = 0; k < HA; ++k)
                if (q[k] != NONE) stage_prim(stage + k, rprims + q[k], lane);
            commit_stage();
            wait_staged_but<0>();
#pragma unroll
            for (int k = 0; k < RA; ++k) {
                stage_rows<KIND>(T, rslots + k * RW, q[k] != NONE && !hidden<FAST>(stage + k, tzmin), stage + k, rows);
                commit_stage();
            }
            uint32_t r = 0;  // row slot of t_i (mod RA+1)
            uint32_t h = 0;  // header slot of t_i (mod HA+1)
            uint32_t visits = 0;  // triangles rasterised (FAST: tzmin refreshed every 8)
            for (;;) {
                const uint32_t hn = h == 0 ? HS - 1 : h - 1;                // t_{i+HA}: t_{i-1}'s old slot
                const uint32_t hr = h + RA >= HS ? h + RA - HS : h + RA;    // t_{i+RA}
                const uint32_t rr = r == 0 ? RS - 1 : r - 1;                // t_{i+RA}: t_{i-1}'s old slot
                if (q[HA] != NONE) stage_prim(stage + hn, rprims + q[HA], lane);
                // A triangle whose depth bound is at most the tile's least
                // depth fails the Less test at every pixel: its rows are not
                // fetched and its visit is skipped (the tile's depths only rise).
                stage_rows<KIND>(T, rslots + rr * RW, q[RA] != NONE && !hidden<FAST>(stage + hr, tzmin),
                                 stage + hr, rows);
                commit_stage();
                wait_staged_but<RA>();
                if (!hidden<FAST>(stage + h, tzmin)) {
                    raster_prim<KIND, FAST>(T, draws, stage + h, prims + q[0], rslots + r * RW);
                    if constexpr (FAST) {
                        if ((++visits & 7u) == 0u) it.zcut = tzmin = tile_depth_min<TW>(T);
                    }
                }
                __syncwarp();
                if (q[1] == NONE) break;
                const uint32_t qn = q[HA] != NONE ? it.next() : NONE;
#pragma unroll
                for (int k = 0; k < HA; ++k) q[k] = q[k + 1];
                q[HA] = qn;
                r = r + 1 == RS ? 0 : r + 1;
                h = h + 1 == HS ? 0 : h + 1;
            }
            asm volatile("cp.async.wait_all;\n" ::: "memory");
            __syncwarp();
        }
        if (!loaded && J.clear_flags) {
            load_tile();
            loaded = true;
        }
        if (loaded) {
            if (vec) {
                if constexpr (TW % 32 == 0) {
                    tile_store_bulk<TW>(scol, reinterpret_cast<uint32_t *>(sdep), T.has_depth, stg, gcol, gdep,
                                        J.w, rows_ok, lane);
                } else {
                    tile_rows_coalesced<TW, false>(scol, stg, gcol, J.w, rows_ok, lane);
                    if (T.has_depth)
                        tile_rows_coalesced<TW, false>(reinterpret_cast<uint32_t *>(sdep), stg, gdep, J.w,
                                                       rows_ok, lane);
                }
            } else if (T.row_ok) {
                for (uint32_t x = 0; x < ncols; ++x) {
                    const uint32_t i = x * RF_TILE_H + lane;
                    J.color[row_off + x] = scol[i];
                    if (T.has_depth) J.depth[row_off + x] = sdep[i];
                }
            }
        }
        __syncwarp();
        const uint32_t j0 = __shfl_sync(0xFFFFFFFFu, ji, 0);
        warp_add_u64(&stats[j0].frags_o, T.frags_o, true);
    }
    // (shared memory stays allocated until the last write-back has read it)
    if constexpr (TW % 32 == 0) bulk_store_drain();
}

namespace rfk {

// The opt-in to more than 48 KB of dynamic shared memory is a property of
// each kernel on each device: set once per (kernel, device) -- the flags
// live in the instantiation for that kernel (Tag), since every k_raster
// variant has the same function type -- under a lock so host threads
// driving contexts on several devices may launch concurrently, and with
// its status returned.
template <class Tag, class K>
static cudaError_t opt_in_smem(K kernel, int bytes) {
    constexpr int MAX_DEV = 64;
    static std::mutex mu;
    static bool done[MAX_DEV] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEV) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    std::lock_guard<std::mutex> lk(mu);
    if (!done[dev]) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        done[dev] = true;
    }
    return cudaSuccess;
}

template <int TW, int KIND, bool FAST>
static cudaError_t launch_raster_k(const JobDev *jobs, uint32_t nj, const DrawDev *draws,
                                   const PrimRec *prims, const RasterPrim *rprims,
                                   const uint32_t *rows, const uint32_t *tcnt,
                                   const uint32_t *toff, const uint32_t *mask, uint32_t ntiles,
                                   const uint32_t *items, const uint32_t *nitems, uint32_t *queue,
                                   StatsDev *stats, uint32_t warps, int nsm, cudaStream_t s) {
    // Shared memory per block: at most the 227 KB opt-in limit, so the
    // block takes as many warps as fit (wide tiles of the generic kind).
    constexpr size_t SMEM_MAX = 227 * 1024;
    constexpr size_t per_warp = (size_t)raster_warp_words<TW, KIND>() * 4;
    if ((size_t)warps * per_warp > SMEM_MAX) warps = (uint32_t)(SMEM_MAX / per_warp);
    const size_t smem = (size_t)warps * per_warp;
    struct Tag {};  // one per (TW, KIND, FAST)
    cudaError_t e = opt_in_smem<Tag>(k_raster<TW, KIND, FAST>, (int)SMEM_MAX);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raster<TW, KIND, FAST>, warps * 32, smem);
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)per_sm * (uint32_t)nsm;
    const uint32_t need = (ntiles + warps - 1) / warps;  // (a few crowded-tile slices more are shared out)
    if (blocks > need) blocks = need;
    if (blocks == 0) blocks = 1;
    k_raster<TW, KIND, FAST><<<blocks, warps * 32, smem, s>>>(jobs, nj, draws, prims, rprims, rows,
                                                             tcnt, toff, mask, ntiles, items, nitems, queue, stats);
    return cudaGetLastError();
}

// Launcher for one tile width: picks the kernel specialised for the job's
// shader kind and context (fast = the default context on a depth target;
// any other context runs the generic kernel).
template <int TW>
static cudaError_t launch_raster_for_width(int kind, bool fast, const JobDev *jobs, uint32_t nj,
                                           const DrawDev *draws, const PrimRec *prims,
                                           const RasterPrim *rprims, const uint32_t *rows,
                                           const uint32_t *tcnt, const uint32_t *toff,
                                           const uint32_t *mask, uint32_t ntiles, const uint32_t *items, const uint32_t *nitems,
                          uint32_t *queue,
                                           StatsDev *stats, uint32_t warps, int nsm, cudaStream_t s) {
    if (!fast)
        return launch_raster_k<TW, RF_K_ANY, false>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
    switch (kind) {
        case RF_K_FLAT:
            return launch_raster_k<TW, RF_K_FLAT, true>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        case RF_K_GOURAUD:
            return launch_raster_k<TW, RF_K_GOURAUD, true>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        case RF_K_TEXTURED:
            return launch_raster_k<TW, RF_K_TEXTURED, true>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        case RF_K_TEX_GOURAUD:
            return launch_raster_k<TW, RF_K_TEX_GOURAUD, true>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        case RF_K_GOURAUD_SRGB:
            return launch_raster_k<TW, RF_K_GOURAUD_SRGB, true>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
        default:
            return launch_raster_k<TW, RF_K_ANY, true>(jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask, ntiles, items, nitems, queue, stats, warps, nsm, s);
    }
}

}  // namespace rfk

#endif
