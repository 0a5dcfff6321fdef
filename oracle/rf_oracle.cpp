// rf_oracle.cpp — CPU restatement of retrofire's triangle render path.
//
// TEST INFRASTRUCTURE ONLY (see rf_oracle.h).  Each function cites the
// reference file:line it restates (paths relative to the retrofire tree).
// The arithmetic is written in the reference's operation order with f32
// only, and the file must be compiled with -ffp-contract=off so that no
// a*b+c is fused: Rust evaluates every f32 operation with one rounding.
//
// Rust `as` casts from f32 saturate (NaN -> 0); C++ casts of out-of-range
// floats are undefined, so every cast goes through an explicit helper.

#include "rf_oracle.h"

#include <cmath>
#include <algorithm>
#include <utility>
#include <vector>
#include <cstring>

namespace {

// ---------------------------------------------------------------- casts ---
// Rust `f32 as usize` / `as u32` / `as i32` / `as u8` (saturating).
inline uint64_t as_usize(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)x;
}
inline uint32_t as_u32(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 4294967296.0f) return UINT32_MAX;
    return (uint32_t)x;
}
inline int32_t as_i32(float x) {
    if (x != x) return 0;
    if (x <= -2147483648.0f) return INT32_MIN;
    if (x >= 2147483648.0f) return INT32_MAX;
    return (int32_t)x;
}
inline uint8_t as_u8(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 255.0f) return 255;
    return (uint8_t)x;
}

// f32::total_cmp (core::f32): order by sign-magnitude flipped bits.
inline int32_t total_key(float x) {
    int32_t i;
    std::memcpy(&i, &x, 4);
    i ^= (int32_t)(((uint32_t)(i >> 31)) >> 1);
    return i;
}

// raster.rs:304-307 round_up_to_half; float.rs (std) floor is exact.
inline float round_up_to_half(float x) { return std::floor(x + 0.5f) + 0.5f; }

// vec.rs:231-238 dot: zip-map-mul then fold from 0.0 with add.
inline float dot4(const float *a, const float *b) {
    float acc = 0.0f;
    acc = acc + a[0] * b[0];
    acc = acc + a[1] * b[1];
    acc = acc + a[2] * b[2];
    acc = acc + a[3] * b[3];
    return acc;
}

// ------------------------------------------------------------- clipping ---
// clip.rs:215-222 PLANES (normal x,y,z and -offset), bits 1..32.
const float PLANES[6][4] = {
    {0.0f, 0.0f, -1.0f, -1.0f},  // near   0x01
    {0.0f, 0.0f, 1.0f, -1.0f},   // far    0x02
    {-1.0f, 0.0f, 0.0f, -1.0f},  // left   0x04
    {1.0f, 0.0f, 0.0f, -1.0f},   // right  0x08
    {0.0f, -1.0f, 0.0f, -1.0f},  // bottom 0x10
    {0.0f, 1.0f, 0.0f, -1.0f},   // top    0x20
};

template <int NA>
struct ClipVert {  // clip.rs:57-61
    float pos[4];
    float a[NA > 0 ? NA : 1];
    uint8_t oc;
};

// clip.rs:240-242 outcode = sum of (signed_dist > 0) * bit (clip.rs:101-111).
inline uint8_t outcode(const float *p) {
    uint8_t oc = 0;
    for (int i = 0; i < 6; ++i) oc = (uint8_t)(oc + ((dot4(PLANES[i], p) > 0.0f) ? (1u << i) : 0u));
    return oc;
}

// clip.rs:121-145 ClipPlane::intersect.
template <int NA>
bool intersect(int plane, const ClipVert<NA> &v0, const ClipVert<NA> &v1, ClipVert<NA> &out) {
    float d0 = dot4(PLANES[plane], v0.pos);
    float d1 = dot4(PLANES[plane], v1.pos);
    if (!(d0 * d1 < 0.0f)) return false;
    float t = -d0 / (d1 - d0);
    // Lerp (math.rs:196-198): self + (other - self) * t per component.
    for (int i = 0; i < 4; ++i) out.pos[i] = v0.pos[i] + (v1.pos[i] - v0.pos[i]) * t;
    for (int i = 0; i < NA; ++i) out.a[i] = v0.a[i] + (v1.a[i] - v0.a[i]) * t;
    out.oc = outcode(out.pos);  // ClipVert::new, clip.rs:303-309
    return true;
}

// Polygon capacity.  A triangle clipped by six planes has at most nine
// vertices; the cap only bounds pathological inputs (the reference's Vec
// would grow instead).
constexpr int POLY_CAP = 64;

// clip.rs:167-193 ClipPlane::clip_simple_polygon.
template <int NA>
int clip_poly_plane(int plane, const ClipVert<NA> *in, int nin, ClipVert<NA> *out) {
    int nout = 0;
    if (nin == 0) return 0;
    const uint8_t bit = (uint8_t)(1u << plane);
    for (int i = 0; i < nin; ++i) {
        const ClipVert<NA> &v0 = in[i];
        const ClipVert<NA> &v1 = in[(i + 1) % nin];  // chain(&verts_in[..1])
        if ((v0.oc & bit) == 0 && nout < POLY_CAP) out[nout++] = v0;
        ClipVert<NA> v;
        if (intersect<NA>(plane, v0, v1, v) && nout < POLY_CAP) out[nout++] = v;
    }
    return nout;
}

// clip.rs:350-400 Clip for [Tri]: status, Sutherland-Hodgman, fan.
// Returns the number of triangles written to out (<= POLY_CAP - 2).
template <int NA>
int clip_tri(const ClipVert<NA> tri[3], ClipVert<NA> out[][3]) {
    // clip.rs:245-267 status
    uint8_t all_out = 0xFF, any_out = 0;
    for (int i = 0; i < 3; ++i) {
        all_out &= tri[i].oc;
        any_out |= tri[i].oc;
    }
    if (all_out != 0) return 0;  // Hidden
    if (any_out == 0) {          // Visible
        for (int i = 0; i < 3; ++i) out[0][i] = tri[i];
        return 1;
    }
    // clip.rs:283-301 clip_simple_polygon over the six planes in order.
    ClipVert<NA> bufa[POLY_CAP], bufb[POLY_CAP];
    ClipVert<NA> *vin = bufa, *vout = bufb;
    int nin = 3, nout = 0;
    for (int i = 0; i < 3; ++i) vin[i] = tri[i];
    for (int p = 0; p < 6; ++p) {
        nout = clip_poly_plane<NA>(p, vin, nin, vout);
        nin = 0;
        if (nout == 0) break;
        if (p < 5) {
            ClipVert<NA> *t = vin;
            vin = vout;
            vout = t;
            nin = nout;
            nout = 0;
        }
    }
    // Fan [p, rest[i], rest[i+1]] (clip.rs:373-396).
    int n = 0;
    for (int i = 1; i + 1 < nout; ++i) {
        out[n][0] = vout[0];
        out[n][1] = vout[i];
        out[n][2] = vout[i + 1];
        ++n;
    }
    return n;
}

// ------------------------------------------------------------ raster ---
// Varyings<V> = (ScreenPt, V): three position floats then NA attributes.
template <int NA>
struct Var {
    float p[3];
    float a[NA > 0 ? NA : 1];
};

// Lerp for tuples / Point3 / Vector / Color3f: self + (other - self) * t.
template <int NA>
inline Var<NA> vlerp(const Var<NA> &s, const Var<NA> &o, float t) {
    Var<NA> r{};
    for (int i = 0; i < 3; ++i) r.p[i] = s.p[i] + (o.p[i] - s.p[i]) * t;
    for (int i = 0; i < NA; ++i) r.a[i] = s.a[i] + (o.a[i] - s.a[i]) * t;
    return r;
}
// Vary::step (space.rs:211-214): self + delta.
template <int NA>
inline Var<NA> vstep(const Var<NA> &s, const Var<NA> &d) {
    Var<NA> r{};
    for (int i = 0; i < 3; ++i) r.p[i] = s.p[i] + d.p[i];
    for (int i = 0; i < NA; ++i) r.a[i] = s.a[i] + d.a[i];
    return r;
}
// Vary::dv_dt (space.rs:205-208): (other - self) * recip_dt.
template <int NA>
inline Var<NA> vdvdt(const Var<NA> &s, const Var<NA> &o, float recip) {
    Var<NA> r{};
    for (int i = 0; i < 3; ++i) r.p[i] = (o.p[i] - s.p[i]) * recip;
    for (int i = 0; i < NA; ++i) r.a[i] = (o.a[i] - s.a[i]) * recip;
    return r;
}

// raster.rs:45-51 ScanlineIter state.
template <int NA>
struct ScanIter {
    float y;
    Var<NA> left, dl;
    float right, dr;
    Var<NA> dv_dx;
    uint32_t n;
};

// raster.rs:248-302 scan().
template <int NA>
ScanIter<NA> scan(float y0, float y1, const Var<NA> &l0, const Var<NA> &l1,
                  const Var<NA> &r0, const Var<NA> &r1) {
    float recip_dy = 1.0f / (y1 - y0);
    Var<NA> dl_dy = vdvdt(l0, l1, recip_dy);
    Var<NA> dr_dy = vdvdt(r0, r1, recip_dy);
    Var<NA> l0s = vstep(l0, dl_dy), r0s = vstep(r0, dr_dy);
    float dx = r0s.p[0] - l0s.p[0];
    Var<NA> dv_dx = vdvdt(l0s, r0s, 1.0f / dx);
    float y0r = round_up_to_half(y0);
    float y1r = round_up_to_half(y1);
    float y_tweak = y0r - y0;
    ScanIter<NA> it;
    it.y = y0r;
    it.left = vlerp(l0, vstep(l0, dl_dy), y_tweak);
    it.dl = dl_dy;
    it.right = r0.p[0] + dr_dy.p[0] * y_tweak;
    it.dr = dr_dy.p[0];
    it.dv_dx = dv_dx;
    it.n = as_u32(y1r - y0r);
    return it;
}

// A scanline as emitted by ScanlineIter::next (raster.rs:80-114).
template <int NA>
struct Scanline {
    uint64_t y, x0, x1;  // y, xs.start, xs.end (usize)
    Var<NA> v0;          // varyings of the first fragment
    Var<NA> dv_dx;
    uint32_t count;      // vary(..., Some(count))
};

// Scanline origins beyond +-2^22 px are outside the supported domain (the
// row arithmetic y0r + j stops being exact); such a half is skipped and
// reported through `oob` instead of being walked.
constexpr float MAX_COORD = 4194304.0f;

// raster.rs:80-114 + vary.rs:142-155: emits every scanline of one half.
template <int NA, class F, class G>
void run_scan(ScanIter<NA> it, F &&f, G &&oob) {
    if (it.n != 0 && !(std::fabs(it.y) < MAX_COORD)) {
        oob();
        return;
    }
    while (it.n != 0) {
        Var<NA> v0 = it.left;                 // left.next(): current value ...
        it.left = vstep(it.left, it.dl);      // ... then step
        float x1 = it.right;
        it.right = it.right + it.dr;
        float x0r = round_up_to_half(v0.p[0]);
        float x1r = round_up_to_half(x1);
        Scanline<NA> sl;
        sl.v0 = vlerp(v0, vstep(v0, it.dv_dx), x0r - v0.p[0]);
        sl.dv_dx = it.dv_dx;
        sl.count = as_u32(x1r - x0r);
        sl.y = as_usize(it.y);
        sl.x0 = as_usize(x0r);
        sl.x1 = as_usize(x1r);
        it.y = it.y + 1.0f;
        it.n -= 1;
        f(sl);
    }
}

// raster.rs:185-224 tri_fill.
template <int NA, class F, class G>
void tri_fill(const Var<NA> verts_in[3], F &&f, G &&oob) {
    // Stable sort by y with total_cmp (slice::sort_by is stable).
    Var<NA> v[3] = {verts_in[0], verts_in[1], verts_in[2]};
    for (int i = 1; i < 3; ++i)
        for (int j = i; j > 0 && total_key(v[j - 1].p[1]) > total_key(v[j].p[1]); --j) {
            Var<NA> t = v[j];
            v[j] = v[j - 1];
            v[j - 1] = t;
        }
    const Var<NA> &top = v[0], &mid0 = v[1], &bot = v[2];
    float top_y = top.p[1], mid_y = mid0.p[1], bot_y = bot.p[1];
    Var<NA> mid1 = vlerp(top, bot, (mid_y - top_y) / (bot_y - top_y));
    const Var<NA> &left = (mid0.p[0] < mid1.p[0]) ? mid0 : mid1;
    const Var<NA> &right = (mid0.p[0] < mid1.p[0]) ? mid1 : mid0;
    run_scan<NA>(scan<NA>(top_y, mid_y, top, left, top, right), f, oob);
    run_scan<NA>(scan<NA>(mid_y, bot_y, left, bot, right, bot), f, oob);
}

// ------------------------------------------------------------ shading ---
inline uint32_t rgba_pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return r | (g << 8) | (b << 16) | (a << 24);
}

// tex.rs:218-357 samplers on a Texture<Buf2<Color4>> (row-major, stride w).
inline uint32_t sample(const rfo_draw *d, float tu, float tv) {
    float w = (float)d->tw, h = (float)d->th;
    uint32_t u, v;
    if (d->sampler == RFO_REPEAT_POT) {  // tex.rs:240-266
        float su = w * tu, sv = h * tv;
        u = (uint32_t)as_i32(std::floor(su)) & (d->tw - 1);
        v = (uint32_t)as_i32(std::floor(sv)) & (d->th - 1);
    } else if (d->sampler == RFO_CLAMP) {  // tex.rs:272-304
        float su = tu * w, sv = tv * h;
        // f32::clamp: NaN passes through.
        float cu = su < 0.0f ? 0.0f : (su > w - 1.0f ? w - 1.0f : su);
        float cv = sv < 0.0f ? 0.0f : (sv > h - 1.0f ? h - 1.0f : sv);
        u = as_u32(std::floor(cu));
        v = as_u32(std::floor(cv));
    } else {  // SamplerOnce tex.rs:313-357; out-of-range index clamped (the reference panics)
        u = as_u32(w * tu);
        v = as_u32(h * tv);
        if (u >= d->tw) u = d->tw - 1;
        if (v >= d->th) v = d->th - 1;
    }
    return d->tex[(uint64_t)v * d->tw + u];
}

// color.rs:253-263 Color3f::to_color4: (256 * c) as u8, alpha 0xFF.
inline uint32_t to_color4(float r, float g, float b) {
    return rgba_pack(as_u8(256.0f * r), as_u8(256.0f * g), as_u8(256.0f * b), 0xFF);
}

const float INV_GAMMA = 1.0f / 2.2f;  // color.rs:99-103

template <int NA, int S>
inline uint32_t shade(const rfo_draw *d, const Var<NA> &v) {
    if constexpr (S == RFO_FLAT) {
        return d->flat_rgba;
    } else if constexpr (S == RFO_GOURAUD) {
        return to_color4(v.a[0], v.a[1], v.a[2]);
    } else if constexpr (S == RFO_TEXTURED) {
        return sample(d, v.a[0], v.a[1]);
    } else if constexpr (S == RFO_TEX_GOURAUD) {
        // (texel.to_rgb().to_color3f() * col).to_color4(): color.rs:159-163,
        // channel-wise Mul color.rs:723-733.
        uint32_t t = sample(d, v.a[3], v.a[4]);
        float tr = (float)(t & 0xFF) / 256.0f;
        float tg = (float)((t >> 8) & 0xFF) / 256.0f;
        float tb = (float)((t >> 16) & 0xFF) / 256.0f;
        return to_color4(tr * v.a[0], tg * v.a[1], tb * v.a[2]);
    } else {  // GOURAUD_SRGB: Color3f<LinRgb>::to_srgb (color.rs:383-392)
        return to_color4(std::pow(v.a[0], INV_GAMMA), std::pow(v.a[1], INV_GAMMA),
                         std::pow(v.a[2], INV_GAMMA));
    }
}

template <int S>
constexpr uint32_t zdiv_mask() {
    // Which attributes divide by z (ZDiv): TexCoord does (vec.rs:666-677),
    // Color does not (color.rs:628).
    return S == RFO_TEXTURED ? 0x3u : (S == RFO_TEX_GOURAUD ? 0x18u : 0u);
}

}  // namespace

// pixfmt.rs:76-103: u32::from_be_bytes of the format's byte order.
// render/scene.rs BBox::of (:37-39, extend :42-46: f32::min / f32::max
// from the empty box), BBox::verts (:60-67) and BBox::visibility (:80-87):
// the corners through the vertex transform (mat.rs:952-973), ClipVert::new
// outcodes and view_frustum::status (clip.rs:245-267).  Returns 0 Visible,
// 1 Clipped, 2 Hidden.
extern "C" int32_t rfo_bbox_status(const float *verts, uint32_t nverts, uint32_t stride,
                                   const float mvp[16]) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < nverts; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::fmin(lo[k], verts[(uint64_t)i * stride + k]);
            hi[k] = std::fmax(hi[k], verts[(uint64_t)i * stride + k]);
        }
    uint8_t all = 0xFF, any = 0;
    for (int c = 0; c < 8; ++c) {
        const float hom[4] = {(c & 4) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 1) ? hi[2] : lo[2], 1.0f};
        float p[4];
        for (int k = 0; k < 4; ++k) p[k] = dot4(mvp + 4 * k, hom);
        const uint8_t oc = outcode(p);
        all &= oc;
        any |= oc;
    }
    return all != 0 ? 2 : (any == 0 ? 0 : 1);
}

extern "C" uint32_t rfo_pack(uint32_t c, int32_t fmt) {
    uint32_t r = c & 0xFF, g = (c >> 8) & 0xFF, b = (c >> 16) & 0xFF, a = c >> 24;
    switch (fmt) {
        case RFO_ARGB8888: return (a << 24) | (r << 16) | (g << 8) | b;
        case RFO_XRGB8888: return (r << 16) | (g << 8) | b;
        case RFO_RGBA8888: return (r << 24) | (g << 16) | (b << 8) | a;
        default: return (b << 24) | (g << 16) | (r << 8) | a;  // BGRA8888
    }
}

namespace {

// render.rs:134-207 for Tri<usize>, with Framebuf / Colorbuf targets
// (target.rs:163-198 rasterize_fb, target.rs:138-161 rasterize).
template <int NA, int S>
void render_t(const rfo_draw *d, const float vp[16], uint32_t *color, float *depth,
              uint32_t w, uint32_t h, int32_t fmt, const rfo_ctx *ctx, rfo_stats *st) {
    constexpr uint32_t ZM = zdiv_mask<S>();
    st->calls += 1;
    st->prims_i += d->ntri;
    st->verts_i += d->nverts;
    const uint32_t stride = d->pos_dim + d->nattr;

    // 1. Vertex shader + ClipVert::new (render.rs:157-165, mat.rs:952-973).
    ClipVert<NA> *cv = new ClipVert<NA>[d->nverts > 0 ? d->nverts : 1];
    for (uint32_t i = 0; i < d->nverts; ++i) {
        const float *src = d->verts + (uint64_t)i * stride;
        if (d->pos_dim == 4) {
            for (int k = 0; k < 4; ++k) cv[i].pos[k] = src[k];
        } else {
            const float hom[4] = {src[0], src[1], src[2], 1.0f};  // point.rs:247-252
            for (int k = 0; k < 4; ++k) cv[i].pos[k] = dot4(d->mvp + 4 * k, hom);
        }
        for (int k = 0; k < NA; ++k) cv[i].a[k] = src[d->pos_dim + k];
        cv[i].oc = outcode(cv[i].pos);
    }

    // 2-4. Primitive assembly, clipping, then per clipped tri: to_screen,
    // face culling, tri_fill.  Clipped output order = input order with each
    // clipped tri's fan in place (render.rs:167-205), optionally sorted by
    // depth first (render.rs:180-182).
    auto draw_clipped = [&](const ClipVert<NA> (&ct)[3]) {
        {
            // prim.rs:62-88 to_screen.
            Var<NA> sv[3];
            for (int k = 0; k < 3; ++k) {
                const ClipVert<NA> &v = ct[k];
                float wv = v.pos[3];
                const float ndc[4] = {v.pos[0] / wv, v.pos[1] / wv, 1.0f / wv, 1.0f};
                sv[k].p[0] = dot4(vp + 0, ndc);  // Mat4 apply, mat.rs:945-949
                sv[k].p[1] = dot4(vp + 4, ndc);
                sv[k].p[2] = dot4(vp + 8, ndc);
                for (int a = 0; a < NA; ++a)
                    sv[k].a[a] = ((ZM >> a) & 1) ? v.a[a] / wv : v.a[a];
            }
            // prim.rs:25-27 -> geom/prim.rs:152-156,288-294 winding.
            float ux = sv[1].p[0] - sv[0].p[0], uy = sv[1].p[1] - sv[0].p[1];
            float vx = sv[2].p[0] - sv[0].p[0], vy = sv[2].p[1] - sv[0].p[1];
            float z = 0.0f;
            z = z + (-uy) * vx;
            z = z + ux * vy;
            bool backface = z < 0.0f;
            // ctx.rs:95-101 face_cull.
            if ((ctx->face_cull == RFO_CULL_BACK && backface) ||
                (ctx->face_cull == RFO_CULL_FRONT && !backface))
                return;
            st->prims_o += 1;
            st->verts_o += 3;

            tri_fill<NA>(sv, [&](const Scanline<NA> &sl) {
                // The reference panics when a scanline leaves the buffer
                // (buf.rs slice indexing).  Here a row below the buffer only
                // counts in oob; a span past the right edge counts in oob,
                // keeps its frags.i and drops the pixels past the edge.
                if (sl.y >= h) {
                    st->oob += 1;
                    return;
                }
                uint64_t x0 = sl.x0;
                uint64_t x1 = sl.x1 > x0 ? sl.x1 : x0;
                st->frags_i += x1 - x0;
                if (x1 > w) st->oob += 1;
                uint64_t nfr = x1 - x0;
                if (sl.count < nfr) nfr = sl.count;  // zip() truncation
                Var<NA> v = sl.v0;
                uint64_t row = sl.y * (uint64_t)w;
                for (uint64_t k = 0; k < nfr; ++k) {
                    uint64_t x = x0 + k;
                    if (x >= w) break;
                    // raster.rs:60-69 fragments(): var.z_div(pos.z).
                    Var<NA> f = v;
                    for (int a = 0; a < NA; ++a)
                        if ((ZM >> a) & 1) f.a[a] = v.a[a] / v.p[2];
                    float new_z = v.p[2];
                    bool pass = true;
                    if (depth) {
                        float cur = depth[row + x];
                        // ctx.rs:86-89: curr.partial_cmp(&new) == depth_test.
                        switch (ctx->depth_test) {
                            case RFO_DEPTH_NONE: pass = true; break;
                            case RFO_DEPTH_LESS: pass = cur < new_z; break;
                            case RFO_DEPTH_EQUAL: pass = cur == new_z; break;
                            default: pass = cur > new_z; break;
                        }
                    }
                    if (pass) {
                        uint32_t col = shade<NA, S>(d, f);
                        if (ctx->color_write) {
                            st->frags_o += 1;
                            color[row + x] = rfo_pack(col, fmt);
                        }
                        if (depth && ctx->depth_write) depth[row + x] = new_z;
                    }
                    v = vstep(v, sl.dv_dx);  // Iter::next, vary.rs:146-154
                }
            }, [&] { st->oob += 1; });
        }
    };
    struct Clipped {
        ClipVert<NA> v[3];
    };
    std::vector<Clipped> sorted;
    ClipVert<NA> clipped[POLY_CAP][3];
    for (uint32_t t = 0; t < d->ntri; ++t) {
        ClipVert<NA> tri[3];
        for (int k = 0; k < 3; ++k) tri[k] = cv[d->idx[3 * t + k]];
        int nc = clip_tri<NA>(tri, clipped);
        for (int c = 0; c < nc; ++c) {
            if (ctx->depth_sort == RFO_SORT_NONE) {
                draw_clipped(clipped[c]);
            } else {
                Clipped e;
                for (int k = 0; k < 3; ++k) e.v[k] = clipped[c][k];
                sorted.push_back(e);
            }
        }
    }
    if (ctx->depth_sort != RFO_SORT_NONE) {
        // render.rs:209-219 depth_sort: key Render::depth = mean clip-space
        // z (prim.rs:21-23), ordered by f32::total_cmp, ascending for
        // FrontToBack and descending for BackToFront.  The reference's
        // sort_unstable_by leaves equal keys in an unspecified order; this
        // sort is stable (equal keys keep their submission and fan order).
        auto depth = [](const Clipped &e) {
            return (e.v[0].pos[2] + e.v[1].pos[2] + e.v[2].pos[2]) / 3.0f;
        };
        const bool back = ctx->depth_sort == RFO_SORT_BACK_TO_FRONT;
        std::stable_sort(sorted.begin(), sorted.end(), [&](const Clipped &a, const Clipped &b) {
            const int32_t ka = total_key(depth(a)), kb = total_key(depth(b));
            return back ? kb < ka : ka < kb;
        });
        for (const Clipped &e : sorted) draw_clipped(e.v);
    }
    delete[] cv;
}

}  // namespace

extern "C" void rfo_render(const rfo_draw *d, const float vp[16], uint32_t *color,
                           float *depth, uint32_t w, uint32_t h, int32_t fmt,
                           const rfo_ctx *ctx, rfo_stats *st) {
    switch (d->shader) {
        case RFO_FLAT: render_t<0, RFO_FLAT>(d, vp, color, depth, w, h, fmt, ctx, st); break;
        case RFO_GOURAUD: render_t<3, RFO_GOURAUD>(d, vp, color, depth, w, h, fmt, ctx, st); break;
        case RFO_TEXTURED: render_t<2, RFO_TEXTURED>(d, vp, color, depth, w, h, fmt, ctx, st); break;
        case RFO_TEX_GOURAUD:
            render_t<5, RFO_TEX_GOURAUD>(d, vp, color, depth, w, h, fmt, ctx, st);
            break;
        default: render_t<3, RFO_GOURAUD_SRGB>(d, vp, color, depth, w, h, fmt, ctx, st); break;
    }
}

// render.rs:134-207 for Edge<usize> (prim.rs:41-60): vertex shader,
// line clipping (clip.rs:311-348), to_screen (prim.rs:62-88),
// face_cull(is_backface = false: render.rs:92-94 default) and line()
// (raster.rs:115-173); every pixel is a one-pixel scanline into
// rasterize_fb (target.rs:163-198) carrying the first vertex's position and
// varyings.  idx holds nlines index pairs.
// Lines longer than this many pixels along their stepping axis (far past
// any target; the reference would index out of bounds) count once in oob.
constexpr uint64_t LINE_MAX_SPAN = 4194304u;

template <int NA, int S>
void render_lines_t(const rfo_draw *d, const uint32_t *idx, uint32_t nlines, const float vp[16],
                    uint32_t *color, float *depth, uint32_t w, uint32_t h, int32_t fmt,
                    const rfo_ctx *ctx, rfo_stats *st) {
    constexpr uint32_t ZM = zdiv_mask<S>();
    st->calls += 1;
    st->prims_i += nlines;
    st->verts_i += d->nverts;
    const uint32_t stride = d->pos_dim + d->nattr;
    ClipVert<NA> *cv = new ClipVert<NA>[d->nverts > 0 ? d->nverts : 1];
    for (uint32_t i = 0; i < d->nverts; ++i) {
        const float *src = d->verts + (uint64_t)i * stride;
        if (d->pos_dim == 4) {
            for (int k = 0; k < 4; ++k) cv[i].pos[k] = src[k];
        } else {
            const float hom[4] = {src[0], src[1], src[2], 1.0f};
            for (int k = 0; k < 4; ++k) cv[i].pos[k] = dot4(d->mvp + 4 * k, hom);
        }
        for (int k = 0; k < NA; ++k) cv[i].a[k] = src[d->pos_dim + k];
        cv[i].oc = outcode(cv[i].pos);
    }
    // One pixel of a line: the one-pixel scanline {y, x..x+1} with the
    // line's first-vertex varyings v (target.rs:163-198; a row below the
    // buffer counts in oob only, a pixel past the right edge keeps frags.i
    // and counts in oob, as for triangle spans).
    auto pixel = [&](uint64_t x, uint64_t y, const Var<NA> &v) {
        if (y >= h) {
            st->oob += 1;
            return;
        }
        st->frags_i += 1;
        if (x >= w) {
            st->oob += 1;
            return;
        }
        Var<NA> f = v;
        for (int a = 0; a < NA; ++a)
            if ((ZM >> a) & 1) f.a[a] = v.a[a] / v.p[2];
        const float new_z = v.p[2];
        const uint64_t i = y * (uint64_t)w + x;
        bool pass = true;
        if (depth) {
            const float cur = depth[i];
            switch (ctx->depth_test) {
                case RFO_DEPTH_NONE: pass = true; break;
                case RFO_DEPTH_LESS: pass = cur < new_z; break;
                case RFO_DEPTH_EQUAL: pass = cur == new_z; break;
                default: pass = cur > new_z; break;
            }
        }
        if (pass) {
            const uint32_t col = shade<NA, S>(d, f);
            if (ctx->color_write) {
                st->frags_o += 1;
                color[i] = rfo_pack(col, fmt);
            }
            if (depth && ctx->depth_write) depth[i] = new_z;
        }
    };
    for (uint32_t l = 0; l < nlines; ++l) {
        ClipVert<NA> a = cv[idx[2 * l]], b = cv[idx[2 * l + 1]];
        if (a.oc & b.oc) continue;  // both outside one plane
        if (a.oc | b.oc) {
            bool drop = false;
            for (int p = 0; p < 6 && !drop; ++p) {
                const bool a_in = (a.oc & (1u << p)) == 0, b_in = (b.oc & (1u << p)) == 0;
                if (!a_in && !b_in) {
                    drop = true;
                    break;
                }
                ClipVert<NA> v;
                if (intersect<NA>(p, a, b, v)) {
                    if (a_in) b = v;
                    else if (b_in) a = v;
                }
            }
            if (drop) continue;
        }
        Var<NA> sv[2];
        const ClipVert<NA> *e[2] = {&a, &b};
        for (int k = 0; k < 2; ++k) {
            const ClipVert<NA> &v = *e[k];
            const float wv = v.pos[3];
            const float ndc[4] = {v.pos[0] / wv, v.pos[1] / wv, 1.0f / wv, 1.0f};
            sv[k].p[0] = dot4(vp + 0, ndc);
            sv[k].p[1] = dot4(vp + 4, ndc);
            sv[k].p[2] = dot4(vp + 8, ndc);
            for (int q = 0; q < NA; ++q) sv[k].a[q] = ((ZM >> q) & 1) ? v.a[q] / wv : v.a[q];
        }
        if (ctx->face_cull == RFO_CULL_FRONT) continue;  // face_cull(false)
        st->prims_o += 1;
        st->verts_o += 3;
        // raster.rs:121-173 line().
        Var<NA> v0 = sv[0], v1 = sv[1];
        if (v0.p[1] > v1.p[1]) std::swap(v0, v1);
        const float dx = v1.p[0] - v0.p[0], dy = v1.p[1] - v0.p[1];
        if (std::fabs(dx) > dy) {
            if (dx < 0.0f) std::swap(v0, v1);  // dx, dy keep their values
            const float x0 = round_up_to_half(v0.p[0]), x1 = round_up_to_half(v1.p[0]);
            const float dy_dx = dy / dx;
            float y = v0.p[1] + dy_dx * (x0 - v0.p[0]);
            if (as_usize(x1) > as_usize(x0) && as_usize(x1) - as_usize(x0) > LINE_MAX_SPAN) {
                st->oob += 1;  // out of the supported range: counted, not drawn
                continue;
            }
            for (uint64_t x = as_usize(x0), xe = as_usize(x1); x < xe; ++x) {
                pixel(x, as_usize(y), v0);
                y = y + dy_dx;
            }
        } else {
            const float y0 = round_up_to_half(v0.p[1]), y1 = round_up_to_half(v1.p[1]);
            const float dx_dy = dx / dy;
            float x = v0.p[0] + dx_dy * (y0 - v0.p[1]);
            if (as_usize(y1) > as_usize(y0) && as_usize(y1) - as_usize(y0) > LINE_MAX_SPAN) {
                st->oob += 1;
                continue;
            }
            for (uint64_t y = as_usize(y0), ye = as_usize(y1); y < ye; ++y) {
                pixel(as_usize(x), y, v0);
                x = x + dx_dy;
            }
        }
    }
    delete[] cv;
}

extern "C" void rfo_render_lines(const rfo_draw *d, const uint32_t *idx, uint32_t nlines,
                                 const float vp[16], uint32_t *color, float *depth, uint32_t w,
                                 uint32_t h, int32_t fmt, const rfo_ctx *ctx, rfo_stats *st) {
    switch (d->shader) {
        case RFO_FLAT: render_lines_t<0, RFO_FLAT>(d, idx, nlines, vp, color, depth, w, h, fmt, ctx, st); break;
        case RFO_GOURAUD: render_lines_t<3, RFO_GOURAUD>(d, idx, nlines, vp, color, depth, w, h, fmt, ctx, st); break;
        case RFO_TEXTURED: render_lines_t<2, RFO_TEXTURED>(d, idx, nlines, vp, color, depth, w, h, fmt, ctx, st); break;
        case RFO_TEX_GOURAUD:
            render_lines_t<5, RFO_TEX_GOURAUD>(d, idx, nlines, vp, color, depth, w, h, fmt, ctx, st);
            break;
        default: render_lines_t<3, RFO_GOURAUD_SRGB>(d, idx, nlines, vp, color, depth, w, h, fmt, ctx, st); break;
    }
}

// front/src/lib.rs:103-120 Frame::clear.
extern "C" void rfo_clear(uint32_t *color, float *depth, uint32_t w, uint32_t h,
                          int32_t fmt, const uint32_t *clear_rgba, const float *depth_clear) {
    uint64_t n = (uint64_t)w * h;
    if (clear_rgba && color) {
        uint32_t px = rfo_pack(*clear_rgba, fmt);
        for (uint64_t i = 0; i < n; ++i) color[i] = px;
    }
    if (depth_clear && depth) {
        float z = 1.0f / *depth_clear;  // f32::recip
        for (uint64_t i = 0; i < n; ++i) depth[i] = z;
    }
}

extern "C" int32_t rfo_clip_batch(uint32_t n, const float *pos, const float *attr,
                                  uint32_t *counts, float *out_pos, float *out_attr) {
    int32_t ok = 1;
    ClipVert<1> out[POLY_CAP][3];
    for (uint32_t t = 0; t < n; ++t) {
        ClipVert<1> tri[3];
        for (int k = 0; k < 3; ++k) {
            for (int c = 0; c < 4; ++c) tri[k].pos[c] = pos[12 * t + 4 * k + c];
            tri[k].a[0] = attr ? attr[3 * t + k] : 0.0f;
            tri[k].oc = outcode(tri[k].pos);
        }
        int nc = clip_tri<1>(tri, out);
        counts[t] = (uint32_t)nc;
        for (int c = 0; c < nc; ++c)
            for (int k = 0; k < 3; ++k) {
                const ClipVert<1> &v = out[c][k];
                for (int q = 0; q < 3; ++q)
                    if (!(std::fabs(v.pos[q] / v.pos[3]) <= 1.00001f)) ok = 0;
                if (out_pos)
                    for (int q = 0; q < 4; ++q)
                        out_pos[(uint64_t)t * 84 + c * 12 + k * 4 + q] = v.pos[q];
                if (out_attr) out_attr[(uint64_t)t * 21 + c * 3 + k] = v.a[0];
            }
    }
    return ok;
}

namespace {
template <int NA>
uint32_t tri_fill_test(const float *screen, const float *attr, uint32_t zmask, uint64_t *rows,
                       uint32_t max_rows, float *frags, uint64_t max_frags, uint64_t *nfrags) {
    Var<NA> v[3]{};
    for (int k = 0; k < 3; ++k) {
        for (int c = 0; c < 3; ++c) v[k].p[c] = screen[3 * k + c];
        for (int a = 0; a < NA; ++a) v[k].a[a] = attr[NA * k + a];
    }
    uint32_t nr = 0;
    uint64_t nf = 0;
    tri_fill<NA>(v, [&](const Scanline<NA> &sl) {
        if (nr < max_rows) {
            rows[4 * nr + 0] = sl.y;
            rows[4 * nr + 1] = sl.x0;
            rows[4 * nr + 2] = sl.x1;
            rows[4 * nr + 3] = sl.count;
        }
        ++nr;
        Var<NA> q = sl.v0;
        for (uint32_t k = 0; k < sl.count; ++k) {
            if (nf < max_frags)
                for (int a = 0; a < NA; ++a)
                    frags[nf * NA + a] = ((zmask >> a) & 1) ? q.a[a] / q.p[2] : q.a[a];
            ++nf;
            q = vstep(q, sl.dv_dx);
        }
    }, [] {});
    *nfrags = nf;
    return nr;
}
}  // namespace

extern "C" uint32_t rfo_tri_fill(const float *screen, const float *attr, uint32_t nattr,
                                 uint32_t zmask, uint64_t *rows, uint32_t max_rows,
                                 float *frags, uint64_t max_frags, uint64_t *nfrags) {
    switch (nattr) {
        case 0: return tri_fill_test<0>(screen, attr, zmask, rows, max_rows, frags, max_frags, nfrags);
        case 1: return tri_fill_test<1>(screen, attr, zmask, rows, max_rows, frags, max_frags, nfrags);
        case 2: return tri_fill_test<2>(screen, attr, zmask, rows, max_rows, frags, max_frags, nfrags);
        case 3: return tri_fill_test<3>(screen, attr, zmask, rows, max_rows, frags, max_frags, nfrags);
        default: return tri_fill_test<5>(screen, attr, zmask, rows, max_rows, frags, max_frags, nfrags);
    }
}

extern "C" uint32_t rfo_sample(const uint32_t *tex, uint32_t tw, uint32_t th, int32_t sampler,
                               float u, float v) {
    rfo_draw d;
    std::memset(&d, 0, sizeof d);
    d.tex = tex;
    d.tw = tw;
    d.th = th;
    d.sampler = sampler;
    return sample(&d, u, v);
}
