// rf_exact.cuh — f32 arithmetic with the reference renderer's exact semantics,
// usable from host and device code.
//
// Every operation rounds once (IEEE-754 binary32, round to nearest even):
// device code goes through __fadd_rn/__fmul_rn/__fdiv_rn so that no a*b+c is
// contracted into an FMA, whatever the compiler flags.  Casts follow Rust's
// saturating `as` (NaN -> 0).
//
// rf_seq_add_n(s, d, k) returns the value reached by k sequential additions
// `s = s + d`, bit-identical to the loop, in a handful of integer operations:
// inside one binade every addition moves the bit pattern by the same
// integer, so k steps collapse into one multiply-add.  This is what lets the
// tile rasteriser start a scanline in the middle of a span, or a span in the
// middle of a triangle, and still reproduce the reference's running sums
// (core/src/math/vary.rs:142-155 Iter::next; core/src/render/raster.rs:80-114).
#ifndef RF_EXACT_CUH
#define RF_EXACT_CUH

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define RF_HD __host__ __device__ __forceinline__
#define RF_HD_COLD static __host__ __device__ __noinline__
#else
#define RF_HD inline
#define RF_HD_COLD static inline
#endif

namespace rfx {

RF_HD uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}
RF_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

// Single-rounding primitives (never contracted).
RF_HD float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}
RF_HD float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
RF_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}
RF_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    volatile float r = a / b;
    return r;
#endif
}
RF_HD float ffloor(float x) { return floorf(x); }

// Rust `f32 as usize` (64-bit), `as u32`, `as i32`, `as u8`: truncation
// toward zero, saturated to the type's range, NaN to 0.  On the device: one
// float-to-integer cvt with round-toward-zero.  For 8- and 32-bit results
// it is Rust's `as` by itself on sm_103a (measured: NaN, -NaN, -inf, -1 and
// -0.9 give 0; 255.9, 1e10 and +inf the type's maximum; the signed form
// gives INT32_MIN for -inf and 0 for NaN).  The 64-bit form is built from
// the 32-bit one and the float's bits instead (the 64-bit convert runs on
// the FP64 pipe, narrow on this part, and gives 2^63 for NaN): below 2^32
// -- NaN and negatives included -- the 32-bit convert; from 2^32 (an
// integer-valued float) its significand shifted into place; from 2^64
// (+inf too) the maximum.
RF_HD uint32_t as_u32(float x);
RF_HD uint64_t as_usize(float x) {
#if defined(__CUDA_ARCH__)
    if (!(x >= 4294967296.0f)) return as_u32(x);
    if (x >= 18446744073709551616.0f) return UINT64_MAX;
    const uint32_t b = __float_as_uint(x);  // biased exponent 159 .. 190
    return (uint64_t)((b & 0x7FFFFFu) | 0x800000u) << (((b >> 23) & 0xFFu) - 150u);
#else
    if (!(x > 0.0f)) return 0;
    if (x >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)x;
#endif
}
RF_HD uint32_t as_u32(float x) {
#if defined(__CUDA_ARCH__)
    uint32_t r;
    asm("cvt.rzi.u32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
#else
    if (!(x > 0.0f)) return 0;
    if (x >= 4294967296.0f) return UINT32_MAX;
    return (uint32_t)x;
#endif
}
RF_HD int32_t as_i32(float x) {
#if defined(__CUDA_ARCH__)
    int32_t r;
    asm("cvt.rzi.s32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
#else
    if (x != x) return 0;
    if (x <= -2147483648.0f) return INT32_MIN;
    if (x >= 2147483648.0f) return INT32_MAX;
    return (int32_t)x;
#endif
}
RF_HD uint32_t as_u8(float x) {
#if defined(__CUDA_ARCH__)
    uint32_t r;
    asm("cvt.rzi.u8.f32 %0, %1;" : "=r"(r) : "f"(x));  // zero-extended to 32 bits
    return r;
#else
    if (!(x > 0.0f)) return 0;
    if (x >= 255.0f) return 255;
    return (uint32_t)x;
#endif
}

// f32::total_cmp key (signed comparison of the returned value).
RF_HD int32_t total_key(float x) {
    int32_t i = (int32_t)f2u(x);
    return i ^ (int32_t)(((uint32_t)(i >> 31)) >> 1);
}

// raster.rs:304-307: floor(x + 0.5) + 0.5.
RF_HD float round_up_to_half(float x) { return fadd(ffloor(fadd(x, 0.5f)), 0.5f); }

// vec.rs:231-238: fold from 0.0 in index order.
RF_HD float dot4(const float *a, const float *b) {
    float acc = 0.0f;
    acc = fadd(acc, fmul(a[0], b[0]));
    acc = fadd(acc, fmul(a[1], b[1]));
    acc = fadd(acc, fmul(a[2], b[2]));
    acc = fadd(acc, fmul(a[3], b[3]));
    return acc;
}

// Lerp (math.rs:196-198): a + (b - a) * t.
RF_HD float lerp(float a, float b, float t) { return fadd(a, fmul(fsub(b, a), t)); }

// floor(a / b) for 0 <= a < 2^24, 1 <= b < 2^24, without an integer divide on
// the device: the float quotient is within a few units (relative error of
// the reciprocal and the product), then corrected exactly.
RF_HD uint32_t udiv24(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    uint32_t q = (uint32_t)__fmul_rz((float)a, __frcp_rn((float)b));
    while ((uint64_t)q * b > a) --q;
    while ((uint64_t)(q + 1) * b <= a) ++q;
    return q;
#else
    return a / b;
#endif
}

// ---------------------------------------------------------------------------
// rf_seq_add_n: k sequential additions s += d, exactly.
//
// Representation: for a finite s with biased exponent e (e <= 1 is the
// uniform grid 0..2^24 of step 2^-149 shared by subnormals and the first
// normal binade), let m be its integer significand; the magnitude bits are
// ((max(e,1) - 1) << 23) + m.  If every step of a run keeps the exact sum
// inside the same binade (m in [lo, 2^24-1], lo = 2^23+1 for e >= 2 and 1
// for e <= 1), each addition rounds the same way and adds the same integer
// `inc` to m, so k steps add k*inc.  Ties (d an odd half-multiple of the
// ulp) round to even: after one explicit step m is even and the increment is
// constant again.  Steps that touch a binade edge are taken explicitly with
// the hardware adder, so every boundary rounding is the IEEE one by
// construction.  A step that leaves s unchanged is a fixed point.
// ---------------------------------------------------------------------------
RF_HD_COLD float seq_add_n(float s, float d, uint32_t k) {
    while (k != 0) {
        const uint32_t sb = f2u(s), db = f2u(d);
        const uint32_t se = (sb >> 23) & 0xFFu, de = (db >> 23) & 0xFFu;
        if (se == 0xFFu || de == 0xFFu || (db & 0x7FFFFFFFu) == 0u || (sb & 0x7FFFFFFFu) == 0u) {
            // inf/NaN operand or d == +-0: one addition reaches a fixed point.
            // s == +-0: take the step explicitly (sign of zero rules).
            const float t = fadd(s, d);
            if ((sb & 0x7FFFFFFFu) == 0u && se != 0xFFu && de != 0xFFu && (db & 0x7FFFFFFFu) != 0u) {
                s = t;
                --k;
                continue;
            }
            return t;
        }
        const uint32_t ee = se > 1u ? se : 1u;             // effective exponent of s
        const uint32_t m = (sb & 0x7FFFFFu) | (se ? 0x800000u : 0u);
        const uint32_t md = (db & 0x7FFFFFu) | (de ? 0x800000u : 0u);
        const int32_t ed = de > 1u ? (int32_t)de : 1;
        const int32_t sh = (int32_t)ee - ed;               // d / ulp(s) = md * 2^-sh
        uint32_t q = 0, rem_up = 0, tie = 0;
        bool explicit_step = false;
        if (sh <= 0) {
            if (sh < -7) explicit_step = true;            // |d| >= 2^31 ulp: leaves the binade
            else q = md << (uint32_t)(-sh);
        } else if (sh < 25) {
            q = md >> (uint32_t)sh;
            const uint32_t rem = md & ((1u << (uint32_t)sh) - 1u);
            const uint32_t half = 1u << (uint32_t)(sh - 1);
            rem_up = rem > half;
            tie = rem == half;
        }  // sh >= 25: |d| < ulp/2, q = 0, no rounding up
        const bool grow = ((sb ^ db) >> 31) == 0u;        // |s| increases
        const uint32_t lo = se > 1u ? 0x800001u : 1u;
        const uint32_t hi = 0xFFFFFFu;
        uint32_t inc = 0;
        if (!explicit_step) {
            if (tie) {
                if (m & 1u) explicit_step = true;
                else inc = q + (q & 1u);
            } else {
                inc = q + rem_up;
            }
        }
        if (!explicit_step) {
            if (inc == 0u) {
                // |d| rounds away inside the binade: s is a fixed point,
                // except at the bottom edge where the exact sum can fall
                // into the finer binade below.
                if (grow || m >= lo) return s;
                explicit_step = true;
            }
        }
        if (!explicit_step) {
            const uint64_t total = (uint64_t)inc * (uint64_t)k;
            uint32_t n;
            if (grow) {
                if ((uint64_t)m + total <= hi) {
                    const uint32_t mag = ((ee - 1u) << 23) + m + (uint32_t)total;
                    return u2f((sb & 0x80000000u) | mag);
                }
                n = udiv24(hi - m, inc);
            } else {
                if ((uint64_t)m >= total + lo) {
                    const uint32_t mag = ((ee - 1u) << 23) + m - (uint32_t)total;
                    return u2f((sb & 0x80000000u) | mag);
                }
                n = m >= lo ? udiv24(m - lo, inc) : 0u;
            }
            if (n != 0u) {  // n < k: advance to the edge of the binade
                const uint32_t mm = grow ? m + n * inc : m - n * inc;
                s = u2f((sb & 0x80000000u) | (((ee - 1u) << 23) + mm));
                k -= n;
            }
        }
        // One explicit step across the edge (or for a tie from an odd m).
        const float t = fadd(s, d);
        --k;
        if (f2u(t) == f2u(s)) return s;
        s = t;
    }
    return s;
}

// ---------------------------------------------------------------------------
// The single-binade run, precomputed.  fast_params(s, d) returns dinc and
// kmax such that for every k <= kmax the k-step sum is the bit pattern of s
// plus k * dinc (two's complement on the whole pattern: the sign never
// changes inside a run).  kmax = 0 when no run applies (then only k = 0 is
// covered).  Used for per-row steps, whose start and step are fixed per
// half-triangle: a row anywhere in the triangle costs one multiply-add.
// ---------------------------------------------------------------------------
RF_HD void fast_params(float s, float d, int32_t &dinc, uint32_t &kmax) {
    dinc = 0;
    kmax = 0;
    const uint32_t sb = f2u(s), db = f2u(d);
    const uint32_t se = (sb >> 23) & 0xFFu, de = (db >> 23) & 0xFFu;
    if (se == 0xFFu || de == 0xFFu || (db & 0x7FFFFFFFu) == 0u || (sb & 0x7FFFFFFFu) == 0u) return;
    const uint32_t ee = se > 1u ? se : 1u;
    const uint32_t m = (sb & 0x7FFFFFu) | (se ? 0x800000u : 0u);
    const uint32_t md = (db & 0x7FFFFFu) | (de ? 0x800000u : 0u);
    const int32_t ed = de > 1u ? (int32_t)de : 1;
    const int32_t sh = (int32_t)ee - ed;
    uint32_t q = 0, rem_up = 0, tie = 0;
    if (sh <= 0) {
        if (sh < -7) return;
        q = md << (uint32_t)(-sh);
    } else if (sh < 25) {
        q = md >> (uint32_t)sh;
        const uint32_t rem = md & ((1u << (uint32_t)sh) - 1u);
        const uint32_t half = 1u << (uint32_t)(sh - 1);
        rem_up = rem > half;
        tie = rem == half;
    }
    const bool grow = ((sb ^ db) >> 31) == 0u;
    const uint32_t lo = se > 1u ? 0x800001u : 1u;
    const uint32_t hi = 0xFFFFFFu;
    uint32_t inc;
    if (tie) {
        if (m & 1u) return;
        inc = q + (q & 1u);
    } else {
        inc = q + rem_up;
    }
    if (inc == 0u) {
        if (grow || m >= lo) kmax = 0xFFFFFFFFu;  // fixed point
        return;
    }
    if (inc > hi) return;
    if (grow) {
        kmax = udiv24(hi - m, inc);
        dinc = (int32_t)inc;
    } else {
        kmax = m >= lo ? udiv24(m - lo, inc) : 0u;
        dinc = -(int32_t)inc;
    }
}

// k sequential additions with the single-binade run tried inline first and
// the general loop out of line (it is rarely needed).
//
// run_try: one run of k steps from s inside its binade; on success returns
// true with the result in out.  Otherwise returns false with n = the steps
// that do stay inside the binade (n < k; 0 when none or when s is not a
// normal number above the first binade, d not normal, or a tie).
RF_HD bool run_try(float s, float d, uint32_t k, float &out, uint32_t &n) {
    n = 0;
    const uint32_t sb = f2u(s), db = f2u(d);
    const uint32_t se = (sb >> 23) & 0xFFu, de = (db >> 23) & 0xFFu;
    if (!(se - 2u < 253u && de - 1u < 254u)) return false;
    const uint32_t m = (sb & 0x7FFFFFu) | 0x800000u;
    const uint32_t md = (db & 0x7FFFFFu) | 0x800000u;
    const int32_t sh = (int32_t)se - (int32_t)de;
    if (sh < -7) return false;
    uint32_t inc = 0;
    if (sh <= 0) {
        inc = md << (uint32_t)(-sh);
    } else if (sh < 25) {
        const uint32_t q = md >> (uint32_t)sh;
        const uint32_t rem = md & ((1u << (uint32_t)sh) - 1u);
        const uint32_t half = 1u << (uint32_t)(sh - 1);
        if (rem == half) return false;  // ties take the general path
        inc = q + (rem > half ? 1u : 0u);
    }
    if (inc == 0u) return false;
    const uint64_t total = (uint64_t)inc * (uint64_t)k;
    if (((sb ^ db) >> 31) == 0u) {
        if ((uint64_t)m + total <= 0xFFFFFFull) {
            out = u2f(sb + (uint32_t)total);
            return true;
        }
        n = udiv24(0xFFFFFFu - m, inc);
    } else {
        if ((uint64_t)m >= total + 0x800001ull) {
            out = u2f(sb - (uint32_t)total);
            return true;
        }
        n = m >= 0x800001u ? udiv24(m - 0x800001u, inc) : 0u;
    }
    out = u2f(((sb ^ db) >> 31) == 0u ? sb + n * inc : sb - n * inc);
    return false;
}

// Inline: one run, or one run to the binade edge, the explicit edge step
// and a second run; anything else goes to the general loop.
RF_HD float jump(float s, float d, uint32_t k) {
    if (k == 0u) return s;
    float r;
    uint32_t n;
    if (run_try(s, d, k, r, n)) return r;
    if (n == 0u) return seq_add_n(s, d, k);
    const float t = fadd(r, d);  // the step across the edge
    const uint32_t k2 = k - n - 1u;
    if (k2 == 0u) return t;
    uint32_t n2;
    if (run_try(t, d, k2, r, n2)) return r;
    return seq_add_n(t, d, k2);
}

}  // namespace rfx

#endif
