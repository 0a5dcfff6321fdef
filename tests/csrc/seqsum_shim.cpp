// Host build of the product's exact-arithmetic header, for CPU tests of
// rfx::seq_add_n against plain sequential loops.
#include "../../retrofire_gb300/csrc/rf_exact.cuh"

extern "C" float shim_seq_add_n(float s, float d, uint32_t k) { return rfx::seq_add_n(s, d, k); }

extern "C" float shim_seq_loop(float s, float d, uint32_t k) {
    for (uint32_t i = 0; i < k; ++i) s = rfx::fadd(s, d);
    return s;
}

// Counts mismatches over n cases (arrays of s, d, k).
extern "C" uint64_t shim_check(const float *s, const float *d, const uint32_t *k, uint64_t n,
                               uint64_t *first_bad) {
    uint64_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float a = shim_seq_loop(s[i], d[i], k[i]);
        const float b = rfx::seq_add_n(s[i], d[i], k[i]);
        const bool both_nan = a != a && b != b;
        if (rfx::f2u(a) != rfx::f2u(b) && !both_nan) {
            if (!bad) *first_bad = i;
            ++bad;
        }
    }
    return bad;
}

// The precomputed single-binade run and the inline-first jump, checked the
// same way: every k <= kmax must match the loop, and jump() must equal it.
extern "C" uint64_t shim_check_fast(const float *s, const float *d, const uint32_t *k, uint64_t n,
                                    uint64_t *first_bad) {
    uint64_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float a = shim_seq_loop(s[i], d[i], k[i]);
        const float b = rfx::jump(s[i], d[i], k[i]);
        int32_t dinc;
        uint32_t kmax;
        rfx::fast_params(s[i], d[i], dinc, kmax);
        bool okf = true;
        if (k[i] <= kmax) {
            const float c = rfx::u2f(rfx::f2u(s[i]) + k[i] * (uint32_t)dinc);
            okf = rfx::f2u(a) == rfx::f2u(c) || (a != a && c != c);
        }
        const bool okj = rfx::f2u(a) == rfx::f2u(b) || (a != a && b != b);
        if (!okf || !okj) {
            if (!bad) *first_bad = i;
            ++bad;
        }
    }
    return bad;
}
