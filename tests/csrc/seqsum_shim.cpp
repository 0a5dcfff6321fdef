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
