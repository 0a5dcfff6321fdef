// rf_device.cuh — device helpers shared by the kernel translation units.
#ifndef RF_DEVICE_CUH
#define RF_DEVICE_CUH

#include <cuda_runtime.h>

#include "rf_exact.cuh"
#include "rf_internal.cuh"
#include "rf_kernels.cuh"

namespace rfd {
using namespace rfx;

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

// upper_index for the 32 lanes of a warp whose x do not decrease with the
// lane (all lanes call): one binary search for lane 0's x, then each lane
// steps forward over the few records between (same result per lane).
template <class F>
__device__ __forceinline__ uint32_t warp_upper_index(uint32_t n, uint32_t x, F key) {
    const uint32_t x0 = __shfl_sync(0xFFFFFFFFu, x, 0);
    uint32_t d = 0;
    if ((threadIdx.x & 31) == 0) d = upper_index(n, x0, key);
    d = __shfl_sync(0xFFFFFFFFu, d, 0);
    while (d + 1 < n && key(d + 1) <= x) ++d;
    return d;
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

// Row quantity r of half H after j scanlines (see HalfRuns): one of the two
// precomputed single-binade runs U, else the general loop from the second.
__device__ __forceinline__ float row_value(const HalfRec *__restrict__ H, const HalfRuns *__restrict__ U,
                                           int r, uint32_t j) {
    const uint32_t e0 = U->e0[r];
    if (j <= e0) return u2f(H->b0[r] + j * (uint32_t)U->i0[r]);
    const uint32_t j1 = j - e0 - 1u;
    if (j <= U->e1[r]) return u2f(U->b1[r] + j1 * (uint32_t)U->i1[r]);
    return seq_add_n(u2f(U->b1[r]), H->d[r], j1);
}

}  // namespace rfd

#endif
