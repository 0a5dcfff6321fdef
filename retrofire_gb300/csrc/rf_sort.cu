// rf_sort.cu — Context::depth_sort (core/src/render.rs:180-182, 209-219):
// the clipped triangles of each render() call ordered by Render::depth, the
// mean of their three clip-space z (prim.rs:21-23), under f32::total_cmp,
// before setup.  A stable LSD radix sort of (draw, depth key) pairs over
// the frame's clipped triangles; draws whose job does not sort get key 0
// and keep their order.  The reference's sort_unstable_by leaves equal
// keys in an unspecified order; this sort keeps them in clipped order.
#include <cuda_runtime.h>

#include "rf_device.cuh"

namespace {
using namespace rfx;

constexpr uint32_t RS_THREADS = 256;
constexpr uint32_t RS_CHUNKS = 8;                       // 256-item chunks per block
constexpr uint32_t RS_TILE = RS_THREADS * RS_CHUNKS;     // items per block
constexpr uint32_t RS_DIGITS = 256;                      // 8-bit digits

// f32::total_cmp as an unsigned key: -NaN < -inf < ... < -0 < +0 < ... < inf < NaN.
__device__ __forceinline__ uint32_t total_order_u32(float x) {
    const uint32_t b = f2u(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// One thread per input triangle: the key of each of its clipped triangles.
__global__ void k_dsort_keys(const DrawDev *__restrict__ draws, uint32_t nd, const JobDev *__restrict__ jobs,
                             uint32_t nt, const float4 *__restrict__ cpos, const uint32_t *__restrict__ tcnt,
                             const uint32_t *__restrict__ toff, const uint32_t *__restrict__ tpoly,
                             const PolyVert *__restrict__ pool, unsigned long long *__restrict__ keys,
                             uint32_t *__restrict__ vals, uint32_t *__restrict__ ptri) {
    for (uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x; gt < nt; gt += gridDim.x * blockDim.x) {
        const uint32_t cnt = tcnt[gt];
        if (!cnt) continue;
        const uint32_t di = rfd::upper_index(nd, gt, [&](uint32_t i) { return draws[i].tri_base; });
        const DrawDev &d = draws[di];
        const int32_t mode = jobs[d.job].depth_sort;
        const uint32_t slot = tpoly[gt], p0 = toff[gt];
        for (uint32_t c = 0; c < cnt; ++c) {
            float z[3];
            for (int k = 0; k < 3; ++k) {
                if (slot == RF_NO_POLY) {
                    z[k] = cpos[d.vert_base + d.idx[3 * (size_t)(gt - d.tri_base) + k]].z;
                } else {
                    z[k] = pool[(size_t)slot * RF_POLY_STORE + (k == 0 ? 0u : c + (uint32_t)k)].pos[2];
                }
            }
            // (a.pos.z() + b.pos.z() + c.pos.z()) / 3.0
            const float depth = fdiv(fadd(fadd(z[0], z[1]), z[2]), 3.0f);
            const uint32_t tk = total_order_u32(depth);
            const uint32_t lo = mode == 0 ? 0u : (mode == 1 ? tk : ~tk);
            keys[p0 + c] = ((unsigned long long)di << 32) | lo;
            vals[p0 + c] = p0 + c;
            ptri[p0 + c] = gt;
        }
    }
}

__device__ __forceinline__ uint32_t digit_of(unsigned long long k, uint32_t shift) {
    return (uint32_t)(k >> shift) & (RS_DIGITS - 1u);
}

// Per block, how many of its items have each digit: hist[digit * nb + block].
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned long long *__restrict__ keys, uint32_t n,
                                                        uint32_t shift, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[RS_DIGITS];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RS_TILE;
    for (uint32_t i = threadIdx.x; i < RS_TILE; i += RS_THREADS)
        if (base + i < n) atomicAdd(&h[digit_of(keys[base + i], shift)], 1u);
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: items of the block in order, chunk by chunk; an item's
// place = its digit's offset for this block (offs, the exclusive scan of
// hist) + the items of that digit before it in the block.
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned long long *__restrict__ kin,
                                                           const uint32_t *__restrict__ vin, uint32_t n,
                                                           uint32_t shift, const uint32_t *__restrict__ offs,
                                                           unsigned long long *__restrict__ kout,
                                                           uint32_t *__restrict__ vout) {
    constexpr uint32_t NW = RS_THREADS / 32;
    __shared__ uint32_t run[RS_DIGITS];       // next place of each digit
    __shared__ uint32_t wcnt[NW][RS_DIGITS];  // per warp: its items of each digit in this chunk
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    run[threadIdx.x] = offs[threadIdx.x * gridDim.x + blockIdx.x];
    const uint32_t base = blockIdx.x * RS_TILE;
    for (uint32_t ch = 0; ch < RS_CHUNKS; ++ch) {
        const uint32_t i = base + ch * RS_THREADS + threadIdx.x;
        for (uint32_t k = 0; k < NW; ++k) wcnt[k][threadIdx.x] = 0;
        __syncthreads();
        const bool have = i < n;
        const unsigned long long key = have ? kin[i] : 0ull;
        const uint32_t dg = have ? digit_of(key, shift) : RS_DIGITS;  // RS_DIGITS: no item
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dg);
        const uint32_t below = __popc(peers & ((1u << lane) - 1u));
        if (have && below == 0) wcnt[w][dg] = __popc(peers);
        __syncthreads();
        // Thread t: digit t's count in the warps before each warp (in place).
        uint32_t acc = 0;
        for (uint32_t k = 0; k < NW; ++k) {
            const uint32_t c = wcnt[k][threadIdx.x];
            wcnt[k][threadIdx.x] = acc;
            acc += c;
        }
        __syncthreads();
        if (have) {
            const uint32_t dst = run[dg] + wcnt[w][dg] + below;
            kout[dst] = key;
            vout[dst] = vin[i];
        }
        __syncthreads();
        run[threadIdx.x] += acc;
        __syncthreads();
    }
}

__global__ void k_draw_counts(const DrawDev *__restrict__ draws, uint32_t nd, uint32_t nt,
                              const uint32_t *__restrict__ toff, const uint32_t *__restrict__ counters,
                              uint32_t *__restrict__ nout) {
    const uint32_t total = counters[RF_CNT_PRIMS];
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        const uint32_t t0 = draws[d].tri_base, t1 = t0 + draws[d].ntri;
        if (t1 == t0) {
            nout[d] = 0;
            continue;
        }
        const uint32_t e = t1 < nt ? toff[t1] : total;
        nout[d] = e - toff[t0];
    }
}

__global__ void k_iota(uint32_t *__restrict__ toff, uint32_t *__restrict__ tcnt, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        toff[i] = i;
        tcnt[i] = 1u;
    }
}

struct SortScratch {
    unsigned long long *k0, *k1;
    uint32_t *v1, *hist, *total;  // hist: counts, then their exclusive scan
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

SortScratch carve(void *p, uint32_t np) {
    char *b = static_cast<char *>(p);
    const uint32_t nb = (np + RS_TILE - 1) / RS_TILE;
    SortScratch s;
    s.k0 = reinterpret_cast<unsigned long long *>(b);
    b += align256((size_t)np * 8);
    s.k1 = reinterpret_cast<unsigned long long *>(b);
    b += align256((size_t)np * 8);
    s.v1 = reinterpret_cast<uint32_t *>(b);
    b += align256((size_t)np * 4);
    s.hist = reinterpret_cast<uint32_t *>(b);
    b += align256((size_t)nb * RS_DIGITS * 4 * 2);
    s.total = reinterpret_cast<uint32_t *>(b);
    return s;
}

}  // namespace

namespace rfk {

uint32_t dsort_scan_items(uint32_t np) { return (np + RS_TILE - 1) / RS_TILE * RS_DIGITS; }

size_t dsort_scratch_bytes(uint32_t np) {
    const size_t nb = (np + RS_TILE - 1) / RS_TILE;
    return align256((size_t)np * 8) * 2 + align256((size_t)np * 4) + align256(nb * RS_DIGITS * 4 * 2) + 256;
}

cudaError_t launch_draw_counts(const DrawDev *draws, uint32_t nd, uint32_t nt, const uint32_t *toff,
                               const uint32_t *counters, uint32_t *nout, cudaStream_t s) {
    if (nd == 0) return cudaSuccess;
    k_draw_counts<<<(nd + 255) / 256, 256, 0, s>>>(draws, nd, nt, toff, counters, nout);
    return cudaGetLastError();
}

cudaError_t launch_dsort(const DrawDev *draws, uint32_t nd, const JobDev *jobs, uint32_t nt,
                         uint32_t np, const float4 *cpos, const uint32_t *tcnt, const uint32_t *toff,
                         const uint32_t *tpoly, const PolyVert *pool, const uint32_t *counters,
                         uint32_t *perm, uint32_t *ptri, void *scratch, uint32_t *scan_scratch,
                         cudaStream_t s) {
    cudaError_t e;
    if (np == 0) return cudaSuccess;
    SortScratch S = carve(scratch, np);
    const uint32_t kb = min((nt + 255) / 256, 4096u);
    k_dsort_keys<<<kb, 256, 0, s>>>(draws, nd, jobs, nt, cpos, tcnt, toff, tpoly, pool, S.k0, perm, ptri);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // Digits to sort: the 32 key bits, then the draw index's bits.
    uint32_t dbits = 0;
    while (dbits < 32 && (nd - 1u) >> dbits) dbits += 8;
    const uint32_t passes = 4 + dbits / 8;
    const uint32_t nb = (np + RS_TILE - 1) / RS_TILE;
    unsigned long long *kin = S.k0, *kout = S.k1;
    uint32_t *vin = perm, *vout = S.v1;
    uint32_t *offs = S.hist + (size_t)nb * RS_DIGITS;
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t shift = 8 * p;
        k_rs_hist<<<nb, RS_THREADS, 0, s>>>(kin, np, shift, S.hist);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = launch_scan(S.hist, offs, nb * RS_DIGITS, scan_scratch, S.total, s)) != cudaSuccess) return e;
        k_rs_scatter<<<nb, RS_THREADS, 0, s>>>(kin, vin, np, shift, offs, kout, vout);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        unsigned long long *tk = kin;
        kin = kout;
        kout = tk;
        uint32_t *tv = vin;
        vin = vout;
        vout = tv;
    }
    if (vin != perm) return cudaMemcpyAsync(perm, vin, (size_t)np * 4, cudaMemcpyDeviceToDevice, s);
    return cudaSuccess;
}

cudaError_t launch_iota(uint32_t *toff, uint32_t *tcnt, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_iota<<<min((n + 255) / 256, 4096u), 256, 0, s>>>(toff, tcnt, n);
    return cudaGetLastError();
}

}  // namespace rfk
