// Device-wide primitives of the schedule builder and the RePair compressor:
// scans of uint32 (exclusive sum, inclusive maximum) and a stable
// least-significant-digit radix sort of 64-bit keys that optionally carry a
// 32-bit value.
//
// Scan: reduce-then-scan in three launches per level of recursion (tile sums,
// scan of the tile sums, scan of each tile from its offset).
// Radix sort: 8-bit digits.  Per pass, each CTA histograms a tile of 2048
// keys, the digit-major table of tile counts is scanned, and each CTA scatters
// its tile in 8 rounds of 256 keys; within a round, lanes holding the same
// digit find each other with __match_any_sync and per-warp counts are scanned
// in shared memory, so keys keep their input order within a digit (stable).
#pragma once

#include <algorithm>
#include <cstdint>

#include "device_util.cuh"

namespace gmr {
namespace dev {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

inline int64_t tiles(int64_t n) { return (n + kTile - 1) / kTile; }
inline int grid_for(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + kThreads - 1) / kThreads, 1), 152 * 32); }

struct SumOp {
    static constexpr uint32_t identity = 0;
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
};
struct MaxOp {
    static constexpr uint32_t identity = 0;
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a > b ? a : b; }
};

// Block-wide exclusive scan of one value per thread (blockDim.x == kThreads);
// *total = the block's reduction.
template <class Op>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kThreads / 32];
    const Op op;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;  // inclusive within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = op(y, x);
    }
    uint32_t ex = __shfl_up_sync(0xffffffffu, x, 1);  // exclusive within the warp
    if (lane == 0) ex = Op::identity;
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? warp_sums[lane] : Op::identity;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w = op(y, w);
        }
        if (lane < kThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const uint32_t base = warp ? warp_sums[warp - 1] : Op::identity;
    *total = warp_sums[kThreads / 32 - 1];
    __syncthreads();
    return op(base, ex);
}

template <class Op>
__global__ void __launch_bounds__(kThreads) k_scan_reduce(const uint32_t* __restrict__ in, int64_t n,
                                                          uint32_t* __restrict__ sums) {
    const Op op;
    const int64_t base = (int64_t)blockIdx.x * kTile;
    uint32_t s = Op::identity;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const int64_t i = base + j * kThreads + threadIdx.x;
        if (i < n) s = op(s, in[i]);
    }
    uint32_t total;
    block_exclusive_scan<Op>(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive (or inclusive) scan of each tile from its offset offs[tile];
// out[n] = the whole reduction (exclusive scans only).  in and out may be the
// same array.
template <class Op, bool INCLUSIVE>
__global__ void __launch_bounds__(kThreads) k_scan_down(const uint32_t* in, uint32_t* out, int64_t n,
                                                        const uint32_t* __restrict__ offs) {
    const Op op;
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    uint32_t v[kItems], s = Op::identity;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        v[j] = base + j < n ? in[base + j] : Op::identity;
        s = op(s, v[j]);
    }
    uint32_t total;
    const uint32_t off = offs ? offs[blockIdx.x] : Op::identity;
    uint32_t run = op(off, block_exclusive_scan<Op>(s, &total));
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        if (INCLUSIVE) run = op(run, v[j]);
        if (base + j < n) out[base + j] = run;
        if (!INCLUSIVE) run = op(run, v[j]);
    }
    if (!INCLUSIVE && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = op(off, total);
}

// uint32 words of scratch a scan of n items needs.
inline int64_t scan_scratch(int64_t n) {
    int64_t s = 0;
    for (int64_t m = tiles(n); m > 1; m = tiles(m)) s += m + 1;
    return s + 1;
}

template <class Op, bool INCLUSIVE>
inline void scan(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st) {
    if (n <= 0) {
        if (!INCLUSIVE) GMR_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), st));
        return;
    }
    const int64_t nb = tiles(n);
    if (nb == 1) {
        k_scan_down<Op, INCLUSIVE><<<1, kThreads, 0, st>>>(in, out, n, nullptr);
    } else {
        k_scan_reduce<Op><<<(unsigned)nb, kThreads, 0, st>>>(in, n, tmp);
        scan<Op, false>(tmp, tmp, nb, tmp + nb + 1, st);
        k_scan_down<Op, INCLUSIVE><<<(unsigned)nb, kThreads, 0, st>>>(in, out, n, tmp);
    }
    GMR_CUDA(cudaGetLastError());
}

// Exclusive sum of in[0, n) into out[0, n], out[n] = total; out may alias in
// and must hold n + 1 words.  tmp holds scan_scratch(n) words.
inline void exclusive_scan(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st) {
    scan<SumOp, false>(in, out, n, tmp, st);
}

// Inclusive running maximum of in[0, n) into out[0, n) (out may alias in).
inline void inclusive_max_scan(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st) {
    scan<MaxOp, true>(in, out, n, tmp, st);
}

static __global__ void __launch_bounds__(kThreads) k_radix_hist(const uint64_t* __restrict__ keys, int64_t n, int shift,
                                                         int64_t nblk, uint32_t* __restrict__ counts) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const int64_t i = base + j * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(int64_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

template <bool VALS>
__global__ void __launch_bounds__(kThreads) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                            int64_t n, int shift, int64_t nblk,
                                                            const uint32_t* __restrict__ offs) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wc[kThreads / 32][256];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    run[t] = offs[(int64_t)t * nblk + blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * kTile;
    for (int j = 0; j < kItems; ++j) {
        const int64_t i = base + j * kThreads + t;
        const bool ok = i < n;
        const uint64_t k = ok ? kin[i] : 0;
        const uint32_t v = VALS && ok ? vin[i] : 0;
        const int d = ok ? (int)((k >> shift) & 255u) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
#pragma unroll
        for (int q = 0; q < kThreads / 32; ++q) wc[q][t] = 0;
        __syncthreads();
        if (ok && rank == 0) wc[w][d] = (uint32_t)__popc(peers);
        __syncthreads();
        uint32_t acc = 0;  // thread t owns digit t
#pragma unroll
        for (int q = 0; q < kThreads / 32; ++q) {
            const uint32_t c = wc[q][t];
            wc[q][t] = acc;
            acc += c;
        }
        __syncthreads();
        if (ok) {
            const uint32_t pos = run[d] + wc[w][d] + (uint32_t)rank;
            kout[pos] = k;
            if (VALS) vout[pos] = v;
        }
        __syncthreads();
        run[t] += acc;
    }
}

// Scratch (uint32 words) radix_sort needs for n items.
inline int64_t sort_scratch(int64_t n) {
    const int64_t m = 256 * tiles(n);
    return m + 1 + scan_scratch(m);
}

// Stable sort of n keys by their bits [0, bits), values (if any) alongside.
// Ping-pongs between (k, v) and (k2, v2); on return k and v point at the
// sorted data.  tmp holds sort_scratch(n) words.
inline void radix_sort(uint64_t*& k, uint64_t*& k2, uint32_t*& v, uint32_t*& v2, int64_t n, int bits, uint32_t* tmp,
                       cudaStream_t st) {
    if (n <= 1 || bits <= 0) return;
    const int64_t nblk = tiles(n), m = 256 * nblk;
    if (n >= (int64_t)UINT32_MAX) throw Error(GMR_ERR_RANGE, "radix sort: too many keys");
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<(unsigned)nblk, kThreads, 0, st>>>(k, n, shift, nblk, tmp);
        exclusive_scan(tmp, tmp, m, tmp + m + 1, st);
        if (v)
            k_radix_scatter<true><<<(unsigned)nblk, kThreads, 0, st>>>(k, v, k2, v2, n, shift, nblk, tmp);
        else
            k_radix_scatter<false><<<(unsigned)nblk, kThreads, 0, st>>>(k, nullptr, k2, nullptr, n, shift, nblk, tmp);
        GMR_CUDA(cudaGetLastError());
        std::swap(k, k2);
        if (v) std::swap(v, v2);
    }
}

}  // namespace dev
}  // namespace gmr
