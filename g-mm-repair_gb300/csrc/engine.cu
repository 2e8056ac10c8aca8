// GB300 (sm_103a) sweep engine: right multiplication Y = M X over a
// grammar-compressed M, level by level, with emit-on-the-spot.
//
// Method (the reference's, gpu-engine/gpu_engine.cu:85-133): terminals expand
// to leaf(V[val], X[col]) (init_T_terminals, :64-83), every rule of level k
// is oplus(apply(cv(left), coeff), cv(right)) of values computed below it
// (eval_level_layered, :85-102), and every occurrence of a symbol in a row's
// top-level sequence is folded into that row of Y at the symbol's own level
// (emit_level / emit_terminals, :104-133).
//
// Layout and execution (new):
//   * values of one multiply live in an arena [slot][Bw] (Bw = B words per
//     slot, right-hand sides innermost), slots level-major and child-sorted by
//     the plan builder; identity pass-throughs are references, not copies;
//   * a thread group of G = Bw / VEC lanes handles one rule or emission and
//     moves VEC consecutive words per lane with 8- or 16-byte accesses;
//   * one launch per level k evaluates the rules of level k AND folds the
//     emissions of level k-1 (complete since the previous launch), so a
//     multiply is D + 2 launches instead of the reference's 2D + 4;
//   * emissions are sorted by (row, source): a warp reduces each row segment
//     in registers (shuffles for (+,x), __reduce_or/min_sync for the
//     idempotent semirings) and issues one atomic per segment;
//   * the launch chain can be captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "gmr_internal.h"
#include "async_copy.cuh"
#include "device_util.cuh"

namespace gmr {

// ------------------------------------------------------------------ semirings
struct SPlus {
    using T = float;
    static __device__ __forceinline__ T zero() { return 0.0f; }
    static __device__ __forceinline__ T oplus(T a, T b) { return a + b; }
    static __device__ __forceinline__ T apply(T v, float c) { return c * v; }
    // leaf(V, x) = V * x  (gpu_engine.h:50)
    static __device__ __forceinline__ T leaf(float v, T x) { return v * x; }
    static __device__ __forceinline__ void red(T* p, T v) { atomicAdd(p, v); }
};
struct SBool {  // 32 right-hand sides per word
    using T = uint32_t;
    static __device__ __forceinline__ T zero() { return 0u; }
    static __device__ __forceinline__ T oplus(T a, T b) { return a | b; }
    static __device__ __forceinline__ T apply(T v, float) { return v; }
    // leaf = (V != 0 && x != 0) per bit  (gpu_engine.h:63)
    static __device__ __forceinline__ T leaf(float v, T x) { return v != 0.0f ? x : 0u; }
    static __device__ __forceinline__ void red(T* p, T v) { atomicOr(p, v); }
};
struct STrop {  // (min, +) on int32, 1e9 = +inf
    using T = int32_t;
    static __device__ __forceinline__ T zero() { return GMR_TROPICAL_INF; }
    static __device__ __forceinline__ T oplus(T a, T b) { return a < b ? a : b; }
    static __device__ __forceinline__ T apply(T v, float) { return v; }
    // leaf = (int)V + x unless either is >= 1e9  (gpu_engine.h:79-86)
    static __device__ __forceinline__ T leaf(float v, T x) {
        int iv = __float2int_rz(v);
        if (iv >= GMR_TROPICAL_INF || x >= GMR_TROPICAL_INF) return GMR_TROPICAL_INF;
        return iv + x;
    }
    static __device__ __forceinline__ void red(T* p, T v) { atomicMin(p, v); }
};

// ------------------------------------------------------------------ vectors
template <class T, int N>
struct alignas(sizeof(T) * N) Vec {
    T v[N];
};

// 32-byte accesses (8 words per lane): one 256-bit load or store per lane.
// Volatile asm keeps each access where the program places it (in particular
// on its side of a grid barrier in the persistent sweep).
#define GMR_V8_OUT(u) "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7])
template <int MODE>  // 0 read-only path (.nc), 1 plain, 2 L2 only (.cg)
__device__ __forceinline__ void ld_v8(const void* p, uint32_t (&u)[8]) {
    if constexpr (MODE == 0)
        asm volatile("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];" : GMR_V8_OUT(u) : "l"(p));
    else if constexpr (MODE == 1)
        asm volatile("ld.global.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];" : GMR_V8_OUT(u) : "l"(p) : "memory");
    else
        asm volatile("ld.global.cg.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];" : GMR_V8_OUT(u) : "l"(p) : "memory");
}
#undef GMR_V8_OUT
__device__ __forceinline__ void st_v8(void* p, const uint32_t (&u)[8]) {
    asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "r"(u[0]), "r"(u[1]), "r"(u[2]),
                 "r"(u[3]), "r"(u[4]), "r"(u[5]), "r"(u[6]), "r"(u[7])
                 : "memory");
}

template <class T, int N>
__device__ __forceinline__ Vec<T, N> vload(const T* p) {
    Vec<T, N> r;
    if constexpr (N == 8) {
        uint32_t u[8];
        ld_v8<0>(p, u);
        memcpy(&r, u, 32);
    } else if constexpr (N == 4) {
        uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
        memcpy(&r, &u, 16);
    } else if constexpr (N == 2) {
        uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
        memcpy(&r, &u, 8);
    } else {
        r.v[0] = __ldg(p);
    }
    return r;
}
// Loads of values written earlier in the same multiply (no read-only path).
// CG = true loads through L2 only (ld.global.cg): needed inside one launch
// that reads what other SMs wrote in an earlier phase (the persistent sweep),
// where a line left in this SM's L1 could be stale.
template <class T, int N, bool CG = false>
__device__ __forceinline__ Vec<T, N> vload_rw(const T* p) {
    if constexpr (N == 8) {
        Vec<T, N> r;
        uint32_t u[8];
        ld_v8<CG ? 2 : 1>(p, u);
        memcpy(&r, u, 32);
        return r;
    } else if constexpr (CG) {
        Vec<T, N> r;
        if constexpr (N == 4) {
            uint4 u = __ldcg(reinterpret_cast<const uint4*>(p));
            memcpy(&r, &u, 16);
        } else if constexpr (N == 2) {
            uint2 u = __ldcg(reinterpret_cast<const uint2*>(p));
            memcpy(&r, &u, 8);
        } else {
            uint32_t u = __ldcg(reinterpret_cast<const uint32_t*>(p));
            memcpy(&r, &u, 4);
        }
        return r;
    } else {
        return *reinterpret_cast<const Vec<T, N>*>(p);
    }
}
template <class T, int N>
__device__ __forceinline__ void vstore(T* p, const Vec<T, N>& v) {
    if constexpr (N == 8) {
        uint32_t u[8];
        memcpy(u, &v, 32);
        st_v8(p, u);
    } else {
        *reinterpret_cast<Vec<T, N>*>(p) = v;
    }
}

template <class S, int N>
__device__ __forceinline__ Vec<typename S::T, N> voplus(const Vec<typename S::T, N>& a,
                                                        const Vec<typename S::T, N>& b) {
    Vec<typename S::T, N> r;
#pragma unroll
    for (int j = 0; j < N; ++j) r.v[j] = S::oplus(a.v[j], b.v[j]);
    return r;
}
template <class S, int N>
__device__ __forceinline__ Vec<typename S::T, N> vzero() {
    Vec<typename S::T, N> r;
#pragma unroll
    for (int j = 0; j < N; ++j) r.v[j] = S::zero();
    return r;
}
template <class S, int N>
__device__ __forceinline__ void vred(typename S::T* p, const Vec<typename S::T, N>& v) {
    if constexpr (std::is_same<S, SPlus>::value && N == 8) {
        atomicAdd(reinterpret_cast<float4*>(p), make_float4(v.v[0], v.v[1], v.v[2], v.v[3]));
        atomicAdd(reinterpret_cast<float4*>(p + 4), make_float4(v.v[4], v.v[5], v.v[6], v.v[7]));
    } else if constexpr (std::is_same<S, SPlus>::value && N == 4) {
        atomicAdd(reinterpret_cast<float4*>(p), make_float4(v.v[0], v.v[1], v.v[2], v.v[3]));
    } else if constexpr (std::is_same<S, SPlus>::value && N == 2) {
        atomicAdd(reinterpret_cast<float2*>(p), make_float2(v.v[0], v.v[1]));
    } else {
#pragma unroll
        for (int j = 0; j < N; ++j) S::red(p + j, v.v[j]);
    }
}

// ------------------------------------------------------------------ kernels
// Work decomposition: a launch covers right-hand-side tiles
// [t0, t0 + gridDim.y) of Bt words each (blockIdx.y = tile).  Within a tile an
// item is (unit, lane): G = Bt / VEC lanes per unit (rule, emission or row
// segment), each lane moving VEC consecutive words.  G is a power of two
// given as GLOG (shifts, no division); GLOG < 0 selects a generic G.
// The arena and the terminal table are tile-major ([tile][slot][Bt]) so the
// values of one tile are dense; X and Y keep the caller's [row][Bw] layout.
struct SweepArgs {
    void* arena;   // [ntile][n_ops][Bt]
    void* T;       // [ntile][U][Bt]
    void* Y;       // [rows][ldy]
    const void* X; // [cols][ldx]
    const float* V;
    const int32_t* term_val;
    const int32_t* term_col;
    int64_t n_terms;  // U (zero terminal included)
    int64_t n_ops;
    int64_t rows;
    int ldx, ldy;     // words per row of X / Y
    int Bt;           // words per slot in one tile
    int G;            // lanes per unit
    int t0;           // first tile of the launch
    // Direct terminal emissions (graphs, whose terminal table dwarfs X): the
    // terminal emissions carry codes val * cols + col (em_tcode) and fold
    // leaf(V[val], X[col]) straight from X; the prologue then fills T only for
    // the terminals that rules reference (rule_terms).  nullptr: off.
    const int32_t* em_tcode = nullptr;
    const int32_t* rule_terms = nullptr;
    int64_t n_rule_terms = 0;
    int32_t cols = 0;
};

struct LevelArgs {
    const int2* ops;    // (left, right) references
    const float* op_c;  // nullptr: all coefficients are 1
    int64_t op_first;   // first arena slot of the level
    int64_t n_ops;
    const int32_t* em_src;
    const int32_t* em_row;
    int64_t em_first;
    int64_t n_em;
    const int32_t* seg_row;
    const int64_t* seg_start;
    int64_t seg_first;
    int64_t n_seg;
    int em_blocks;      // blocks [0, em_blocks) fold emissions, the rest evaluate ops
    int em_chunk;       // emissions per lane group (chunked segmented mode)
    bool direct;        // em_src holds terminal codes (see SweepArgs::em_tcode)
    bool direct_ops;    // ops' terminal children are codes: -1 zero terminal, -(code + 2)
    // Push: the ops of this launch fold their own values into the rows that
    // emit them (rows of slot s: pe_row[pe_off[s] .. pe_off[s+1])), straight
    // from registers with one vector reduction per (emission, lane); the next
    // launch then folds nothing of this level.  nullptr: pulled as usual.
    const int32_t* pe_off = nullptr;
    const int32_t* pe_row = nullptr;
    // Staging (k_level_staged): bytes of the shared-memory window, and the
    // error word a wait that gives up sets (err[0] = 1, err[1] = -(level)).
    int stage_bytes = 0;
    int* err = nullptr;
    int level = 0;
};

template <int GLOG>
__device__ __forceinline__ int64_t unit_of(int64_t t, int G) {
    if constexpr (GLOG >= 0) return t >> GLOG;
    else return t / G;
}
template <int GLOG>
__device__ __forceinline__ int lane_of(int64_t t, int G) {
    if constexpr (GLOG >= 0) return (int)(t & ((1 << GLOG) - 1));
    else return (int)(t % G);
}
template <int GLOG>
__device__ __forceinline__ int64_t items_of(int64_t units, int G) {
    if constexpr (GLOG >= 0) return units << GLOG;
    else return units * G;
}

// Per-tile view of the value space: arena slots (refs >= 0) and terminals
// (refs < 0, T[-ref-1]); the address is selected without branching.
template <class S, int VEC, bool CG = false>
struct Values {
    using T = typename S::T;
    const T* arena;
    const T* term;
    const T* X;
    const float* V;
    int Bt, ldx;
    uint32_t cols;
    __device__ __forceinline__ Values(const SweepArgs& a, int tile)
        : arena(static_cast<const T*>(a.arena) + (int64_t)tile * a.n_ops * a.Bt),
          term(static_cast<const T*>(a.T) + (int64_t)tile * a.n_terms * a.Bt),
          X(static_cast<const T*>(a.X) + (int64_t)tile * a.Bt),
          V(a.V),
          Bt(a.Bt),
          ldx(a.ldx),
          cols((uint32_t)a.cols) {}
    __device__ __forceinline__ const T* addr(int32_t c, int lane) const {
        const bool slot = c >= 0;
        const int64_t idx = slot ? (int64_t)c : (-(int64_t)c - 1);
        return (slot ? arena : term) + idx * Bt + lane * VEC;
    }
    __device__ __forceinline__ Vec<T, VEC> get(int32_t c, int lane) const {
        return vload_rw<T, VEC, CG>(addr(c, lane));
    }
    // leaf(V[val], X[col]) of the terminal with code val * cols + col.
    __device__ __forceinline__ Vec<T, VEC> leaf_of(uint32_t code, int lane) const {
        const uint32_t vi = code / cols, col = code - vi * cols;
        const float v = __ldg(V + vi);
        const Vec<T, VEC> x = vload<T, VEC>(X + (int64_t)col * ldx + lane * VEC);
        Vec<T, VEC> out;
#pragma unroll
        for (int j = 0; j < VEC; ++j) out.v[j] = S::leaf(v, x.v[j]);
        return out;
    }
    // An emission's value: its reference, or with DIRECT a terminal code
    // (< 0: the zero terminal) evaluated from X.
    template <bool DIRECT>
    __device__ __forceinline__ Vec<T, VEC> get_em(int32_t c, int lane) const {
        if constexpr (!DIRECT) {
            return get(c, lane);
        } else {
            if (c < 0) return vzero<S, VEC>();
            return leaf_of((uint32_t)c, lane);
        }
    }
    // A rule child: a slot, the zero terminal (-1), or with DIRECT a
    // terminal code stored as -(code + 2).
    template <bool DIRECT>
    __device__ __forceinline__ Vec<T, VEC> get_op(int32_t c, int lane) const {
        if constexpr (!DIRECT) {
            return get(c, lane);
        } else {
            if (c >= -1) return get(c, lane);
            return leaf_of((uint32_t)(-(int64_t)c - 2), lane);
        }
    }
};

template <class T>
__device__ __forceinline__ T* yptr(const SweepArgs& a, int64_t row, int tile, int lane, int vec) {
    return static_cast<T*>(a.Y) + row * a.ldy + (int64_t)tile * a.Bt + lane * vec;
}

// Prologue: Y = zero, T[0] = zero, T[q] = leaf(V[val], X[col]).
template <class S, int VEC, int GLOG>
__device__ __forceinline__ void do_prologue(const SweepArgs& a, int tile, int64_t t0, int64_t stride) {
    using T = typename S::T;
    const int64_t nq = a.rule_terms ? a.n_rule_terms : a.n_terms;
    const int64_t ny = items_of<GLOG>(a.rows, a.G), nt = items_of<GLOG>(nq, a.G);
    T* Tt = static_cast<T*>(a.T) + (int64_t)tile * a.n_terms * a.Bt;
    for (int64_t t = t0; t < ny + nt; t += stride) {
        if (t < ny) {
            vstore<T, VEC>(yptr<T>(a, unit_of<GLOG>(t, a.G), tile, lane_of<GLOG>(t, a.G), VEC), vzero<S, VEC>());
        } else {
            const int64_t u = t - ny;
            const int64_t i = unit_of<GLOG>(u, a.G);
            const int64_t q = a.rule_terms ? (int64_t)__ldg(a.rule_terms + i) : i;
            const int lane = lane_of<GLOG>(u, a.G);
            Vec<T, VEC> out;
            if (q == 0) {
                out = vzero<S, VEC>();
            } else {
                float v = __ldg(a.V + __ldg(a.term_val + q - 1));
                int32_t col = __ldg(a.term_col + q - 1);
                Vec<T, VEC> x = vload<T, VEC>(static_cast<const T*>(a.X) + (int64_t)col * a.ldx +
                                              (int64_t)tile * a.Bt + lane * VEC);
#pragma unroll
                for (int j = 0; j < VEC; ++j) out.v[j] = S::leaf(v, x.v[j]);
            }
            vstore<T, VEC>(Tt + q * a.Bt + lane * VEC, out);
        }
    }
}

template <class S, int VEC, int GLOG>
__global__ void __launch_bounds__(256) k_prologue(SweepArgs a) {
    do_prologue<S, VEC, GLOG>(a, a.t0 + blockIdx.y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                              (int64_t)gridDim.x * blockDim.x);
}

// Push of two freshly computed values into the rows that emit them: the
// reductions are fire-and-forget (no value comes back), and Y is small
// enough to stay in L2, so they cost L2 atomic bandwidth but no gather.
// Row lists are walked four ahead; the second value's list follows the first.
template <class S, int VEC>
__device__ __forceinline__ void push_rows(const SweepArgs& a, const LevelArgs& L, int64_t slot, int tile, int lane,
                                          const Vec<typename S::T, VEC>& v) {
    using T = typename S::T;
    const int32_t p1 = __ldg(L.pe_off + slot + 1);
    int32_t p = __ldg(L.pe_off + slot);
    for (; p + 4 <= p1; p += 4) {
        int32_t r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j] = __ldg(L.pe_row + p + j);
#pragma unroll
        for (int j = 0; j < 4; ++j) vred<S, VEC>(yptr<T>(a, r[j], tile, lane, VEC), v);
    }
    for (; p < p1; ++p) vred<S, VEC>(yptr<T>(a, __ldg(L.pe_row + p), tile, lane, VEC), v);
}

// Evaluate the ops of one level, two items per thread in flight; with
// L.pe_off set, each value is also pushed into its emitting rows of Y.
template <class S, int VEC, int GLOG, bool CG = false, bool DIR = false>
__device__ __forceinline__ void do_ops(const SweepArgs& a, const LevelArgs& L, int tile, int64_t t0,
                                       int64_t stride) {
    using T = typename S::T;
    const Values<S, VEC, CG> val(a, tile);
    T* out = static_cast<T*>(a.arena) + (int64_t)tile * a.n_ops * a.Bt;
    const int64_t items = items_of<GLOG>(L.n_ops, a.G);
    for (int64_t t = t0; t < items; t += 2 * stride) {
        const int64_t tb = t + stride;
        const bool hb = tb < items;
        const int64_t sa = L.op_first + unit_of<GLOG>(t, a.G), sb = L.op_first + unit_of<GLOG>(hb ? tb : t, a.G);
        const int la = lane_of<GLOG>(t, a.G), lb = lane_of<GLOG>(hb ? tb : t, a.G);
        const int2 oa = __ldg(L.ops + sa), ob = __ldg(L.ops + sb);
        Vec<T, VEC> la_v = val.template get_op<DIR>(oa.x, la), ra_v = val.template get_op<DIR>(oa.y, la);
        Vec<T, VEC> lb_v = val.template get_op<DIR>(ob.x, lb), rb_v = val.template get_op<DIR>(ob.y, lb);
        if (L.op_c) {
            const float ca = __ldg(L.op_c + sa), cb = __ldg(L.op_c + sb);
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                la_v.v[j] = S::apply(la_v.v[j], ca);
                lb_v.v[j] = S::apply(lb_v.v[j], cb);
            }
        }
        const Vec<T, VEC> va = voplus<S, VEC>(la_v, ra_v), vb = voplus<S, VEC>(lb_v, rb_v);
        vstore<T, VEC>(out + sa * a.Bt + la * VEC, va);
        if (hb) vstore<T, VEC>(out + sb * a.Bt + lb * VEC, vb);
        if (L.pe_off) {
            push_rows<S, VEC>(a, L, sa, tile, la, va);
            if (hb) push_rows<S, VEC>(a, L, sb, tile, lb, vb);
        }
    }
}

// One atomic per (emission, word): the reference's emit scheme.
template <class S, int VEC, int GLOG, bool CG = false, bool DIR = false>
__device__ __forceinline__ void do_emits_atomic(const SweepArgs& a, const LevelArgs& L, int tile, int64_t t0,
                                                int64_t stride) {
    using T = typename S::T;
    const Values<S, VEC, CG> val(a, tile);
    const int64_t items = items_of<GLOG>(L.n_em, a.G);
    for (int64_t t = t0; t < items; t += stride) {
        const int64_t e = L.em_first + unit_of<GLOG>(t, a.G);
        const int lane = lane_of<GLOG>(t, a.G);
        const int32_t src = __ldg(L.em_src + e), row = __ldg(L.em_row + e);
        vred<S, VEC>(yptr<T>(a, row, tile, lane, VEC), val.template get_em<DIR>(src, lane));
    }
}

// Warp-segmented emits when G == 1: lane = emission; rows are sorted, so
// equal rows are contiguous lanes; each segment is reduced in registers
// (shuffles for (+,x), __reduce_*_sync for OR / min) and its first lane issues
// one atomic per word.  Two warp-blocks are in flight per iteration.
template <class S, int VEC>
__device__ __forceinline__ Vec<typename S::T, VEC> warp_segment_reduce(Vec<typename S::T, VEC> v, unsigned peers,
                                                                       int lane) {
    using T = typename S::T;
    Vec<T, VEC> tot;
    if constexpr (std::is_same<S, SBool>::value) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) tot.v[j] = __reduce_or_sync(peers, v.v[j]);
    } else if constexpr (std::is_same<S, STrop>::value) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) tot.v[j] = __reduce_min_sync(peers, v.v[j]);
    } else {
        const int last = 31 - __clz(peers);  // segments are contiguous lanes
        tot = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                T o = __shfl_down_sync(0xffffffffu, tot.v[j], d);
                if (lane + d <= last) tot.v[j] = S::oplus(tot.v[j], o);
            }
        }
    }
    return tot;
}

template <class S, int VEC, bool CG = false, bool DIR = false>
__device__ __forceinline__ void do_emits_warp(const SweepArgs& a, const LevelArgs& L, int tile, int64_t t0,
                                              int64_t stride) {
    using T = typename S::T;
    const Values<S, VEC, CG> val(a, tile);
    const int lane = threadIdx.x & 31;
    const int64_t n = L.n_em;
    for (int64_t base = t0 - lane; base < n; base += 2 * stride) {  // warp-uniform trip count
        const int64_t ea = base + lane, eb = base + stride + lane;
        const bool va = ea < n, vb = eb < n;
        const int32_t ra = va ? __ldg(L.em_row + L.em_first + ea) : -1 - lane;
        const int32_t rb = vb ? __ldg(L.em_row + L.em_first + eb) : -1 - lane;
        const int32_t sa = va ? __ldg(L.em_src + L.em_first + ea) : -1;
        const int32_t sb = vb ? __ldg(L.em_src + L.em_first + eb) : -1;
        Vec<T, VEC> xa = val.template get_em<DIR>(sa, 0), xb = val.template get_em<DIR>(sb, 0);  // -1: zero
        const unsigned pa = __match_any_sync(0xffffffffu, ra), pb = __match_any_sync(0xffffffffu, rb);
        Vec<T, VEC> ta = warp_segment_reduce<S, VEC>(xa, pa, lane);
        Vec<T, VEC> tb = warp_segment_reduce<S, VEC>(xb, pb, lane);
        if (va && lane == __ffs(pa) - 1) vred<S, VEC>(yptr<T>(a, ra, tile, 0, VEC), ta);
        if (vb && lane == __ffs(pb) - 1) vred<S, VEC>(yptr<T>(a, rb, tile, 0, VEC), tb);
    }
}

// Chunked segmented emits: each lane group walks em_chunk consecutive
// emissions (loads four ahead), accumulating while the row stays the same.
template <class S, int VEC, int GLOG, bool CG = false, bool DIR = false>
__device__ __forceinline__ void do_emits_chunk(const SweepArgs& a, const LevelArgs& L, int tile, int64_t t0,
                                               int64_t stride) {
    using T = typename S::T;
    const Values<S, VEC, CG> val(a, tile);
    const int64_t groups = (L.n_em + L.em_chunk - 1) / L.em_chunk;
    const int64_t items = items_of<GLOG>(groups, a.G);
    const int32_t* rows = L.em_row + L.em_first;
    const int32_t* srcs = L.em_src + L.em_first;
    for (int64_t t = t0; t < items; t += stride) {
        const int64_t g = unit_of<GLOG>(t, a.G);
        const int lane = lane_of<GLOG>(t, a.G);
        const int64_t e0 = g * L.em_chunk, e1 = min(e0 + (int64_t)L.em_chunk, L.n_em);
        int32_t cur = __ldg(rows + e0);
        Vec<T, VEC> acc = vzero<S, VEC>();
        int64_t e = e0;
        for (; e + 4 <= e1; e += 4) {
            int32_t r[4], s[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                r[j] = __ldg(rows + e + j);
                s[j] = __ldg(srcs + e + j);
            }
            Vec<T, VEC> v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = val.template get_em<DIR>(s[j], lane);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (r[j] != cur) {
                    vred<S, VEC>(yptr<T>(a, cur, tile, lane, VEC), acc);
                    acc = v[j];
                    cur = r[j];
                } else {
                    acc = voplus<S, VEC>(acc, v[j]);
                }
            }
        }
        for (; e < e1; ++e) {
            const int32_t r = __ldg(rows + e);
            Vec<T, VEC> v = val.template get_em<DIR>(__ldg(srcs + e), lane);
            if (r != cur) {
                vred<S, VEC>(yptr<T>(a, cur, tile, lane, VEC), acc);
                acc = v;
                cur = r;
            } else {
                acc = voplus<S, VEC>(acc, v);
            }
        }
        vred<S, VEC>(yptr<T>(a, cur, tile, lane, VEC), acc);
    }
}

// Row-owned emits: one lane group folds a whole (level, row) segment and
// updates its row of Y with a plain read-modify-write.  Within a launch every
// (row, tile) belongs to exactly one segment and levels are separate launches,
// so no atomics are needed and the (+,x) summation order is fixed.
template <class S, int VEC, int GLOG, bool CG = false, bool DIR = false>
__device__ __forceinline__ void do_emits_rows(const SweepArgs& a, const LevelArgs& L, int tile, int64_t t0,
                                              int64_t stride) {
    using T = typename S::T;
    const Values<S, VEC, CG> val(a, tile);
    const int64_t items = items_of<GLOG>(L.n_seg, a.G);
    for (int64_t t = t0; t < items; t += stride) {
        const int64_t s = L.seg_first + unit_of<GLOG>(t, a.G);
        const int lane = lane_of<GLOG>(t, a.G);
        const int64_t e0 = __ldg(L.seg_start + s), e1 = __ldg(L.seg_start + s + 1);
        const int32_t row = __ldg(L.seg_row + s);
        Vec<T, VEC> acc0 = vzero<S, VEC>(), acc1 = vzero<S, VEC>();
        int64_t e = e0;
        for (; e + 4 <= e1; e += 4) {
            const int32_t s0 = __ldg(L.em_src + e), s1 = __ldg(L.em_src + e + 1);
            const int32_t s2 = __ldg(L.em_src + e + 2), s3 = __ldg(L.em_src + e + 3);
            Vec<T, VEC> v0 = val.template get_em<DIR>(s0, lane), v1 = val.template get_em<DIR>(s1, lane);
            Vec<T, VEC> v2 = val.template get_em<DIR>(s2, lane), v3 = val.template get_em<DIR>(s3, lane);
            acc0 = voplus<S, VEC>(acc0, voplus<S, VEC>(v0, v1));
            acc1 = voplus<S, VEC>(acc1, voplus<S, VEC>(v2, v3));
        }
        for (; e < e1; ++e) acc0 = voplus<S, VEC>(acc0, val.template get_em<DIR>(__ldg(L.em_src + e), lane));
        T* yp = yptr<T>(a, row, tile, lane, VEC);
        vstore<T, VEC>(yp, voplus<S, VEC>(vload_rw<T, VEC, CG>(yp), voplus<S, VEC>(acc0, acc1)));
    }
}

// Emission fold of one launch; DIR: the sources are terminal codes (see
// SweepArgs::em_tcode).  A compile-time choice, so each fold keeps its batched
// loads free of per-item branches.
template <class S, int VEC, int GLOG, int EMIT, bool CG, bool DIR>
__device__ __forceinline__ void emits_t(const SweepArgs& a, const LevelArgs& L, int tile, int64_t t0, int64_t stride) {
    if constexpr (EMIT == GMR_EMIT_ATOMIC) do_emits_atomic<S, VEC, GLOG, CG, DIR>(a, L, tile, t0, stride);
    else if constexpr (EMIT == GMR_EMIT_ROWS) do_emits_rows<S, VEC, GLOG, CG, DIR>(a, L, tile, t0, stride);
    else if constexpr (GLOG == 0) do_emits_warp<S, VEC, CG, DIR>(a, L, tile, t0, stride);
    else do_emits_chunk<S, VEC, GLOG, CG, DIR>(a, L, tile, t0, stride);
}

// One level launch: blocks [0, em_blocks) fold emissions, the rest evaluate ops.
// DIRK (direct terminals): 0 off; 1 rule children are terminal codes; 2 the
// emissions too (the launch that folds the terminal emissions).
template <class S, int VEC, int GLOG, int EMIT, int DIRK = 0>
__global__ void __launch_bounds__(256, VEC == 8 ? 4 : 1) k_level(SweepArgs a, LevelArgs L) {
    const int tile = a.t0 + blockIdx.y;
    if ((int)blockIdx.x < L.em_blocks) {
        const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const int64_t stride = (int64_t)L.em_blocks * blockDim.x;
        emits_t<S, VEC, GLOG, EMIT, false, DIRK == 2>(a, L, tile, t0, stride);
    } else {
        const int64_t t0 = (int64_t)(blockIdx.x - L.em_blocks) * blockDim.x + threadIdx.x;
        const int64_t stride = (int64_t)(gridDim.x - L.em_blocks) * blockDim.x;
        do_ops<S, VEC, GLOG, false, DIRK >= 1>(a, L, tile, t0, stride);
    }
}

// Shared-memory staging of the left-child window (GMR_LEVEL_STAGE).  Rules of
// a level are sorted by left child, so the slot children of R consecutive
// rules lie in one window [lo, hi] of the arena.  An ops block takes runs of
// R = 2 * (256 / G) rules; for each run one thread posts the window's byte
// count on an mbarrier and issues ONE bulk copy (cp.async.bulk) of the window
// into shared memory when it fits in L.stage_bytes, while every thread loads
// its rules and right children from global memory; the left children are
// then read from shared memory.  Runs whose window does not fit (or holds no
// slot) read both children from global memory.  Emission blocks fold as
// k_level's segmented fold.  The wait is bounded: after the limit the block
// sets L.err, waits (again bounded) for its copy and returns.
static constexpr int kStageBytes = 47 * 1024;  // with the static words, within the 48 KB a block gets without opting in
static constexpr unsigned long long kStageSpinLimit = 20000000ull;

template <class S, int VEC, int GLOG>
__global__ void __launch_bounds__(256, VEC == 8 ? 4 : 1) k_level_staged(SweepArgs a, LevelArgs L) {
    static_assert(GLOG >= 0 && VEC >= 4, "staging needs a power-of-two lane count and 16-byte values");
    using T = typename S::T;
    extern __shared__ __align__(128) unsigned char win_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ long long s_lo, s_hi;
    __shared__ int s_use, s_ok;
    const int tile = a.t0 + blockIdx.y;
    if ((int)blockIdx.x < L.em_blocks) {
        emits_t<S, VEC, GLOG, GMR_EMIT_SEGMENTED, false, false>(
            a, L, tile, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)L.em_blocks * blockDim.x);
        return;
    }
    constexpr int kUnits = 256 >> GLOG;  // rules per pass of the block
    constexpr int R = 2 * kUnits;        // rules per run
    const Values<S, VEC> val(a, tile);
    const T* arena_t = static_cast<const T*>(a.arena) + (int64_t)tile * a.n_ops * a.Bt;
    T* out = static_cast<T*>(a.arena) + (int64_t)tile * a.n_ops * a.Bt;
    const T* win = reinterpret_cast<const T*>(win_raw);
    const int u = threadIdx.x >> GLOG, lane = threadIdx.x & ((1 << GLOG) - 1);
    const int ob = (int)blockIdx.x - L.em_blocks, nob = (int)gridDim.x - L.em_blocks;
    const int2* ops = L.ops + L.op_first;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    uint32_t phase = 0;
    for (int64_t r0 = (int64_t)ob * R; r0 < L.n_ops; r0 += (int64_t)nob * R) {
        const int64_t r1 = min(r0 + (int64_t)R, L.n_ops);
        if (threadIdx.x == 0) {
            int64_t lo_i = r0, hi_i = r1;  // first rule whose left child is a slot
            while (lo_i < hi_i) {
                const int64_t mid = (lo_i + hi_i) >> 1;
                if (__ldg(&ops[mid].x) >= 0) hi_i = mid;
                else lo_i = mid + 1;
            }
            int use = 0;
            long long lo = 0, hi = -1;
            if (lo_i < r1) {
                lo = __ldg(&ops[lo_i].x);
                hi = __ldg(&ops[r1 - 1].x);
                const long long bytes = (hi - lo + 1) * (long long)a.Bt * 4;
                if (bytes <= L.stage_bytes) {
                    use = 1;
                    fence_proxy_async_smem();  // the previous run's reads of the window come first
                    mbar_arrive_expect_tx(&bar, (uint32_t)bytes);
                    bulk_g2s(win_raw, arena_t + lo * a.Bt, (uint32_t)bytes, &bar);
                }
            }
            s_use = use;
            s_lo = lo;
            s_hi = hi;
        }
        __syncthreads();
        const int use = s_use;
        const long long lo = s_lo, hi = s_hi;
        const int64_t ia = r0 + u, ib = r0 + u + kUnits;
        const bool ha = ia < r1, hb = ib < r1;
        const int2 oa = ha ? __ldg(ops + ia) : make_int2(-1, -1);
        const int2 ob2 = hb ? __ldg(ops + ib) : make_int2(-1, -1);
        Vec<T, VEC> ra_v = val.get(oa.y, lane), rb_v = val.get(ob2.y, lane);
        Vec<T, VEC> la_v, lb_v;
        if (use) {
            if (threadIdx.x == 0) s_ok = mbar_wait(&bar, phase, kStageSpinLimit) ? 1 : 0;
            __syncthreads();
            if (!s_ok) {
                if (threadIdx.x == 0) {
                    L.err[1] = -L.level;
                    __threadfence();
                    atomicExch(L.err, 1);
                    mbar_wait(&bar, phase, kStageSpinLimit);  // the copy still lands in this block's memory
                }
                __syncthreads();
                return;
            }
            phase ^= 1u;
            // a child outside [lo, hi] (not possible for a level sorted by
            // left child, checked anyway) is read from global memory
            la_v = oa.x >= lo && oa.x <= hi
                       ? *reinterpret_cast<const Vec<T, VEC>*>(win + (oa.x - lo) * a.Bt + lane * VEC)
                       : val.get(oa.x, lane);
            lb_v = ob2.x >= lo && ob2.x <= hi
                       ? *reinterpret_cast<const Vec<T, VEC>*>(win + (ob2.x - lo) * a.Bt + lane * VEC)
                       : val.get(ob2.x, lane);
        } else {
            la_v = val.get(oa.x, lane);
            lb_v = val.get(ob2.x, lane);
        }
        if (L.op_c) {
            const float ca = ha ? __ldg(L.op_c + L.op_first + ia) : 1.0f;
            const float cb = hb ? __ldg(L.op_c + L.op_first + ib) : 1.0f;
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                la_v.v[j] = S::apply(la_v.v[j], ca);
                lb_v.v[j] = S::apply(lb_v.v[j], cb);
            }
        }
        if (ha) vstore<T, VEC>(out + (L.op_first + ia) * a.Bt + lane * VEC, voplus<S, VEC>(la_v, ra_v));
        if (hb) vstore<T, VEC>(out + (L.op_first + ib) * a.Bt + lane * VEC, voplus<S, VEC>(lb_v, rb_v));
        __syncthreads();  // every read of the window is done before the next run's copy
    }
}

// Persistent sweep: one cooperative launch walks the prologue and every
// level, separated by grid barriers.  Each barrier wait is bounded: a block
// that waits longer than spin_limit polls (or sees another block's failure)
// records the phase in err[1], sets err[0] and every block returns; the host
// reads err and reports GMR_ERR_TIMEOUT.  There are no asynchronous copies
// in flight at a barrier, so returning early leaves nothing pending.
struct PersistArgs {
    const int64_t* lvl_off;  // depth + 1 (device)
    const int64_t* em_off;   // depth + 2
    const int64_t* seg_off;  // depth + 2
    int depth;
    unsigned* bar;           // [0] arrivals, [1] generation
    int* err;                // [0] failed, [1] phase that gave up
    unsigned long long spin_limit;
};

__device__ __forceinline__ bool grid_barrier(const PersistArgs& P, int phase) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = P.bar + 1;
        volatile int* err = P.err;
        const unsigned g0 = *gen;  // before arriving: cannot change until every block has arrived
        __threadfence();
        const unsigned arrived = atomicAdd(P.bar, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(P.bar, 0u);
            __threadfence();
            atomicAdd(P.bar + 1, 1u);
        } else {
            unsigned long long n = 0;
            while (*gen == g0) {
                if (*err) break;
                if (++n > P.spin_limit) {
                    P.err[1] = phase;
                    __threadfence();
                    atomicExch(P.err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)P.err == 0;
}

template <class S, int VEC, int GLOG, int EMIT>
__global__ void __launch_bounds__(256) k_persistent(SweepArgs a, LevelArgs L0, PersistArgs P) {
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    do_prologue<S, VEC, GLOG>(a, 0, t0, stride);
    if (!grid_barrier(P, 0)) return;
    for (int k = 1; k <= P.depth + 1; ++k) {
        LevelArgs L = L0;
        if (k <= P.depth) {
            L.op_first = P.lvl_off[k - 1];
            L.n_ops = P.lvl_off[k] - P.lvl_off[k - 1];
        } else {
            L.n_ops = 0;
        }
        L.em_first = P.em_off[k - 1];
        L.n_em = P.em_off[k] - P.em_off[k - 1];
        L.seg_first = P.seg_off[k - 1];
        L.n_seg = P.seg_off[k] - P.seg_off[k - 1];
        emits_t<S, VEC, GLOG, EMIT, true, false>(a, L, 0, t0, stride);
        do_ops<S, VEC, GLOG, true, false>(a, L, 0, t0, stride);
        if (!grid_barrier(P, k)) return;
    }
}

// Several grammars in ONE persistent launch.  Each grammar brings its own
// plan, scratch, X, Y and batch width (its lane layout is `kind`, a
// (VEC, GLOG) class); phase k runs level k of every grammar that still has
// one (rules of level k, emissions of level k-1; phase 0 the prologues),
// every grammar over the whole grid one after another, so a small grammar's
// few rules fill the threads a big grammar leaves idle.  One bounded grid
// barrier separates the phases.
struct PackGrammar {
    SweepArgs a;
    LevelArgs L;  // level-independent fields (arrays, chunk)
    const int64_t* lvl_off;
    const int64_t* em_off;
    const int64_t* seg_off;
    int depth;
    int kind;     // 0-6: VEC 4 with GLOG 0..5 / generic; 7, 8: VEC 2 / 1 with G = 1; 9, 10: VEC 2 / 1 generic
};

// The grammar's argument structs are copied into locals first: read through
// a pointer they would be reloaded from global memory inside the loops.
template <class S, int VEC, int GLOG, int EMIT>
__device__ __forceinline__ void pack_phase(const PackGrammar& g, int k, int64_t t0, int64_t stride) {
    const SweepArgs a = g.a;
    if (k == 0) {
        do_prologue<S, VEC, GLOG>(a, 0, t0, stride);
        return;
    }
    LevelArgs L = g.L;
    if (k <= g.depth) {
        L.op_first = g.lvl_off[k - 1];
        L.n_ops = g.lvl_off[k] - g.lvl_off[k - 1];
    } else {
        L.n_ops = 0;
    }
    L.em_first = g.em_off[k - 1];
    L.n_em = g.em_off[k] - g.em_off[k - 1];
    L.seg_first = g.seg_off[k - 1];
    L.n_seg = g.seg_off[k] - g.seg_off[k - 1];
    emits_t<S, VEC, GLOG, EMIT, true, false>(a, L, 0, t0, stride);
    do_ops<S, VEC, GLOG, true, false>(a, L, 0, t0, stride);
}

template <class S, int EMIT>
__global__ void __launch_bounds__(256) k_pack(const PackGrammar* __restrict__ gs, int n, int max_depth, PersistArgs P) {
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int k = 0; k <= max_depth + 1; ++k) {
        for (int i = 0; i < n; ++i) {
            const PackGrammar& g = gs[i];
            if (k > g.depth + 1) continue;
            switch (g.kind) {
                case 0: pack_phase<S, 4, 0, EMIT>(g, k, t0, stride); break;
                case 1: pack_phase<S, 4, 1, EMIT>(g, k, t0, stride); break;
                case 2: pack_phase<S, 4, 2, EMIT>(g, k, t0, stride); break;
                case 3: pack_phase<S, 4, 3, EMIT>(g, k, t0, stride); break;
                case 4: pack_phase<S, 4, 4, EMIT>(g, k, t0, stride); break;
                case 5: pack_phase<S, 4, 5, EMIT>(g, k, t0, stride); break;
                case 6: pack_phase<S, 4, -1, EMIT>(g, k, t0, stride); break;
                case 7: pack_phase<S, 2, 0, EMIT>(g, k, t0, stride); break;
                case 8: pack_phase<S, 1, 0, EMIT>(g, k, t0, stride); break;
                case 9: pack_phase<S, 2, -1, EMIT>(g, k, t0, stride); break;
                default: pack_phase<S, 1, -1, EMIT>(g, k, t0, stride); break;
            }
        }
        if (!grid_barrier(P, k)) return;
    }
}

// The same pack as one launch per level (GMR_PACK_LEVELS): launch k covers
// level k of every grammar, grammar i on blocks [blk[i], blk[i+1]), the first
// em_blocks[i] of them folding its emissions of level k-1 and the rest
// evaluating its rules of level k (k = 0: the prologues).  Plain cached loads:
// launch boundaries order the levels.
static constexpr int kMaxPackLevels = 32;  // grammars per pack in this mode
struct PackLaunch {
    int n, k;
    int blk[kMaxPackLevels + 1];
    int em_blocks[kMaxPackLevels];
};

template <class S, int VEC, int GLOG, int EMIT>
__device__ __forceinline__ void pack_level_part(const PackGrammar& g, int k, int b, int nb, int eb) {
    const int64_t tid = threadIdx.x;
    const SweepArgs a = g.a;
    if (k == 0) {
        do_prologue<S, VEC, GLOG>(a, 0, (int64_t)b * blockDim.x + tid, (int64_t)nb * blockDim.x);
        return;
    }
    LevelArgs L = g.L;
    if (k <= g.depth) {
        L.op_first = g.lvl_off[k - 1];
        L.n_ops = g.lvl_off[k] - g.lvl_off[k - 1];
    } else {
        L.n_ops = 0;
    }
    L.em_first = g.em_off[k - 1];
    L.n_em = g.em_off[k] - g.em_off[k - 1];
    L.seg_first = g.seg_off[k - 1];
    L.n_seg = g.seg_off[k] - g.seg_off[k - 1];
    if (b < eb) emits_t<S, VEC, GLOG, EMIT, false, false>(a, L, 0, (int64_t)b * blockDim.x + tid, (int64_t)eb * blockDim.x);
    else do_ops<S, VEC, GLOG, false, false>(a, L, 0, (int64_t)(b - eb) * blockDim.x + tid, (int64_t)(nb - eb) * blockDim.x);
}

template <class S, int EMIT>
__global__ void __launch_bounds__(256) k_pack_level(const PackGrammar* __restrict__ gs, PackLaunch P) {
    int i = 0;
    while (i + 1 < P.n && (int)blockIdx.x >= P.blk[i + 1]) ++i;
    const PackGrammar& g = gs[i];
    const int b = (int)blockIdx.x - P.blk[i], nb = P.blk[i + 1] - P.blk[i], eb = P.em_blocks[i];
    switch (g.kind) {
        case 0: pack_level_part<S, 4, 0, EMIT>(g, P.k, b, nb, eb); break;
        case 1: pack_level_part<S, 4, 1, EMIT>(g, P.k, b, nb, eb); break;
        case 2: pack_level_part<S, 4, 2, EMIT>(g, P.k, b, nb, eb); break;
        case 3: pack_level_part<S, 4, 3, EMIT>(g, P.k, b, nb, eb); break;
        case 4: pack_level_part<S, 4, 4, EMIT>(g, P.k, b, nb, eb); break;
        case 5: pack_level_part<S, 4, 5, EMIT>(g, P.k, b, nb, eb); break;
        case 6: pack_level_part<S, 4, -1, EMIT>(g, P.k, b, nb, eb); break;
        case 7: pack_level_part<S, 2, 0, EMIT>(g, P.k, b, nb, eb); break;
        case 8: pack_level_part<S, 1, 0, EMIT>(g, P.k, b, nb, eb); break;
        case 9: pack_level_part<S, 2, -1, EMIT>(g, P.k, b, nb, eb); break;
        default: pack_level_part<S, 1, -1, EMIT>(g, P.k, b, nb, eb); break;
    }
}

// ------------------------------------------------------------------ engine
// Fully resolved launch configuration of one multiply.
// Kernel variants a k_level launch can use: emission folding strategy and
// chunk, and how many CTAs evaluate the level's rules (few CTAs = many
// rules per CTA).  Variant v = emit index + GMR_N_EMIT_VARIANTS * grid index.
struct EmitVariant {
    int emit, chunk;
};
static constexpr EmitVariant kEmitVariants[] = {
    {GMR_EMIT_SEGMENTED, 16}, {GMR_EMIT_SEGMENTED, 8}, {GMR_EMIT_SEGMENTED, 32}, {GMR_EMIT_ROWS, 0},
    {GMR_EMIT_ATOMIC, 0}};
static constexpr int kNumEmitVariants = 5;
static constexpr int kOpsCtasPerSm[] = {32, 4};
// v = emit + 5 * grid + 10 * chunked (chunked: fold the emissions of a level
// one source chunk at a time, see gmr_engine::ch_*)
static_assert(kNumEmitVariants * 2 * 2 == GMR_N_LEVEL_VARIANTS, "variant table size");
static constexpr int64_t kChunkSlots = 1 << 19;  // source slots per chunk (64 MB of values at 32 words)

struct Launch {
    int semiring, B, Bw, VEC, G, variant, emit, chunk;
    int Bt, ntile, tile_levels;
    int push_mode;  // GMR_PUSH_*
    unsigned long long spin_limit;
    std::vector<uint8_t> lv;  // per-launch variant (index = launch slot), empty = uniform emit/chunk
    bool operator==(const Launch& o) const {
        return semiring == o.semiring && B == o.B && Bw == o.Bw && VEC == o.VEC && variant == o.variant &&
               emit == o.emit && chunk == o.chunk && Bt == o.Bt && tile_levels == o.tile_levels &&
               push_mode == o.push_mode && lv == o.lv;
    }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    Launch lc{};
    int64_t launches = 0;  // kernel launches inside the graph (one iteration for a fixpoint loop)
    const void* X = nullptr;
    void* Y = nullptr;
    bool fixpoint = false;  // a whole fixpoint loop (conditional while node) rather than one multiply
};

}  // namespace gmr

struct gmr_engine {
    int device = 0;
    int rows = 0, cols = 0, depth = 0;
    int64_t n_ops = 0, n_terms = 0, n_em = 0;
    bool has_coeff = false;
    std::vector<int64_t> lvl_off, em_off, seg_off;
    gmr::DevBuf ops, op_c, em_src, em_row, seg_row, seg_start, term_val, term_col, V;
    gmr::DevBuf arena, T, hX, hY;  // scratch
    gmr::DevBuf hX2, hY2;          // second staging pair of the pipelined host-buffer multiply
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t pipe_ev[6] = {};    // per staging slot: X copied in, multiply done, Y copied out
    gmr::DevBuf d_lvl_off, d_em_off, d_seg_off, sync;  // persistent variant: level tables, barrier + error words
    // The emissions again, ordered by (source chunk, row, source) within each
    // level, with row segments per chunk: chunk c of level k covers source
    // slots [c, c+1) * kChunkSlots of that level (terminals for level 0).
    // Level k's chunks are [ch_off[k], ch_off[k+1]); chunk i's emissions
    // [ch_em[i], ch_em[i+1]) and segments [ch_seg[i], ch_seg[i+1]).
    gmr::DevBuf em_src_c, em_row_c, seg_row_c, seg_start_c;
    std::vector<int64_t> ch_off, ch_em, ch_seg;
    bool chunked = false;
    int64_t chunk_slots = 1 << 19;  // source slots per chunk
    // Direct terminal emissions (SweepArgs::em_tcode): codes of the terminal
    // emissions and the terminals rules reference.
    gmr::DevBuf em_tcode, rule_terms, ops_direct;
    int64_t n_rule_terms = 0;
    bool direct_terms = false;
    int lane_bytes = 0;  // bytes per lane access when gmr_config::lane_bytes = 0 (0: by semiring and tile); GMR_LANE_BYTES
    // Push lists (LevelArgs::pe_off): the emissions of levels 1..depth ordered
    // by source slot, rows ascending per slot; push_ok[k] = every emission of
    // level k has a slot of level k as its source, so level k can push.
    gmr::DevBuf pe_off, pe_row;
    std::vector<uint8_t> push_ok;
    // Left product (y = x^T M): flat edge lists uploaded by gmr_engine_enable_left.
    gmr::DevBuf le_src, le_tgt, le_split, tcol_off, tcol_q;
    std::vector<int64_t> le_off;
    int64_t n_left_split = 0;
    bool left_ready = false;
    int* status_host = nullptr;                           // pinned copy of the last error words
    bool last_persistent = false;  // the last multiply reported error words (persistent or staged launches)
    // sync (64 bytes, allocated once with the engine so that captured graphs
    // keep a valid address): [0, 8) persistent barrier, [8, 16) persistent
    // error words, [8, 20) fixpoint flag / count / limit, [32, 40) staged-wait
    // error words
    int* stage_err() { return reinterpret_cast<int*>(static_cast<unsigned char*>(sync.p) + 32); }
    cudaStream_t own_stream = nullptr;
    std::vector<gmr::GraphEntry> graphs;
    std::map<std::pair<int, int>, std::vector<uint8_t>> level_variants;  // (semiring, B) -> per-launch variant
    // (semiring, B) -> the last autotune's per-slot times under each pair of
    // emission modes (slot k, level k-1 in mode mp, level k in mode m: entry
    // k * 9 + 3 * mp + m, ms; -1 where not measured)
    std::map<std::pair<int, int>, std::vector<float>> mode_costs;
    int64_t last_launches = 0;
    int sm_count = 152;
    std::mutex mu;
    std::vector<gmr::DevBuf*> schedule_bufs() {
        return {&ops, &op_c, &em_src, &em_row, &seg_row, &seg_start, &term_val, &term_col, &V,
                &d_lvl_off, &d_em_off, &d_seg_off, &sync, &em_src_c, &em_row_c, &seg_row_c, &seg_start_c,
                &le_src, &le_tgt, &le_split, &tcol_off, &tcol_q, &em_tcode, &rule_terms, &ops_direct,
                &pe_off, &pe_row};
    }
};

namespace gmr {


static int words_per_slot(int semiring, int B) { return semiring == GMR_BOOLEAN ? (B + 31) / 32 : B; }

// How the emissions of level k reach Y in this multiply: gathered by the
// next launch (pull), pushed by the rules that make them (push), or level k
// evaluated in source chunks with each chunk's emissions gathered by the
// launch after it (interleave).
enum { kFoldPull = 0, kFoldPush = 1, kFoldInterleave = 2 };

// Source chunks of level k's rules (gmr_engine::chunk_slots each).
static int64_t interleave_chunks(const gmr_engine* e, int k) {
    const int64_t w = e->lvl_off[k] - e->lvl_off[k - 1];
    return (w + e->chunk_slots - 1) / e->chunk_slots;
}

static bool can_push(const gmr_engine* e, int k) {
    return k >= 1 && k <= e->depth && k < (int)e->push_ok.size() && e->push_ok[k];
}
// Interleaving needs the chunked emission order and two chunks or more; the
// levels that run tile by tile (very wide batches) never interleave.
static bool can_interleave(const gmr_engine* e, const Launch& lc, int k) {
    if (k < 1 || k > e->depth || !e->chunked || interleave_chunks(e, k) < 2) return false;
    const int K = lc.ntile > 1 ? std::min(lc.tile_levels, e->depth) : 0;
    return k > K;
}

static int level_mode(const gmr_engine* e, const Launch& lc, int k) {
    if (lc.variant == GMR_VARIANT_PLAIN || lc.variant == GMR_VARIANT_PERSISTENT) return kFoldPull;
    if (k < 1 || k > e->depth || lc.push_mode == GMR_PUSH_NEVER) return kFoldPull;
    if (lc.push_mode == GMR_PUSH_ALWAYS) return can_push(e, k) ? kFoldPush : kFoldPull;
    if (lc.push_mode == GMR_PUSH_INTERLEAVE) return can_interleave(e, lc, k) ? kFoldInterleave : kFoldPull;
    if (lc.lv.empty() || k >= (int)lc.lv.size()) return kFoldPull;
    if ((lc.lv[k] & GMR_LEVEL_INTERLEAVE) && can_interleave(e, lc, k)) return kFoldInterleave;
    if ((lc.lv[k] & GMR_LEVEL_PUSH) && can_push(e, k)) return kFoldPush;
    return kFoldPull;
}

// Whether the rules of level k run k_level_staged (GMR_LEVEL_STAGE in the
// installed table): per-level chains only, plain references (no direct
// terminal codes), 16- or 32-byte lanes in power-of-two groups, and a level
// that does not push its emissions.
static bool level_staged(const gmr_engine* e, const Launch& lc, int k) {
    if (lc.variant == GMR_VARIANT_PLAIN || lc.variant == GMR_VARIANT_PERSISTENT) return false;
    if (lc.lv.empty() || k < 1 || k > e->depth || k >= (int)lc.lv.size() || !(lc.lv[k] & GMR_LEVEL_STAGE)) return false;
    if (e->direct_terms || lc.VEC < 4 || (lc.G & (lc.G - 1)) != 0 || lc.G > 32) return false;
    return level_mode(e, lc, k) != kFoldPush;
}

// Set while the fixpoint loop's body is captured: its conditional body holds
// the level kernels only, so the staged waits' error words are reset and
// read around the whole loop instead of around each multiply.
static thread_local bool t_chain_no_status = false;

static bool any_staged(const gmr_engine* e, const Launch& lc) {
    for (int k = 1; k <= e->depth; ++k)
        if (level_staged(e, lc, k)) return true;
    return false;
}

// Optional per-launch timing: an event is recorded before the first launch
// and after every launch.
struct LaunchTimer {
    std::vector<cudaEvent_t> ev;
    cudaStream_t st = nullptr;
    void mark() {
        cudaEvent_t e;
        GMR_CUDA(cudaEventCreate(&e));
        GMR_CUDA(cudaEventRecord(e, st));
        ev.push_back(e);
    }
    ~LaunchTimer() {
        for (auto e : ev) cudaEventDestroy(e);
    }
};
static thread_local LaunchTimer* t_timer = nullptr;

template <class S, int VEC, int GLOG, int DIRK>
static void launch_level(int emit, dim3 grid, cudaStream_t st, const SweepArgs& s, const LevelArgs& M) {
    if (emit == GMR_EMIT_ATOMIC)
        k_level<S, VEC, GLOG, GMR_EMIT_ATOMIC, DIRK><<<grid, 256, 0, st>>>(s, M);
    else if (emit == GMR_EMIT_ROWS)
        k_level<S, VEC, GLOG, GMR_EMIT_ROWS, DIRK><<<grid, 256, 0, st>>>(s, M);
    else
        k_level<S, VEC, GLOG, GMR_EMIT_SEGMENTED, DIRK><<<grid, 256, 0, st>>>(s, M);
}

// Direct terminal emissions on: the sweep's terminal emissions gather X.
static void set_direct(const gmr_engine* e, SweepArgs& a) {
    a.cols = e->cols;
    if (!e->direct_terms) return;
    a.em_tcode = static_cast<const int32_t*>(e->em_tcode.p);
    a.rule_terms = static_cast<const int32_t*>(e->rule_terms.p);
    a.n_rule_terms = e->n_rule_terms;
}

template <class S, int VEC, int GLOG>
static void launch_chain_t(gmr_engine* e, const Launch& lc, const void* X, void* Y, cudaStream_t st,
                           int64_t& launches) {
    if (lc.ntile > 65535) throw Error(GMR_ERR_RANGE, "batch too wide: more than 65535 right-hand-side tiles");
    if (t_timer) t_timer->mark();
    SweepArgs a;
    a.arena = e->arena.p;
    a.T = e->T.p;
    a.Y = Y;
    a.X = X;
    a.V = static_cast<const float*>(e->V.p);
    a.term_val = static_cast<const int32_t*>(e->term_val.p);
    a.term_col = static_cast<const int32_t*>(e->term_col.p);
    a.n_terms = e->n_terms;
    a.n_ops = e->n_ops;
    a.rows = e->rows;
    a.ldx = lc.Bw;
    a.ldy = lc.Bw;
    a.Bt = lc.Bt;
    a.G = lc.G;
    a.t0 = 0;
    set_direct(e, a);
    const int TPB = 256;
    auto blocks_for = [&](int64_t items, int nt) -> int {
        int64_t b = (items + TPB - 1) / TPB;
        int64_t cap = std::max<int64_t>(1, (int64_t)e->sm_count * 32 / nt);  // grid-stride beyond this
        return (int)std::max<int64_t>(1, std::min(b, cap));
    };
    auto after = [&](bool mark = true) {
        ++launches;
        if (t_timer && mark) t_timer->mark();
    };
    {
        int64_t items = (e->rows + (e->direct_terms ? e->n_rule_terms : e->n_terms)) * (int64_t)lc.G;
        dim3 grid(blocks_for(items, lc.ntile), lc.ntile);
        k_prologue<S, VEC, GLOG><<<grid, TPB, 0, st>>>(a);
        after();
    }
    // ops of level k_ops (0: none) and emissions of level k_em (-1: none), tiles [t0, t0+nt).
    // ops_lo >= 0: only the ops slots [ops_lo, ops_hi) of level k_ops.  em_part >= 0: fold
    // only that source chunk of level k_em (index into ch_em / ch_seg), -2: nothing.
    // mark_end: record the timing mark after the last launch (one mark per launch slot).
    auto level = [&](int k_ops, int k_em, int t0, int nt, bool split, int64_t ops_lo = -1, int64_t ops_hi = -1,
                     int64_t em_part = -1, bool mark_end = true) {
        SweepArgs s = a;
        s.t0 = t0;
        LevelArgs L{};
        L.ops = static_cast<const int2*>(e->direct_terms ? e->ops_direct.p : e->ops.p);
        L.direct_ops = e->direct_terms;
        L.op_c = e->has_coeff ? static_cast<const float*>(e->op_c.p) : nullptr;
        L.em_src = static_cast<const int32_t*>(e->em_src.p);
        L.em_row = static_cast<const int32_t*>(e->em_row.p);
        L.seg_row = static_cast<const int32_t*>(e->seg_row.p);
        L.seg_start = static_cast<const int64_t*>(e->seg_start.p);
        const int slot = k_ops >= 1 ? k_ops : e->depth + 1;  // launch slot of this level launch
        int emit = lc.emit, chunk = lc.chunk, ops_cap = kOpsCtasPerSm[0];
        bool by_chunk = false;
        if (!lc.lv.empty() && slot < (int)lc.lv.size()) {
            const int v = (lc.lv[slot] & ~(GMR_LEVEL_PUSH | GMR_LEVEL_INTERLEAVE | GMR_LEVEL_STAGE)) % GMR_N_LEVEL_VARIANTS;
            emit = kEmitVariants[v % kNumEmitVariants].emit;
            chunk = kEmitVariants[v % kNumEmitVariants].chunk;
            ops_cap = kOpsCtasPerSm[(v / kNumEmitVariants) % 2];
            by_chunk = v >= 2 * kNumEmitVariants;
        }
        if (lc.variant == GMR_VARIANT_PLAIN) emit = GMR_EMIT_ATOMIC;
        // level k_em pushed its emissions in its own launch: nothing to fold
        if (k_em >= 1 && em_part == -1 && level_mode(e, lc, k_em) == kFoldPush) k_em = -1;
        if (em_part == -2) k_em = -1;
        // level k_em was interleaved: only its last source chunk is left to fold
        if (k_em >= 1 && em_part == -1 && level_mode(e, lc, k_em) == kFoldInterleave) {
            const int64_t r = interleave_chunks(e, k_em) - 1, nec = e->ch_off[k_em + 1] - e->ch_off[k_em];
            if (r < nec) em_part = e->ch_off[k_em] + r;
            else k_em = -1;
        }
        if (k_ops >= 1 && level_mode(e, lc, k_ops) == kFoldPush) {
            L.pe_off = static_cast<const int32_t*>(e->pe_off.p);
            L.pe_row = static_cast<const int32_t*>(e->pe_row.p);
            if (emit == GMR_EMIT_ROWS) emit = GMR_EMIT_SEGMENTED;  // the pushes are atomics into the same Y
        }
        if (k_em == 0 && e->direct_terms) {  // terminal emissions fold leaf(V, X) directly
            L.em_src = static_cast<const int32_t*>(e->em_tcode.p);
            L.direct = true;
            by_chunk = false;
        }
        if (chunk <= 0) chunk = 16;
        L.em_chunk = chunk;
        int64_t nops = 0, nem = 0, nseg = 0;
        if (k_ops >= 1) {
            L.op_first = ops_lo >= 0 ? ops_lo : e->lvl_off[k_ops - 1];
            nops = (ops_lo >= 0 ? ops_hi : e->lvl_off[k_ops]) - L.op_first;
        }
        if (k_em >= 0 && em_part >= 0) {  // one source chunk, from the chunked emission order
            L.em_src = static_cast<const int32_t*>(e->em_src_c.p);
            L.em_row = static_cast<const int32_t*>(e->em_row_c.p);
            L.seg_row = static_cast<const int32_t*>(e->seg_row_c.p);
            L.seg_start = static_cast<const int64_t*>(e->seg_start_c.p);
            L.em_first = e->ch_em[em_part];
            nem = e->ch_em[em_part + 1] - e->ch_em[em_part];
            L.seg_first = e->ch_seg[em_part];
            nseg = e->ch_seg[em_part + 1] - e->ch_seg[em_part];
            by_chunk = false;
        } else if (k_em >= 0) {
            L.em_first = e->em_off[k_em];
            nem = e->em_off[k_em + 1] - e->em_off[k_em];
            L.seg_first = e->seg_off[k_em];
            nseg = e->seg_off[k_em + 1] - e->seg_off[k_em];
        }
        auto em_items_seg = [&](int64_t ne) -> int64_t {  // the segmented fold, chunk 16
            if (GLOG == 0) return (ne + 1) / 2;
            return (ne + 15) / 16 * lc.G;
        };
        auto em_items = [&](int64_t ne, int64_t ns) -> int64_t {
            if (emit == GMR_EMIT_ATOMIC) return ne * lc.G;
            if (emit == GMR_EMIT_ROWS) return ns * lc.G;
            if (GLOG == 0) return (ne + 1) / 2;  // two warp-blocks per warp iteration
            return (ne + chunk - 1) / chunk * lc.G;
        };
        auto go = [&](const LevelArgs& base, int64_t no, int64_t ne, int64_t ns, bool mark) {
            LevelArgs M = base;
            M.n_ops = no;
            M.n_em = ne;
            M.n_seg = ns;
            mark = mark && mark_end;
            if (no == 0 && ne == 0) {
                if (t_timer && mark && !split) t_timer->mark();  // keep one timing slot per level launch
                return;
            }
            const int dirk = !M.direct_ops ? 0 : M.direct ? 2 : 1;
            if constexpr (GLOG >= 0 && VEC >= 4) {
                if (no > 0 && dirk == 0 && k_ops >= 1 && level_staged(e, lc, k_ops)) {
                    // staged rules; the launch's emissions use the segmented fold
                    const int64_t R = 2 * (256 >> GLOG);
                    const int eb = ne > 0 ? blocks_for(em_items_seg(ne), nt) : 0;
                    const int ob = (int)std::min<int64_t>((no + R - 1) / R, std::max(1, e->sm_count * ops_cap / nt));
                    M.em_blocks = eb;
                    M.em_chunk = 16;
                    M.stage_bytes = kStageBytes;
                    M.err = e->stage_err();
                    M.level = k_ops;
                    k_level_staged<S, VEC, GLOG><<<dim3(eb + ob, nt), 256, kStageBytes, st>>>(s, M);
                    after(mark);
                    return;
                }
            }
            int eb = ne > 0 ? blocks_for(em_items(ne, ns), nt) : 0;
            int ob = no > 0 ? std::min<int>(blocks_for((no * lc.G + 1) / 2, nt),
                                            std::max(1, e->sm_count * ops_cap / nt)) : 0;
            M.em_blocks = eb;
            dim3 grid(eb + ob, nt);
            if (dirk == 0) launch_level<S, VEC, GLOG, 0>(emit, grid, st, s, M);
            else if (dirk == 1) launch_level<S, VEC, GLOG, 1>(emit, grid, st, s, M);
            else launch_level<S, VEC, GLOG, 2>(emit, grid, st, s, M);
            after(mark);
        };
        if (split) {  // plain: emissions and ops in separate launches
            go(L, 0, nem, nseg, true);
            go(L, nops, 0, 0, true);
            return;
        }
        const int64_t nch = (by_chunk && e->chunked && k_em >= 0) ? e->ch_off[k_em + 1] - e->ch_off[k_em] : 0;
        if (nch < 2) {
            go(L, nops, nem, nseg, true);
            return;
        }
        // one launch per source chunk of level k_em; the first also evaluates level k_ops
        LevelArgs C = L;
        C.em_src = static_cast<const int32_t*>(e->em_src_c.p);
        C.em_row = static_cast<const int32_t*>(e->em_row_c.p);
        C.seg_row = static_cast<const int32_t*>(e->seg_row_c.p);
        C.seg_start = static_cast<const int64_t*>(e->seg_start_c.p);
        for (int64_t c = 0; c < nch; ++c) {
            const int64_t i = e->ch_off[k_em] + c;
            C.em_first = e->ch_em[i];
            C.seg_first = e->ch_seg[i];
            go(C, c == 0 ? nops : 0, e->ch_em[i + 1] - e->ch_em[i], e->ch_seg[i + 1] - e->ch_seg[i], c == nch - 1);
        }
    };
    const int D = e->depth;
    const bool staged = any_staged(e, lc) && !t_chain_no_status;
    if (staged) GMR_CUDA(cudaMemsetAsync(e->stage_err(), 0, 8, st));  // the staged waits' error words
    if (lc.variant == GMR_VARIANT_PLAIN) {
        level(0, 0, 0, lc.ntile, true);  // terminal emissions
        for (int k = 1; k <= D; ++k) {
            level(k, -1, 0, lc.ntile, true);
            level(0, k, 0, lc.ntile, true);
        }
    } else {
        const int K = lc.ntile > 1 ? std::min(lc.tile_levels, D) : 0;
        for (int t = 0; t < (K > 0 ? lc.ntile : 0); ++t)
            for (int k = 1; k <= K; ++k) level(k, k - 1, t, 1, false);
        for (int k = K + 1; k <= D; ++k) {
            if (level_mode(e, lc, k) != kFoldInterleave) {
                level(k, k - 1, 0, lc.ntile, false);
                continue;
            }
            // level k in source chunks: launch c evaluates chunk c and folds the
            // emissions of chunk c - 1, whose values the previous launch left in L2
            const int64_t base = e->lvl_off[k - 1], end = e->lvl_off[k], n_oc = interleave_chunks(e, k);
            const int64_t nec = e->ch_off[k + 1] - e->ch_off[k];
            for (int64_t c = 0; c < n_oc; ++c) {
                const int64_t lo = base + c * e->chunk_slots, hi = std::min(end, lo + e->chunk_slots);
                if (c == 0) level(k, k - 1, 0, lc.ntile, false, lo, hi, -1, n_oc == 1);
                else level(k, k, 0, lc.ntile, false, lo, hi, c - 1 < nec ? e->ch_off[k] + c - 1 : -2, c == n_oc - 1);
            }
        }
        level(0, D, 0, lc.ntile, false);
    }
    if (staged) GMR_CUDA(cudaMemcpyAsync(e->status_host, e->stage_err(), 8, cudaMemcpyDeviceToHost, st));
    GMR_CUDA(cudaGetLastError());
}

template <class S, int VEC, int GLOG, int EMIT>
static void launch_persistent_emit(gmr_engine* e, const Launch& lc, const SweepArgs& a, const LevelArgs& L0,
                                   const PersistArgs& P, cudaStream_t st) {
    auto kernel = k_persistent<S, VEC, GLOG, EMIT>;
    int per_sm = 0;
    GMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
    if (per_sm < 1) throw Error(GMR_ERR_STATE, "persistent kernel cannot be resident");
    const int grid = per_sm * e->sm_count;
    SweepArgs aa = a;
    LevelArgs ll = L0;
    PersistArgs pp = P;
    void* args[] = {&aa, &ll, &pp};
    GMR_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kernel), dim3(grid), dim3(256), args, 0, st));
    (void)lc;
}

template <class S, int VEC, int GLOG>
static void launch_persistent_t(gmr_engine* e, const Launch& lc, const void* X, void* Y, cudaStream_t st,
                                int64_t& launches) {
    if (t_timer) t_timer->mark();
    SweepArgs a;
    a.arena = e->arena.p;
    a.T = e->T.p;
    a.Y = Y;
    a.X = X;
    a.V = static_cast<const float*>(e->V.p);
    a.term_val = static_cast<const int32_t*>(e->term_val.p);
    a.term_col = static_cast<const int32_t*>(e->term_col.p);
    a.n_terms = e->n_terms;
    a.n_ops = e->n_ops;
    a.rows = e->rows;
    a.ldx = lc.Bw;
    a.ldy = lc.Bw;
    a.Bt = lc.Bt;
    a.G = lc.G;
    a.t0 = 0;
    LevelArgs L{};
    L.ops = static_cast<const int2*>(e->ops.p);
    L.op_c = e->has_coeff ? static_cast<const float*>(e->op_c.p) : nullptr;
    L.em_src = static_cast<const int32_t*>(e->em_src.p);
    L.em_row = static_cast<const int32_t*>(e->em_row.p);
    L.seg_row = static_cast<const int32_t*>(e->seg_row.p);
    L.seg_start = static_cast<const int64_t*>(e->seg_start.p);
    L.em_chunk = lc.chunk > 0 ? lc.chunk : 16;
    PersistArgs P;
    P.lvl_off = static_cast<const int64_t*>(e->d_lvl_off.p);
    P.em_off = static_cast<const int64_t*>(e->d_em_off.p);
    P.seg_off = static_cast<const int64_t*>(e->d_seg_off.p);
    P.depth = e->depth;
    P.bar = static_cast<unsigned*>(e->sync.p);
    P.err = reinterpret_cast<int*>(static_cast<unsigned char*>(e->sync.p) + 8);
    P.spin_limit = lc.spin_limit;
    GMR_CUDA(cudaMemsetAsync(e->sync.p, 0, 16, st));
    if (lc.emit == GMR_EMIT_ATOMIC) launch_persistent_emit<S, VEC, GLOG, GMR_EMIT_ATOMIC>(e, lc, a, L, P, st);
    else if (lc.emit == GMR_EMIT_ROWS) launch_persistent_emit<S, VEC, GLOG, GMR_EMIT_ROWS>(e, lc, a, L, P, st);
    else launch_persistent_emit<S, VEC, GLOG, GMR_EMIT_SEGMENTED>(e, lc, a, L, P, st);
    ++launches;
    if (t_timer) t_timer->mark();
    GMR_CUDA(cudaMemcpyAsync(e->status_host, P.err, 8, cudaMemcpyDeviceToHost, st));
}

template <class S>
static void launch_persistent_s(gmr_engine* e, const Launch& lc, const void* X, void* Y, cudaStream_t st,
                                int64_t& n) {
    if (lc.VEC == 4) {
        switch (lc.G) {
            case 1: return launch_persistent_t<S, 4, 0>(e, lc, X, Y, st, n);
            case 2: return launch_persistent_t<S, 4, 1>(e, lc, X, Y, st, n);
            case 4: return launch_persistent_t<S, 4, 2>(e, lc, X, Y, st, n);
            case 8: return launch_persistent_t<S, 4, 3>(e, lc, X, Y, st, n);
            case 16: return launch_persistent_t<S, 4, 4>(e, lc, X, Y, st, n);
            case 32: return launch_persistent_t<S, 4, 5>(e, lc, X, Y, st, n);
            default: return launch_persistent_t<S, 4, -1>(e, lc, X, Y, st, n);
        }
    }
    if constexpr (!std::is_same<S, SBool>::value) {
        if (lc.VEC == 8) {
            switch (lc.G) {
                case 1: return launch_persistent_t<S, 8, 0>(e, lc, X, Y, st, n);
                case 2: return launch_persistent_t<S, 8, 1>(e, lc, X, Y, st, n);
                case 4: return launch_persistent_t<S, 8, 2>(e, lc, X, Y, st, n);
                case 8: return launch_persistent_t<S, 8, 3>(e, lc, X, Y, st, n);
                default: return launch_persistent_t<S, 8, 4>(e, lc, X, Y, st, n);
            }
        }
    }
    if (lc.VEC == 2 && lc.G == 1) return launch_persistent_t<S, 2, 0>(e, lc, X, Y, st, n);
    if (lc.VEC == 1 && lc.G == 1) return launch_persistent_t<S, 1, 0>(e, lc, X, Y, st, n);
    if (lc.VEC == 2) return launch_persistent_t<S, 2, -1>(e, lc, X, Y, st, n);
    return launch_persistent_t<S, 1, -1>(e, lc, X, Y, st, n);
}

static void launch_persistent(gmr_engine* e, const Launch& lc, const void* X, void* Y, cudaStream_t st,
                              int64_t& n) {
    if (lc.semiring == GMR_PLUS_TIMES) launch_persistent_s<SPlus>(e, lc, X, Y, st, n);
    else if (lc.semiring == GMR_BOOLEAN) launch_persistent_s<SBool>(e, lc, X, Y, st, n);
    else launch_persistent_s<STrop>(e, lc, X, Y, st, n);
}

template <class S>
static void launch_chain_s(gmr_engine* e, const Launch& lc, const void* X, void* Y, cudaStream_t st,
                           int64_t& n) {
    if (lc.VEC == 4) {
        switch (lc.G) {
            case 1: return launch_chain_t<S, 4, 0>(e, lc, X, Y, st, n);
            case 2: return launch_chain_t<S, 4, 1>(e, lc, X, Y, st, n);
            case 4: return launch_chain_t<S, 4, 2>(e, lc, X, Y, st, n);
            case 8: return launch_chain_t<S, 4, 3>(e, lc, X, Y, st, n);
            case 16: return launch_chain_t<S, 4, 4>(e, lc, X, Y, st, n);
            case 32: return launch_chain_t<S, 4, 5>(e, lc, X, Y, st, n);
            default: return launch_chain_t<S, 4, -1>(e, lc, X, Y, st, n);
        }
    }
    if constexpr (!std::is_same<S, SBool>::value) {
        if (lc.VEC == 8) {
            switch (lc.G) {
                case 1: return launch_chain_t<S, 8, 0>(e, lc, X, Y, st, n);
                case 2: return launch_chain_t<S, 8, 1>(e, lc, X, Y, st, n);
                case 4: return launch_chain_t<S, 8, 2>(e, lc, X, Y, st, n);
                case 8: return launch_chain_t<S, 8, 3>(e, lc, X, Y, st, n);
                default: return launch_chain_t<S, 8, 4>(e, lc, X, Y, st, n);
            }
        }
    }
    if (lc.VEC == 2 && lc.G == 1) return launch_chain_t<S, 2, 0>(e, lc, X, Y, st, n);
    if (lc.VEC == 1 && lc.G == 1) return launch_chain_t<S, 1, 0>(e, lc, X, Y, st, n);
    if (lc.VEC == 2) return launch_chain_t<S, 2, -1>(e, lc, X, Y, st, n);
    return launch_chain_t<S, 1, -1>(e, lc, X, Y, st, n);
}

static void launch_chain(gmr_engine* e, const Launch& lc, const void* X, void* Y, cudaStream_t st, int64_t& n) {
    if (lc.semiring == GMR_PLUS_TIMES) launch_chain_s<SPlus>(e, lc, X, Y, st, n);
    else if (lc.semiring == GMR_BOOLEAN) launch_chain_s<SBool>(e, lc, X, Y, st, n);
    else launch_chain_s<STrop>(e, lc, X, Y, st, n);
}

// Default tile width: the whole batch (measured: every extra tile pass costs
// about as much as a full pass, the sweep is latency-bound per pass), split
// only so that a tile is at most 128 words (32 lanes of 16-byte accesses).
static int auto_tile(gmr_engine*, int Bw) {
    int bt = Bw;
    while (bt > 128 && bt % 2 == 0) bt /= 2;
    return bt;
}

// max_vec: the widest lane access a caller's kernels instantiate (the pack
// and the left product stop at 4 words).
static Launch resolve_launch(gmr_engine* e, int semiring, int B, const void* X, void* Y, const gmr_config* cfg,
                             int max_vec = 8) {
    Launch lc{};
    lc.semiring = semiring;
    lc.B = B;
    lc.Bw = words_per_slot(semiring, B);
    const int asked = cfg ? cfg->variant : GMR_VARIANT_AUTO;
    lc.variant = asked == GMR_VARIANT_AUTO ? GMR_VARIANT_GRAPH : asked;
    // the persistent kernel reads terminals from T only: with direct terminals
    // (T holds just the zero terminal) the per-level graph runs instead
    if (lc.variant == GMR_VARIANT_PERSISTENT && e->direct_terms) lc.variant = GMR_VARIANT_GRAPH;
    lc.spin_limit = cfg && cfg->spin_limit > 0 ? (unsigned long long)cfg->spin_limit : 20000000ull;
    if (asked == GMR_VARIANT_AUTO && !(cfg && cfg->emit_mode)) {
        auto it = e->level_variants.find({semiring, B});
        if (it != e->level_variants.end()) lc.lv = it->second;
    }
    lc.emit = cfg && cfg->emit_mode ? cfg->emit_mode : GMR_EMIT_SEGMENTED;
    if (lc.variant == GMR_VARIANT_PLAIN) lc.emit = GMR_EMIT_ATOMIC;
    lc.push_mode = cfg ? cfg->push : GMR_PUSH_AUTO;
    if (lc.push_mode < GMR_PUSH_AUTO || lc.push_mode > GMR_PUSH_INTERLEAVE) throw Error(GMR_ERR_ARG, "unknown push mode");
    lc.chunk = cfg && cfg->ops_per_cta > 0 ? cfg->ops_per_cta : 16;
    int bt = cfg && cfg->vec_tile > 0 ? cfg->vec_tile : auto_tile(e, lc.Bw);
    if (bt > lc.Bw || lc.Bw % bt != 0) bt = lc.Bw;  // tiles must divide the batch
    if (lc.variant == GMR_VARIANT_PERSISTENT) bt = lc.Bw;  // one tile: the whole batch in one launch
    lc.Bt = bt;
    lc.ntile = lc.Bw / bt;
    lc.tile_levels = cfg && cfg->tile_levels > 0 ? cfg->tile_levels : e->depth;
    if (!cfg || cfg->tile_levels <= 0) {
        // tile the levels whose values overflow the budget at full width
        int K = 0;
        for (int k = 1; k <= e->depth; ++k)
            if ((e->lvl_off[k] - e->lvl_off[k - 1]) * (int64_t)lc.Bw * 4 > (16ll << 20)) K = k;
        lc.tile_levels = std::max(K, 1);
    }
    auto aligned = [&](size_t al) { return ((uintptr_t)X % al == 0) && ((uintptr_t)Y % al == 0); };
    int lane_bytes = cfg && cfg->lane_bytes ? cfg->lane_bytes : e->lane_bytes;
    if (lane_bytes != 0 && lane_bytes != 16 && lane_bytes != 32) throw Error(GMR_ERR_ARG, "lane_bytes must be 0, 16 or 32");
    // 8 words per lane: fp32 / int32 tiles of 8..128 words (powers of two), 32-byte aligned X and Y
    const bool v8_ok = max_vec >= 8 && semiring != GMR_BOOLEAN && lc.Bt % 8 == 0 && lc.Bw % 8 == 0 &&
                       lc.Bt <= 128 && (lc.Bt & (lc.Bt - 1)) == 0 && aligned(32);
    // measured on the 200k x 10k grammar: 32-byte lanes win for (+,x) tiles of
    // >= 32 words (B = 32 / 64 / 128), lose at 8 words and for (min,+)
    if (lane_bytes == 0) lane_bytes = semiring == GMR_PLUS_TIMES && lc.Bt >= 32 ? 32 : 16;
    if (lane_bytes == 32 && v8_ok) lc.VEC = 8;
    else if (lc.Bt % 4 == 0 && lc.Bw % 4 == 0 && aligned(16)) lc.VEC = 4;
    else if (lc.Bt % 2 == 0 && lc.Bw % 2 == 0 && aligned(8)) lc.VEC = 2;
    else lc.VEC = 1;
    lc.G = lc.Bt / lc.VEC;
    return lc;
}

// Grows the value arena and terminal table; cached graphs bake these
// addresses in, so any reallocation drops them (after the device is idle).
static void ensure_scratch(gmr_engine* e, int Bw) {
    const size_t na = (size_t)std::max<int64_t>(e->n_ops, 1) * Bw * 4;
    const size_t nt = (size_t)std::max<int64_t>(e->n_terms, 1) * Bw * 4;
    if (na <= e->arena.bytes && nt <= e->T.bytes) return;
    GMR_CUDA(cudaDeviceSynchronize());
    for (auto& g : e->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    e->graphs.clear();
    e->arena.ensure(na);
    e->T.ensure(nt);
}

static void multiply_device(gmr_engine* e, int semiring, const void* X, void* Y, int B, const gmr_config* cfg,
                            cudaStream_t st, bool eager = false) {
    if (semiring < 0 || semiring > 2) throw Error(GMR_ERR_ARG, "unknown semiring");
    if (B < 1) throw Error(GMR_ERR_ARG, "B must be >= 1");
    if ((!X && e->cols > 0) || (!Y && e->rows > 0)) throw Error(GMR_ERR_ARG, "null X or Y");
    if (((uintptr_t)X | (uintptr_t)Y) % 4 != 0) throw Error(GMR_ERR_ARG, "X and Y must be 4-byte aligned");
    Launch lc = resolve_launch(e, semiring, B, X, Y, cfg);
    if (eager && lc.variant == GMR_VARIANT_GRAPH) lc.variant = GMR_VARIANT_FUSED;
    ensure_scratch(e, lc.Bw);
    int64_t launches = 0;
    if (lc.variant == GMR_VARIANT_GRAPH) {
        GraphEntry* hit = nullptr;
        for (auto& g : e->graphs)
            if (g.exec && !g.fixpoint && g.lc == lc && g.X == X && g.Y == Y) hit = &g;
        if (!hit) {
            if (e->graphs.size() >= 8) {
                cudaGraphExecDestroy(e->graphs.front().exec);
                e->graphs.erase(e->graphs.begin());
            }
            cudaGraph_t graph = nullptr;
            GMR_CUDA(cudaStreamBeginCapture(e->own_stream, cudaStreamCaptureModeThreadLocal));
            int64_t n = 0;
            try {
                launch_chain(e, lc, X, Y, e->own_stream, n);
            } catch (...) {
                cudaStreamEndCapture(e->own_stream, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            GMR_CUDA(cudaStreamEndCapture(e->own_stream, &graph));
            GraphEntry ge;
            cudaError_t ie = cudaGraphInstantiate(&ge.exec, graph, 0);
            cudaGraphDestroy(graph);
            GMR_CUDA(ie);
            ge.lc = lc;
            ge.X = X;
            ge.Y = Y;
            ge.launches = n;
            e->graphs.push_back(ge);
            hit = &e->graphs.back();
        }
        GMR_CUDA(cudaGraphLaunch(hit->exec, st));
        launches = hit->launches;
    } else if (lc.variant == GMR_VARIANT_PERSISTENT) {
        e->last_persistent = true;
        launch_persistent(e, lc, X, Y, st, launches);
    } else {
        launch_chain(e, lc, X, Y, st, launches);
    }
    if (any_staged(e, lc)) e->last_persistent = true;
    e->last_launches = launches;
}

// ------------------------------------------------------------------ NVML (optional)
struct Nvml {
    void* h = nullptr;
    int (*init)() = nullptr;
    int (*shutdown)() = nullptr;
    int (*by_index)(unsigned, void**) = nullptr;
    int (*energy)(void*, unsigned long long*) = nullptr;
    bool load() {
        h = dlopen("libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) return false;
        init = (int (*)())dlsym(h, "nvmlInit_v2");
        shutdown = (int (*)())dlsym(h, "nvmlShutdown");
        by_index = (int (*)(unsigned, void**))dlsym(h, "nvmlDeviceGetHandleByIndex_v2");
        energy = (int (*)(void*, unsigned long long*))dlsym(h, "nvmlDeviceGetTotalEnergyConsumption");
        return init && shutdown && by_index && energy;
    }
    ~Nvml() {
        if (h) dlclose(h);
    }
};

}  // namespace gmr

using namespace gmr;

// The chunked emission order (see gmr_engine::ch_*), built when some level
// has more than one source chunk: a stable counting sort of each level's
// (row, source)-ordered emissions by source chunk, then row segments per chunk.
// The chunk size is kChunkSlots unless the environment variable
// GMR_CHUNK_SLOTS (read when the engine is created) sets another one.
static void build_chunked_emissions(const gmr_plan& p, gmr_engine& e) {
    const int D = p.depth;
    int64_t kChunkSlots = gmr::kChunkSlots;
    if (const char* env = std::getenv("GMR_CHUNK_SLOTS")) {
        long long v = std::atoll(env);
        if (v >= 1) kChunkSlots = v;
    }
    e.chunk_slots = kChunkSlots;
    bool any = false;
    for (int k = 0; k <= D && !any; ++k) {
        const int64_t width = k == 0 ? p.n_terms() : p.lvl_off[k] - p.lvl_off[k - 1];
        any = width > kChunkSlots && p.em_off[k + 1] > p.em_off[k];
    }
    if (!any) return;
    const int64_t E = (int64_t)p.em_src.size();
    std::vector<int32_t> src(E), row(E), srow;
    std::vector<int64_t> sstart;
    e.ch_off.assign(D + 2, 0);
    e.ch_em.clear();
    e.ch_seg.clear();
    for (int k = 0; k <= D; ++k) {
        e.ch_off[k] = (int64_t)e.ch_em.size();
        const int64_t lo = p.em_off[k], hi = p.em_off[k + 1];
        if (hi == lo) continue;
        const int64_t base = k == 0 ? 0 : p.lvl_off[k - 1];
        auto chunk_of = [&](int32_t c) { return (c >= 0 ? (int64_t)c - base : -(int64_t)c - 1) / kChunkSlots; };
        int64_t nc = 0;
        for (int64_t j = lo; j < hi; ++j) nc = std::max(nc, chunk_of(p.em_src[j]) + 1);
        std::vector<int64_t> pos(nc + 1, 0);
        for (int64_t j = lo; j < hi; ++j) pos[chunk_of(p.em_src[j]) + 1]++;
        for (int64_t c = 0; c < nc; ++c) pos[c + 1] += pos[c];
        std::vector<int64_t> start(pos.begin(), pos.end());
        for (int64_t j = lo; j < hi; ++j) {
            const int64_t d = lo + pos[chunk_of(p.em_src[j])]++;
            src[d] = p.em_src[j];
            row[d] = p.em_row[j];
        }
        for (int64_t c = 0; c < nc; ++c) {
            e.ch_em.push_back(lo + start[c]);
            e.ch_seg.push_back((int64_t)srow.size());
            for (int64_t j = lo + start[c]; j < lo + start[c + 1]; ++j)
                if (j == lo + start[c] || row[j] != row[j - 1]) {
                    srow.push_back(row[j]);
                    sstart.push_back(j);
                }
        }
    }
    e.ch_off[D + 1] = (int64_t)e.ch_em.size();
    e.ch_em.push_back(E);
    e.ch_seg.push_back((int64_t)srow.size());
    sstart.push_back(E);
    upload(src, e.em_src_c);
    upload(row, e.em_row_c);
    upload(srow, e.seg_row_c);
    upload(sstart, e.seg_start_c);
    e.chunked = true;
}

// Direct terminal emissions pay off when the terminal table is much larger
// than X (graphs: one terminal per (weight, column)), so that gathering
// X[col] (small, L2-resident) beats gathering T[q]: terminal emissions and
// rule children then evaluate leaf(V, X[col]) in place and the prologue no
// longer fills T.  GMR_DIRECT_TERMS=0 / 1 forces the choice.
static void build_direct_terms(const gmr_plan& p, gmr_engine& e) {
    const int64_t n_te = p.em_off.size() > 1 ? p.em_off[1] - p.em_off[0] : 0;
    bool on = n_te > 0 && p.n_terms() > 4 * (int64_t)p.cols;
    if (const char* f = std::getenv("GMR_DIRECT_TERMS")) on = n_te > 0 && std::atoi(f) != 0;
    if ((int64_t)p.V.size() * p.cols > INT32_MAX) on = false;  // codes must fit int32
    e.direct_terms = on;
    if (!on) return;
    std::vector<int32_t> code((size_t)n_te);
    for (int64_t i = 0; i < n_te; ++i) {
        const int64_t q = -(int64_t)p.em_src[p.em_off[0] + i] - 1;  // >= 1: terminal emissions
        code[i] = (int32_t)((int64_t)p.term_val[q - 1] * p.cols + p.term_col[q - 1]);
    }
    upload(code, e.em_tcode);
    // rule children: terminals as codes too, so that T keeps only the zero
    // terminal T[0] (still read by the warp fold's idle lanes)
    auto enc = [&](int32_t c) -> int32_t {
        if (c >= -1) return c;
        const int64_t q = -(int64_t)c - 1;
        return (int32_t)(-((int64_t)p.term_val[q - 1] * p.cols + p.term_col[q - 1]) - 2);
    };
    std::vector<int2> ops((size_t)p.n_ops());
    for (int64_t i = 0; i < p.n_ops(); ++i) ops[i] = make_int2(enc(p.op_l[i]), enc(p.op_r[i]));
    upload(ops, e.ops_direct);
    std::vector<int32_t> list{0};
    e.n_rule_terms = 1;
    upload(list, e.rule_terms);
}

// Push lists (gmr_engine::pe_*): a counting sort of the emissions of levels
// 1..depth by source slot.  The plan orders a level's emissions by (row,
// source), so each slot's rows come out ascending.  Offsets are int32: a
// plan with 2^31 or more such emissions gets no push lists.
static void build_push_lists(const gmr_plan& p, gmr_engine& e) {
    const int D = p.depth;
    e.push_ok.assign(D + 2, 0);
    if (D < 1) return;
    const int64_t E0 = p.em_off[1], E1 = p.em_off[D + 1];
    if (E1 - E0 >= (int64_t)INT32_MAX || p.n_ops() >= (int64_t)INT32_MAX) return;
    std::vector<int32_t> off((size_t)p.n_ops() + 1, 0);
    for (int k = 1; k <= D; ++k) {
        bool ok = true;
        for (int64_t j = p.em_off[k]; j < p.em_off[k + 1] && ok; ++j)
            ok = p.em_src[j] >= p.lvl_off[k - 1] && p.em_src[j] < p.lvl_off[k];
        e.push_ok[k] = ok;
        if (!ok) continue;
        for (int64_t j = p.em_off[k]; j < p.em_off[k + 1]; ++j) off[(size_t)p.em_src[j] + 1]++;
    }
    for (size_t s = 0; s + 1 < off.size(); ++s) off[s + 1] += off[s];
    std::vector<int32_t> row((size_t)std::max<int32_t>(off.back(), 1)), fill(off.begin(), off.end() - 1);
    for (int k = 1; k <= D; ++k) {
        if (!e.push_ok[k]) continue;
        for (int64_t j = p.em_off[k]; j < p.em_off[k + 1]; ++j) row[(size_t)fill[(size_t)p.em_src[j]]++] = p.em_row[j];
    }
    upload(off, e.pe_off);
    upload(row, e.pe_row);
}

extern "C" int gmr_engine_create(const gmr_plan* p, int device, gmr_engine** out) {
    return guarded([&] {
        if (!p || !out) throw Error(GMR_ERR_ARG, "null argument");
        validate_plan(*p);
        DeviceGuard dg(device);
        auto e = std::make_unique<gmr_engine>();
        e->device = device;
        e->rows = p->rows;
        e->cols = p->cols;
        e->depth = p->depth;
        e->n_ops = p->n_ops();
        e->n_terms = p->n_terms();
        e->n_em = (int64_t)p->em_src.size();
        e->has_coeff = p->has_coeff();
        e->lvl_off = p->lvl_off;
        e->em_off = p->em_off;
        e->seg_off = p->seg_off;
        try {
            {
                std::vector<int2> ops((size_t)p->n_ops());
                for (int64_t i = 0; i < p->n_ops(); ++i) ops[i] = make_int2(p->op_l[i], p->op_r[i]);
                upload(ops, e->ops);
            }
            if (e->has_coeff) upload(p->op_c, e->op_c);
            upload(p->em_src, e->em_src);
            upload(p->em_row, e->em_row);
            upload(p->seg_row, e->seg_row);
            upload(p->seg_start, e->seg_start);
            upload(p->term_val, e->term_val);
            upload(p->lvl_off, e->d_lvl_off);
            upload(p->em_off, e->d_em_off);
            upload(p->seg_off, e->d_seg_off);
            e->sync.ensure(64);
            GMR_CUDA(cudaMemset(e->sync.p, 0, 64));
            build_chunked_emissions(*p, *e);
            GMR_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&e->status_host), 16, cudaHostAllocDefault));
            std::memset(e->status_host, 0, 16);
            upload(p->term_col, e->term_col);
            upload(p->V, e->V);
            build_direct_terms(*p, *e);
            if (const char* f = std::getenv("GMR_LANE_BYTES")) {
                const int lb = std::atoi(f);
                if (lb == 16 || lb == 32) e->lane_bytes = lb;
            }
            build_push_lists(*p, *e);
            GMR_CUDA(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
            GMR_CUDA(cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, device));
        } catch (...) {
            for (auto* b : e->schedule_bufs()) b->release();
            if (e->own_stream) cudaStreamDestroy(e->own_stream);
            if (e->status_host) cudaFreeHost(e->status_host);
            throw;
        }
        *out = e.release();
    });
}

extern "C" int gmr_engine_multiply(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                                   const gmr_config* cfg, void* stream) {
    return guarded([&] {
        if (!e) throw Error(GMR_ERR_ARG, "null engine");
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        multiply_device(e, semiring, dX, dY, B, cfg, static_cast<cudaStream_t>(stream));
    });
}

extern "C" int gmr_engine_multiply_host(gmr_engine* e, int semiring, const void* hX, void* hY, int B,
                                        const gmr_config* cfg) {
    return guarded([&] {
        if (!e) throw Error(GMR_ERR_ARG, "null engine");
        if (B < 1) throw Error(GMR_ERR_ARG, "B must be >= 1");
        if ((!hX && e->cols > 0) || (!hY && e->rows > 0)) throw Error(GMR_ERR_ARG, "null X or Y");
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        size_t xb = (size_t)e->cols * words_per_slot(semiring, B) * 4;
        size_t yb = (size_t)e->rows * words_per_slot(semiring, B) * 4;
        e->hX.ensure(xb);
        e->hY.ensure(yb);
        cudaStream_t st = e->own_stream;
        if (xb) GMR_CUDA(cudaMemcpyAsync(e->hX.p, hX, xb, cudaMemcpyHostToDevice, st));
        e->last_persistent = false;
        multiply_device(e, semiring, e->hX.p, e->hY.p, B, cfg, st);
        if (yb) GMR_CUDA(cudaMemcpyAsync(hY, e->hY.p, yb, cudaMemcpyDeviceToHost, st));
        GMR_CUDA(cudaStreamSynchronize(st));
        if (e->last_persistent && e->status_host[0] != 0)
            throw Error(GMR_ERR_TIMEOUT, "a bounded device-side wait gave up at phase " +
                                             std::to_string(e->status_host[1]) + "; Y is not valid");
    });
}

extern "C" int gmr_engine_multiply_host_many(gmr_engine* e, int semiring, const void* const* hX, void* const* hY,
                                             int n, int B, const gmr_config* cfg) {
    return guarded([&] {
        if (!e || (n > 0 && (!hX || !hY))) throw Error(GMR_ERR_ARG, "null argument");
        if (B < 1 || n < 0) throw Error(GMR_ERR_ARG, "bad B or n");
        for (int i = 0; i < n; ++i)
            if ((!hX[i] && e->cols > 0) || (!hY[i] && e->rows > 0)) throw Error(GMR_ERR_ARG, "null X or Y");
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        const size_t xb = (size_t)e->cols * words_per_slot(semiring, B) * 4;
        const size_t yb = (size_t)e->rows * words_per_slot(semiring, B) * 4;
        e->hX.ensure(xb);
        e->hY.ensure(yb);
        e->hX2.ensure(xb);
        e->hY2.ensure(yb);
        if (!e->copy_in) GMR_CUDA(cudaStreamCreateWithFlags(&e->copy_in, cudaStreamNonBlocking));
        if (!e->copy_out) GMR_CUDA(cudaStreamCreateWithFlags(&e->copy_out, cudaStreamNonBlocking));
        for (auto& ev : e->pipe_ev)
            if (!ev) GMR_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        void* dx[2] = {e->hX.p, e->hX2.p};
        void* dy[2] = {e->hY.p, e->hY2.p};
        cudaStream_t st = e->own_stream;
        // multiply i runs in staging slot i % 2: its X copy overlaps multiply
        // i - 1, its Y copy overlaps multiply i + 1
        for (int i = 0; i < n; ++i) {
            const int k = i & 1;
            cudaEvent_t x_in = e->pipe_ev[3 * k], done = e->pipe_ev[3 * k + 1], y_out = e->pipe_ev[3 * k + 2];
            if (i >= 2) GMR_CUDA(cudaStreamWaitEvent(e->copy_in, done, 0));
            if (xb) GMR_CUDA(cudaMemcpyAsync(dx[k], hX[i], xb, cudaMemcpyHostToDevice, e->copy_in));
            GMR_CUDA(cudaEventRecord(x_in, e->copy_in));
            GMR_CUDA(cudaStreamWaitEvent(st, x_in, 0));
            if (i >= 2) GMR_CUDA(cudaStreamWaitEvent(st, y_out, 0));
            e->last_persistent = false;
            multiply_device(e, semiring, dx[k], dy[k], B, cfg, st);
            GMR_CUDA(cudaEventRecord(done, st));
            GMR_CUDA(cudaStreamWaitEvent(e->copy_out, done, 0));
            if (yb) GMR_CUDA(cudaMemcpyAsync(hY[i], dy[k], yb, cudaMemcpyDeviceToHost, e->copy_out));
            GMR_CUDA(cudaEventRecord(y_out, e->copy_out));
        }
        GMR_CUDA(cudaStreamSynchronize(e->copy_out));
        GMR_CUDA(cudaStreamSynchronize(st));
        if (e->last_persistent && e->status_host[0] != 0)
            throw Error(GMR_ERR_TIMEOUT, "a bounded device-side wait gave up at phase " +
                                             std::to_string(e->status_host[1]) + "; Y is not valid");
    });
}

extern "C" int gmr_engine_time_launches(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                                        const gmr_config* cfg, void* stream, float* ms, int cap, int* n) {
    return guarded([&] {
        if (!e || !ms || !n) throw Error(GMR_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        gmr_config c = cfg ? *cfg : gmr_config{};
        LaunchTimer timer;
        timer.st = static_cast<cudaStream_t>(stream);
        t_timer = &timer;
        try {
            multiply_device(e, semiring, dX, dY, B, &c, timer.st, /*eager=*/true);
        } catch (...) {
            t_timer = nullptr;
            throw;
        }
        t_timer = nullptr;
        GMR_CUDA(cudaStreamSynchronize(timer.st));
        int m = (int)timer.ev.size() - 1;
        if (m > cap) throw Error(GMR_ERR_RANGE, "need room for " + std::to_string(m) + " launch times");
        for (int i = 0; i < m; ++i) GMR_CUDA(cudaEventElapsedTime(&ms[i], timer.ev[i], timer.ev[i + 1]));
        *n = m;
    });
}

extern "C" int gmr_engine_set_level_variants(gmr_engine* e, int semiring, int B, const uint8_t* v, int n) {
    return guarded([&] {
        if (!e) throw Error(GMR_ERR_ARG, "null engine");
        std::lock_guard<std::mutex> lk(e->mu);
        if (!v || n <= 0) {
            e->level_variants.erase({semiring, B});
            return;
        }
        if (n != e->depth + 2) throw Error(GMR_ERR_ARG, "need depth + 2 = " + std::to_string(e->depth + 2) + " entries");
        for (int i = 0; i < n; ++i) {
            if ((v[i] & ~(GMR_LEVEL_PUSH | GMR_LEVEL_INTERLEAVE | GMR_LEVEL_STAGE)) >= GMR_N_LEVEL_VARIANTS)
                throw Error(GMR_ERR_ARG, "variant index out of range");
            if ((v[i] & GMR_LEVEL_PUSH) && (v[i] & GMR_LEVEL_INTERLEAVE))
                throw Error(GMR_ERR_ARG, "a level cannot both push and interleave");
        }
        e->level_variants[{semiring, B}] = std::vector<uint8_t>(v, v + n);
    });
}

extern "C" int gmr_engine_get_level_variants(const gmr_engine* e, int semiring, int B, uint8_t* v, int cap,
                                             int* n) {
    return guarded([&] {
        if (!e || !n) throw Error(GMR_ERR_ARG, "null argument");
        auto* me = const_cast<gmr_engine*>(e);
        std::lock_guard<std::mutex> lk(me->mu);
        auto it = e->level_variants.find({semiring, B});
        if (it == e->level_variants.end()) {
            *n = 0;
            return;
        }
        *n = (int)it->second.size();
        if (v) {
            if (cap < *n) throw Error(GMR_ERR_RANGE, "buffer too small");
            std::copy(it->second.begin(), it->second.end(), v);
        }
    });
}

extern "C" int gmr_engine_autotune_energy(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                                          void* stream, int reps, float tolerance, float* ms, int cap);

extern "C" int gmr_engine_autotune(gmr_engine* e, int semiring, const void* dX, void* dY, int B, void* stream,
                                   int reps, float* ms, int cap) {
    return gmr_engine_autotune_energy(e, semiring, dX, dY, B, stream, reps, 0.0f, ms, cap);
}

// Source-chunked variants (v >= 10) fold a level's emissions one L2-sized
// chunk of sources at a time, so the gathered values come from L2 instead of
// HBM: the same work with fewer DRAM bytes, hence less energy.  With
// tolerance > 0 a launch takes the chunked twin of its fastest variant when
// that is at most (1 + tolerance) times slower.
extern "C" int gmr_engine_autotune_energy(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                                          void* stream, int reps, float tolerance, float* ms, int cap) {
    return guarded([&] {
        if (tolerance < 0.0f || !(tolerance < 1.0f)) throw Error(GMR_ERR_ARG, "tolerance must be in [0, 1)");
        if (!e) throw Error(GMR_ERR_ARG, "null engine");
        const int nl = e->depth + 2, nv = GMR_N_LEVEL_VARIANTS;
        if (ms && cap < nl * nv) throw Error(GMR_ERR_RANGE, "need room for (depth + 2) x variants times");
        if (reps < 1) reps = 3;
        std::vector<float> med((size_t)nl * nv, 0.f);
        std::vector<uint8_t> uni(nl);
        std::vector<float> buf((size_t)nl + 8);
        for (int v = 0; v < nv; ++v) {
            std::fill(uni.begin(), uni.end(), (uint8_t)v);
            if (gmr_engine_set_level_variants(e, semiring, B, uni.data(), nl) != GMR_OK) throw Error(GMR_ERR_ARG, gmr_last_error());
            std::vector<std::vector<float>> runs;
            for (int r = 0; r < reps; ++r) {
                int n = 0;
                gmr_config c{};
                int rc = gmr_engine_time_launches(e, semiring, dX, dY, B, &c, stream, buf.data(), (int)buf.size(), &n);
                if (rc != GMR_OK) throw Error(rc, gmr_last_error());
                if (n != nl) throw Error(GMR_ERR_STATE, "unexpected launch count " + std::to_string(n));
                runs.emplace_back(buf.begin(), buf.begin() + n);
            }
            for (int l = 0; l < nl; ++l) {
                std::vector<float> xs;
                for (auto& r : runs) xs.push_back(r[l]);
                std::nth_element(xs.begin(), xs.begin() + xs.size() / 2, xs.end());
                med[(size_t)l * nv + v] = xs[xs.size() / 2];
            }
        }
        std::vector<uint8_t> best(nl, 0);
        for (int l = 0; l < nl; ++l) {
            int b = 0;
            for (int v = 1; v < nv; ++v)
                if (med[(size_t)l * nv + v] < med[(size_t)l * nv + b]) b = v;
            const int twin = b + 10;  // v = emit + 5 grid + 10 chunked
            if (tolerance > 0.0f && b < 10 && med[(size_t)l * nv + twin] <= med[(size_t)l * nv + b] * (1.0f + tolerance))
                b = twin;
            best[l] = (uint8_t)b;
        }
        // How each level's emissions reach Y: pull, push or interleave.  Slot k's
        // time depends on the modes of levels k-1 (what is left to fold) and k
        // (what its own launches do), slot depth+1's on level depth's.  Nine
        // tables, mode a on odd levels and b on even ones for every ordered
        // pair (a, b), time every slot under every pair of neighbouring modes;
        // a pass over the levels then picks the cheapest chain of modes.
        const int D = e->depth;
        const Launch lc0 = resolve_launch(e, semiring, B, dX, dY, nullptr);
        auto allowed = [&](int k, int m) {
            if (m == kFoldPull) return true;
            return m == kFoldPush ? can_push(e, k) : can_interleave(e, lc0, k);
        };
        bool any_mode = false;
        for (int k = 1; k <= D; ++k) any_mode |= allowed(k, kFoldPush) || allowed(k, kFoldInterleave);
        auto slot_times = [&](const std::vector<uint8_t>& table) {
            if (gmr_engine_set_level_variants(e, semiring, B, table.data(), nl) != GMR_OK)
                throw Error(GMR_ERR_ARG, gmr_last_error());
            std::vector<std::vector<float>> runs;
            for (int r = 0; r < reps; ++r) {
                int n = 0;
                gmr_config c{};
                int rc = gmr_engine_time_launches(e, semiring, dX, dY, B, &c, stream, buf.data(), (int)buf.size(), &n);
                if (rc != GMR_OK) throw Error(rc, gmr_last_error());
                if (n != nl) throw Error(GMR_ERR_STATE, "unexpected launch count " + std::to_string(n));
                runs.emplace_back(buf.begin(), buf.begin() + n);
            }
            std::vector<float> out(nl);
            for (int l = 0; l < nl; ++l) {
                std::vector<float> xs;
                for (auto& r : runs) xs.push_back(r[l]);
                std::nth_element(xs.begin(), xs.begin() + xs.size() / 2, xs.end());
                out[l] = xs[xs.size() / 2];
            }
            return out;
        };
        if (any_mode) {
            const uint8_t flag[3] = {0, GMR_LEVEL_PUSH, GMR_LEVEL_INTERLEAVE};
            const float kUnset = -1.0f;
            // cost[k][3 * m_prev + m]: slot k with level k-1 in m_prev and level k in m
            std::vector<std::array<float, 9>> cost(nl);
            for (auto& c : cost) c.fill(kUnset);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    std::vector<uint8_t> t = best;
                    std::vector<int> eff(D + 2, kFoldPull);
                    for (int k = 1; k <= D; ++k) {
                        const int m = (k & 1) ? a : b;
                        eff[k] = allowed(k, m) ? m : kFoldPull;
                        t[k] |= flag[eff[k]];
                    }
                    const std::vector<float> tt = slot_times(t);
                    for (int k = 1; k <= D + 1; ++k) {
                        const int m = k <= D ? eff[k] : kFoldPull;
                        float& c = cost[k][3 * eff[k - 1] + m];
                        c = c == kUnset ? tt[k] : std::min(c, tt[k]);
                    }
                }
            std::vector<float>& mc = e->mode_costs[{semiring, B}];
            mc.assign((size_t)nl * 9, kUnset);
            for (int k = 0; k < nl; ++k)
                for (int j = 0; j < 9; ++j) mc[(size_t)k * 9 + j] = cost[k][j];
            const float kInf = 3.0e38f;
            std::vector<std::array<float, 3>> acc(D + 2);
            std::vector<std::array<int, 3>> from(D + 2);
            for (auto& x : acc) x.fill(kInf);
            acc[0][kFoldPull] = 0.0f;
            for (int k = 1; k <= D + 1; ++k)
                for (int m = 0; m < 3; ++m) {
                    if (k <= D ? !allowed(k, m) : m != kFoldPull) continue;
                    for (int mp = 0; mp < 3; ++mp) {
                        const float c = cost[k][3 * mp + m];
                        if (acc[k - 1][mp] >= kInf || c == kUnset) continue;
                        if (acc[k - 1][mp] + c < acc[k][m]) {
                            acc[k][m] = acc[k - 1][mp] + c;
                            from[k][m] = mp;
                        }
                    }
                }
            if (acc[D + 1][kFoldPull] < kInf) {
                int m = from[D + 1][kFoldPull];
                for (int k = D; k >= 1; --k) {
                    best[k] |= flag[m];
                    m = from[k][m];
                }
            }
        }
        // Shared-memory staging of the left-child window: it changes only the
        // launch of its own level, so each level keeps it where that launch
        // measured at least 2 % faster with it.
        if (D >= 1) {
            std::vector<uint8_t> st_table = best;
            for (int k = 1; k <= D; ++k)
                if (!(best[k] & GMR_LEVEL_PUSH)) st_table[k] |= GMR_LEVEL_STAGE;
            const std::vector<float> base_t = slot_times(best), st_t = slot_times(st_table);
            for (int k = 1; k <= D; ++k)
                if (st_table[k] != best[k] && st_t[k] < 0.98f * base_t[k]) best[k] = st_table[k];
        }
        if (gmr_engine_set_level_variants(e, semiring, B, best.data(), nl) != GMR_OK) throw Error(GMR_ERR_ARG, gmr_last_error());
        if (ms) std::copy(med.begin(), med.end(), ms);
    });
}

extern "C" int gmr_engine_status(const gmr_engine* e, int* failed, int* phase) {
    return guarded([&] {
        if (!e) throw Error(GMR_ERR_ARG, "null engine");
        if (failed) *failed = e->status_host ? e->status_host[0] : 0;
        if (phase) *phase = e->status_host ? e->status_host[1] : 0;
    });
}

extern "C" int gmr_engine_mode_costs(gmr_engine* e, int semiring, int B, float* out, int cap, int* n_slots) {
    return guarded([&] {
        if (!e || !out || !n_slots) throw Error(GMR_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(e->mu);
        auto it = e->mode_costs.find({semiring, B});
        if (it == e->mode_costs.end()) {
            *n_slots = 0;
            return;
        }
        if ((size_t)cap < it->second.size()) throw Error(GMR_ERR_RANGE, "need (depth + 2) x 9 floats");
        std::copy(it->second.begin(), it->second.end(), out);
        *n_slots = (int)(it->second.size() / 9);
    });
}

extern "C" int gmr_engine_lane_bytes(gmr_engine* e, int semiring, int B) {
    if (!e || semiring < 0 || semiring > 2 || B < 1) return -1;
    try {
        std::lock_guard<std::mutex> lk(e->mu);
        // 256-byte aligned stand-ins: only the alignment of X and Y enters the choice
        const Launch lc = resolve_launch(e, semiring, B, reinterpret_cast<const void*>(256),
                                         reinterpret_cast<void*>(256), nullptr);
        return lc.VEC * 4;
    } catch (...) {
        return -1;
    }
}

extern "C" int64_t gmr_engine_last_launches(const gmr_engine* e) { return e ? e->last_launches : -1; }

extern "C" int64_t gmr_engine_device_bytes(const gmr_engine* e) {
    if (!e) return -1;
    int64_t t = 0;
    auto bufs = const_cast<gmr_engine*>(e)->schedule_bufs();
    for (auto* b : {&e->arena, &e->T, &e->hX, &e->hY}) bufs.push_back(const_cast<DevBuf*>(b));
    for (auto* b : bufs) t += (int64_t)b->bytes;
    return t;
}

extern "C" void gmr_engine_free(gmr_engine* e) {
    if (!e) return;
    {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(e->device);
        for (auto& g : e->graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (auto* b : e->schedule_bufs()) b->release();
        for (auto* b : {&e->arena, &e->T, &e->hX, &e->hY, &e->hX2, &e->hY2}) b->release();
        for (auto ev : e->pipe_ev)
            if (ev) cudaEventDestroy(ev);
        for (auto s2 : {e->copy_in, e->copy_out})
            if (s2) cudaStreamDestroy(s2);
        if (e->own_stream) cudaStreamDestroy(e->own_stream);
        if (e->status_host) cudaFreeHost(e->status_host);
        if (prev >= 0) cudaSetDevice(prev);
    }
    delete e;
}

// ------------------------------------------------------------------ left product
// y = x^T M (y[c] = (+)_r x[r] (x) M[r][c]) over the same grammar, top-down:
// the "down" value of a symbol is the (+) of its parents' down values (times
// the run-length coefficient for a left child) and of x over the rows that
// emit it; levels run from the top down (a parent is always above its
// children), then every column folds leaf(V, down) over its terminals.
//
// Each level is one launch over its flat edge list (targets ascending): a lane
// group folds a chunk of kLeftChunk edges in registers and writes a target
// whose edges all lie in the chunk with a plain store; a target whose edges
// straddle chunks was set to the semiring zero before the first level and
// each chunk folds its part into it atomically.  Symbols with thousands of
// parents or rows are thereby spread over many lane groups.
namespace gmr {

struct LeftArgs {
    void* down;     // [n_ops][Bw] (the arena): rules' down values
    void* tdown;    // [U][Bw] (the terminal table): terminals' down values
    const void* X;  // [rows][Bw]
    void* Y;        // [cols][Bw]
    const int32_t* src;
    const int32_t* tgt;
    const int32_t* split;
    const int64_t* tcol_off;
    const int32_t* tcol_q;
    const float* op_c;
    const float* V;
    const int32_t* term_val;
    int64_t n_ops, first, count;
    int Bw, G;
    bool terminals;  // targets of this launch are terminals (tdown) rather than rules (down)
};

template <class S, int VEC>
__device__ __forceinline__ Vec<typename S::T, VEC> left_edge_value(const LeftArgs& a, int32_t s, int lane) {
    using T = typename S::T;
    const bool row = (int64_t)s >= a.n_ops;
    const int64_t pp = s >= 0 ? (int64_t)s : (int64_t)~s;
    const T* base = row ? static_cast<const T*>(a.X) + (pp - a.n_ops) * a.Bw : static_cast<const T*>(a.down) + pp * a.Bw;
    Vec<T, VEC> v = vload<T, VEC>(base + lane * VEC);
    if (a.op_c && s >= 0 && !row) {
        const float c = __ldg(a.op_c + pp);
#pragma unroll
        for (int j = 0; j < VEC; ++j) v.v[j] = S::apply(v.v[j], c);
    }
    return v;
}

template <class S, int VEC>
__device__ __forceinline__ void left_flush(const LeftArgs& a, int32_t u, int lane, bool whole,
                                           const Vec<typename S::T, VEC>& acc) {
    using T = typename S::T;
    T* p = static_cast<T*>(a.terminals ? a.tdown : a.down) + (int64_t)u * a.Bw + lane * VEC;
    if (whole) vstore<T, VEC>(p, acc);
    else vred<S, VEC>(p, acc);
}

// Straddling targets start at the semiring zero.
template <class S, int VEC, int GLOG>
__global__ void __launch_bounds__(256) k_left_zero(LeftArgs a) {
    using T = typename S::T;
    const int64_t items = items_of<GLOG>(a.count, a.G);  // count = straddling targets
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < items; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = __ldg(a.split + unit_of<GLOG>(t, a.G));
        const int lane = lane_of<GLOG>(t, a.G);
        T* p = u < a.n_ops ? static_cast<T*>(a.down) + u * a.Bw : static_cast<T*>(a.tdown) + (u - a.n_ops) * a.Bw;
        vstore<T, VEC>(p + lane * VEC, vzero<S, VEC>());
    }
}

template <class S, int VEC, int GLOG>
__global__ void __launch_bounds__(256) k_left_fold(LeftArgs a) {
    using T = typename S::T;
    const int64_t groups = (a.count + kLeftChunk - 1) / kLeftChunk;
    const int64_t items = items_of<GLOG>(groups, a.G);
    const int32_t* src = a.src + a.first;
    const int32_t* tgt = a.tgt + a.first;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < items; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = unit_of<GLOG>(t, a.G);
        const int lane = lane_of<GLOG>(t, a.G);
        const int64_t e0 = g * kLeftChunk, e1 = min(e0 + kLeftChunk, a.count);
        int32_t cur = __ldg(tgt + e0);
        bool whole = e0 == 0 || __ldg(tgt + e0 - 1) != cur;  // cur's first edge is in this chunk
        Vec<T, VEC> acc = vzero<S, VEC>();
        int64_t e = e0;
        for (; e + 4 <= e1; e += 4) {
            int32_t u[4], s4[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                u[j] = __ldg(tgt + e + j);
                s4[j] = __ldg(src + e + j);
            }
            Vec<T, VEC> v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = left_edge_value<S, VEC>(a, s4[j], lane);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (u[j] != cur) {
                    left_flush<S, VEC>(a, cur, lane, whole, acc);
                    whole = true;
                    acc = v[j];
                    cur = u[j];
                } else {
                    acc = voplus<S, VEC>(acc, v[j]);
                }
            }
        }
        for (; e < e1; ++e) {
            const int32_t u = __ldg(tgt + e);
            const Vec<T, VEC> v = left_edge_value<S, VEC>(a, __ldg(src + e), lane);
            if (u != cur) {
                left_flush<S, VEC>(a, cur, lane, whole, acc);
                whole = true;
                acc = v;
                cur = u;
            } else {
                acc = voplus<S, VEC>(acc, v);
            }
        }
        const bool ends = e1 == a.count || __ldg(tgt + e1) != cur;  // cur's last edge is in this chunk
        left_flush<S, VEC>(a, cur, lane, whole && ends, acc);
    }
}

template <class S, int VEC, int GLOG>
__global__ void __launch_bounds__(256) k_left_columns(LeftArgs a) {
    using T = typename S::T;
    const int64_t items = items_of<GLOG>(a.count, a.G);  // count = cols
    const T* tdown = static_cast<const T*>(a.tdown);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < items; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = unit_of<GLOG>(t, a.G);
        const int lane = lane_of<GLOG>(t, a.G);
        Vec<T, VEC> acc = vzero<S, VEC>();
        for (int64_t i = __ldg(a.tcol_off + c), i1 = __ldg(a.tcol_off + c + 1); i < i1; ++i) {
            const int32_t q = __ldg(a.tcol_q + i);
            const Vec<T, VEC> d = vload<T, VEC>(tdown + (int64_t)q * a.Bw + lane * VEC);
            const float v = __ldg(a.V + __ldg(a.term_val + q - 1));
            Vec<T, VEC> l;
#pragma unroll
            for (int j = 0; j < VEC; ++j) l.v[j] = S::leaf(v, d.v[j]);
            acc = voplus<S, VEC>(acc, l);
        }
        vstore<T, VEC>(static_cast<T*>(a.Y) + c * a.Bw + lane * VEC, acc);
    }
}

template <class S, int VEC, int GLOG>
static void left_chain_t(gmr_engine* e, int Bw, int G, const void* X, void* Y, cudaStream_t st) {
    LeftArgs a{};
    a.down = e->arena.p;
    a.tdown = e->T.p;
    a.X = X;
    a.Y = Y;
    a.src = static_cast<const int32_t*>(e->le_src.p);
    a.tgt = static_cast<const int32_t*>(e->le_tgt.p);
    a.split = static_cast<const int32_t*>(e->le_split.p);
    a.tcol_off = static_cast<const int64_t*>(e->tcol_off.p);
    a.tcol_q = static_cast<const int32_t*>(e->tcol_q.p);
    a.op_c = e->has_coeff ? static_cast<const float*>(e->op_c.p) : nullptr;
    a.V = static_cast<const float*>(e->V.p);
    a.term_val = static_cast<const int32_t*>(e->term_val.p);
    a.n_ops = e->n_ops;
    a.Bw = Bw;
    a.G = G;
    auto blocks = [&](int64_t items) {
        return (int)std::max<int64_t>(1, std::min<int64_t>((items + 255) / 256, (int64_t)e->sm_count * 32));
    };
    const int D = e->depth;
    a.count = e->n_left_split;
    if (a.count) k_left_zero<S, VEC, GLOG><<<blocks(a.count * G), 256, 0, st>>>(a);
    for (int j = D; j >= 0; --j) {  // levels D .. 1 from the top, then the terminals (range D + 1)
        const int k = j ? j : D + 1;
        a.first = e->le_off[k - 1];
        a.count = e->le_off[k] - e->le_off[k - 1];
        a.terminals = k == D + 1;
        if (a.count == 0) continue;
        k_left_fold<S, VEC, GLOG><<<blocks((a.count + kLeftChunk - 1) / kLeftChunk * G), 256, 0, st>>>(a);
    }
    a.first = 0;
    a.count = e->cols;
    k_left_columns<S, VEC, GLOG><<<blocks((int64_t)e->cols * G), 256, 0, st>>>(a);
    GMR_CUDA(cudaGetLastError());
}

template <class S>
static void left_chain_s(gmr_engine* e, int Bw, const void* X, void* Y, cudaStream_t st) {
    const bool a16 = ((uintptr_t)X % 16 == 0) && ((uintptr_t)Y % 16 == 0);
    if (Bw % 4 == 0 && a16) {
        switch (Bw / 4) {
            case 1: return left_chain_t<S, 4, 0>(e, Bw, 1, X, Y, st);
            case 2: return left_chain_t<S, 4, 1>(e, Bw, 2, X, Y, st);
            case 4: return left_chain_t<S, 4, 2>(e, Bw, 4, X, Y, st);
            case 8: return left_chain_t<S, 4, 3>(e, Bw, 8, X, Y, st);
            case 16: return left_chain_t<S, 4, 4>(e, Bw, 16, X, Y, st);
            case 32: return left_chain_t<S, 4, 5>(e, Bw, 32, X, Y, st);
            default: return left_chain_t<S, 4, -1>(e, Bw, Bw / 4, X, Y, st);
        }
    }
    if (Bw == 1) return left_chain_t<S, 1, 0>(e, Bw, 1, X, Y, st);
    return left_chain_t<S, 1, -1>(e, Bw, Bw, X, Y, st);
}

}  // namespace gmr

extern "C" int gmr_engine_enable_left(gmr_engine* e, gmr_plan* p) {
    return guarded([&] {
        if (!e || !p) throw Error(GMR_ERR_ARG, "null argument");
        if (p->n_ops() != e->n_ops || p->rows != e->rows || p->cols != e->cols)
            throw Error(GMR_ERR_ARG, "plan does not match the engine");
        int rc = gmr_plan_prepare_left(p);
        if (rc != GMR_OK) throw Error(rc, gmr_last_error());
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        upload(p->le_src, e->le_src);
        upload(p->le_tgt, e->le_tgt);
        upload(p->le_split, e->le_split);
        upload(p->tcol_off, e->tcol_off);
        upload(p->tcol_q, e->tcol_q);
        e->le_off = p->le_off;
        e->n_left_split = (int64_t)p->le_split.size();
        e->left_ready = true;
    });
}

extern "C" int gmr_engine_multiply_left(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                                        void* stream) {
    return guarded([&] {
        if (!e) throw Error(GMR_ERR_ARG, "null engine");
        if (!e->left_ready) throw Error(GMR_ERR_STATE, "call gmr_engine_enable_left first");
        if (semiring < 0 || semiring > 2) throw Error(GMR_ERR_ARG, "unknown semiring");
        if (B < 1) throw Error(GMR_ERR_ARG, "B must be >= 1");
        if ((!dX && e->rows > 0) || (!dY && e->cols > 0)) throw Error(GMR_ERR_ARG, "null X or Y");
        if (((uintptr_t)dX | (uintptr_t)dY) % 4 != 0) throw Error(GMR_ERR_ARG, "X and Y must be 4-byte aligned");
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        const int Bw = words_per_slot(semiring, B);
        ensure_scratch(e, Bw);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (semiring == GMR_PLUS_TIMES) left_chain_s<SPlus>(e, Bw, dX, dY, st);
        else if (semiring == GMR_BOOLEAN) left_chain_s<SBool>(e, Bw, dX, dY, st);
        else left_chain_s<STrop>(e, Bw, dX, dY, st);
        e->last_launches = e->depth + 2 + (e->n_left_split ? 1 : 0);
    });
}

// ------------------------------------------------------------------ fixpoint iteration
// x <- x (+) (M (x) x) until nothing changes, for a square matrix in the
// idempotent semirings: the natural caller of the Boolean and tropical sweeps
// (reachability / BFS frontiers, Bellman-Ford relaxation).
namespace gmr {

template <class S>
__global__ void k_merge_changed(typename S::T* __restrict__ X, const typename S::T* __restrict__ Y, int64_t n,
                                int* __restrict__ changed) {
    bool any = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const typename S::T x = X[i], v = S::oplus(x, Y[i]);
        if (v != x) {
            X[i] = v;
            any = true;
        }
    }
    if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) atomicExch(changed, 1);
}

}  // namespace gmr

namespace gmr {

// End of one fixpoint iteration, on one thread: counts it, keeps the loop
// going while the merge changed something and the count is below the limit,
// and clears the change flag for the next iteration.
__global__ void k_fix_step(int* flag, int* count, const int* max_iters, cudaGraphConditionalHandle h) {
    const int c = *count + 1;
    *count = c;
    const int changed = *flag;
    *flag = 0;
    cudaGraphSetConditional(h, (changed != 0 && c < *max_iters) ? 1u : 0u);
}

__global__ void k_set_i32(int* p, int v) { *p = v; }

// The whole loop as one graph: a conditional while node whose body is one
// multiply (the per-launch kernels, no nested graph), the merge kernel and
// k_fix_step.  The host launches it once and reads the iteration count.
static GraphEntry* fixpoint_graph(gmr_engine* e, const Launch& lc, int semiring, void* X, void* Y, int64_t n,
                                  int* flag, int* count, const int* max_iters) {
    for (auto& g : e->graphs)
        if (g.exec && g.fixpoint && g.lc == lc && g.X == X && g.Y == Y) return &g;
    if (e->graphs.size() >= 8) {
        cudaGraphExecDestroy(e->graphs.front().exec);
        e->graphs.erase(e->graphs.begin());
    }
    cudaGraph_t graph = nullptr;
    GMR_CUDA(cudaGraphCreate(&graph, 0));
    GraphEntry ge;
    ge.lc = lc;
    ge.X = X;
    ge.Y = Y;
    ge.fixpoint = true;
    try {
        cudaGraphConditionalHandle h;
        GMR_CUDA(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        GMR_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        GMR_CUDA(cudaStreamBeginCaptureToGraph(e->own_stream, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
        int64_t launches = 0;
        cudaGraph_t captured = nullptr;
        try {
            t_chain_no_status = true;
            try {
                launch_chain(e, lc, X, Y, e->own_stream, launches);
            } catch (...) {
                t_chain_no_status = false;
                throw;
            }
            t_chain_no_status = false;
            const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)e->sm_count * 8));
            if (semiring == GMR_BOOLEAN)
                k_merge_changed<SBool><<<blocks, 256, 0, e->own_stream>>>(static_cast<uint32_t*>(X),
                                                                         static_cast<const uint32_t*>(Y), n, flag);
            else
                k_merge_changed<STrop><<<blocks, 256, 0, e->own_stream>>>(static_cast<int32_t*>(X),
                                                                         static_cast<const int32_t*>(Y), n, flag);
            k_fix_step<<<1, 1, 0, e->own_stream>>>(flag, count, max_iters, h);
            GMR_CUDA(cudaGetLastError());
        } catch (...) {
            cudaStreamEndCapture(e->own_stream, &captured);
            throw;
        }
        GMR_CUDA(cudaStreamEndCapture(e->own_stream, &captured));
        ge.launches = launches + 2;
        GMR_CUDA(cudaGraphInstantiate(&ge.exec, graph, 0));
    } catch (...) {
        cudaGraphDestroy(graph);
        throw;
    }
    cudaGraphDestroy(graph);
    e->graphs.push_back(ge);
    return &e->graphs.back();
}

}  // namespace gmr

extern "C" int gmr_engine_fixpoint(gmr_engine* e, int semiring, void* dX, void* dY, int B, int max_iters,
                                   void* stream, int* iters) {
    return guarded([&] {
        if (!e || !dX || !dY) throw Error(GMR_ERR_ARG, "null argument");
        if (semiring != GMR_BOOLEAN && semiring != GMR_TROPICAL)
            throw Error(GMR_ERR_ARG, "fixpoint needs an idempotent semiring (boolean or tropical)");
        if (e->rows != e->cols) throw Error(GMR_ERR_ARG, "fixpoint needs a square matrix");
        if (B < 1 || max_iters < 0) throw Error(GMR_ERR_ARG, "bad B or max_iters");
        if (((uintptr_t)dX | (uintptr_t)dY) % 4 != 0) throw Error(GMR_ERR_ARG, "X and Y must be 4-byte aligned");
        std::lock_guard<std::mutex> lk(e->mu);
        DeviceGuard dg(e->device);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (iters) *iters = 0;
        if (max_iters == 0) return;
        Launch lc = resolve_launch(e, semiring, B, dX, dY, nullptr);
        if (lc.variant == GMR_VARIANT_GRAPH || lc.variant == GMR_VARIANT_PERSISTENT) lc.variant = GMR_VARIANT_FUSED;
        ensure_scratch(e, lc.Bw);
        const int64_t n = (int64_t)e->rows * lc.Bw;
        e->sync.ensure(64);
        int* flag = reinterpret_cast<int*>(static_cast<unsigned char*>(e->sync.p) + 8);
        int* count = flag + 1;
        int* limit = flag + 2;
        GraphEntry* g = fixpoint_graph(e, lc, semiring, dX, dY, n, flag, count, limit);
        GMR_CUDA(cudaMemsetAsync(flag, 0, 8, st));
        GMR_CUDA(cudaMemsetAsync(e->stage_err(), 0, 8, st));
        k_set_i32<<<1, 1, 0, st>>>(limit, max_iters);
        GMR_CUDA(cudaGetLastError());
        GMR_CUDA(cudaGraphLaunch(g->exec, st));
        GMR_CUDA(cudaMemcpyAsync(e->status_host + 2, count, 4, cudaMemcpyDeviceToHost, st));
        GMR_CUDA(cudaMemcpyAsync(e->status_host, e->stage_err(), 8, cudaMemcpyDeviceToHost, st));
        GMR_CUDA(cudaStreamSynchronize(st));
        if (iters) *iters = e->status_host[2];
        e->last_launches = g->launches * e->status_host[2] + 1;
        if (e->status_host[0] != 0)
            throw Error(GMR_ERR_TIMEOUT, "fixpoint: a staged-window wait gave up at level " +
                                             std::to_string(-e->status_host[1]) + "; X is not valid");
    });
}

// ------------------------------------------------------------------ packed multi-grammar launch
// Several engines (grammars of uneven size, each with its own X, Y, B and
// semiring) multiplied by ONE graph launch: the capture forks one branch per
// engine (its own stream), so the small grammars' short tails run beside the
// big grammars' wide levels instead of after them.
struct gmr_pack {
    std::vector<gmr_engine*> engines;
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t exec = nullptr;
    std::vector<gmr::Launch> key_lc;
    std::vector<const void*> key_x;
    std::vector<void*> key_y, key_arena;
    int64_t launches = 0;
    int device = 0;
    // one persistent launch (GMR_PACK_PERSISTENT): grammar table on the
    // device, barrier and error words, pinned copy of the error words
    int mode = GMR_PACK_GRAPH;
    unsigned long long spin_limit = 20000000ull;
    cudaGraphExec_t levels_exec = nullptr;  // GMR_PACK_LEVELS: the captured level chain
    int levels_semiring = -1;
    int64_t levels_launches = 0;
    gmr::DevBuf table, sync;
    std::vector<char> key_table;
    int* status_host = nullptr;
    bool last_persistent = false;
};

namespace gmr {

static int pack_kind(const Launch& lc) {
    if (lc.VEC == 4) {
        for (int l = 0; l <= 5; ++l)
            if (lc.G == (1 << l)) return l;
        return 6;
    }
    if (lc.VEC == 2) return lc.G == 1 ? 7 : 9;
    return lc.G == 1 ? 8 : 10;
}

template <class S>
static void launch_pack(gmr_pack* p, const PackGrammar* table, int n, int max_depth, cudaStream_t st) {
    auto kernel = k_pack<S, GMR_EMIT_SEGMENTED>;
    int per_sm = 0, sms = 152;
    GMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
    if (per_sm < 1) throw Error(GMR_ERR_STATE, "packed persistent kernel cannot be resident");
    GMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
    PersistArgs P{};
    P.bar = static_cast<unsigned*>(p->sync.p);
    P.err = reinterpret_cast<int*>(static_cast<unsigned char*>(p->sync.p) + 8);
    P.spin_limit = p->spin_limit;
    GMR_CUDA(cudaMemsetAsync(p->sync.p, 0, 16, st));
    const PackGrammar* tb = table;
    void* args[] = {&tb, &n, &max_depth, &P};
    GMR_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kernel), dim3(per_sm * sms), dim3(256), args, 0, st));
    GMR_CUDA(cudaMemcpyAsync(p->status_host, P.err, 8, cudaMemcpyDeviceToHost, st));
}

// Grammar table of a pack (every engine in one semiring, no direct
// terminals), uploaded again only when the engines' scratch, X, Y or widths
// change.  Returns the deepest grammar's depth; *changed = a new upload.
static int pack_table(gmr_pack* p, const std::vector<Launch>& lcs, const void* const* dX, void* const* dY,
                      cudaStream_t st, std::vector<PackGrammar>& tab, bool* changed) {
    const int n = (int)p->engines.size();
    tab.assign(n, PackGrammar{});
    int max_depth = 0;
    for (int i = 0; i < n; ++i) {
        gmr_engine* e = p->engines[i];
        const Launch& lc = lcs[i];
        PackGrammar& g = tab[i];
        std::memset(static_cast<void*>(&g), 0, sizeof(g));
        SweepArgs& a = g.a;
        a.arena = e->arena.p;
        a.T = e->T.p;
        a.Y = dY[i];
        a.X = dX[i];
        a.V = static_cast<const float*>(e->V.p);
        a.term_val = static_cast<const int32_t*>(e->term_val.p);
        a.term_col = static_cast<const int32_t*>(e->term_col.p);
        a.n_terms = e->n_terms;
        a.n_ops = e->n_ops;
        a.rows = e->rows;
        a.ldx = lc.Bw;
        a.ldy = lc.Bw;
        a.Bt = lc.Bw;
        a.G = lc.Bw / lc.VEC;
        a.t0 = 0;
        a.cols = e->cols;
        LevelArgs& L = g.L;
        L.ops = static_cast<const int2*>(e->ops.p);
        L.op_c = e->has_coeff ? static_cast<const float*>(e->op_c.p) : nullptr;
        L.em_src = static_cast<const int32_t*>(e->em_src.p);
        L.em_row = static_cast<const int32_t*>(e->em_row.p);
        L.seg_row = static_cast<const int32_t*>(e->seg_row.p);
        L.seg_start = static_cast<const int64_t*>(e->seg_start.p);
        L.em_chunk = 16;
        g.lvl_off = static_cast<const int64_t*>(e->d_lvl_off.p);
        g.em_off = static_cast<const int64_t*>(e->d_em_off.p);
        g.seg_off = static_cast<const int64_t*>(e->d_seg_off.p);
        g.depth = e->depth;
        Launch one = lc;
        one.Bt = lc.Bw;
        one.G = a.G;
        g.kind = pack_kind(one);
        max_depth = std::max(max_depth, e->depth);
    }
    const size_t bytes = sizeof(PackGrammar) * (size_t)n;
    std::vector<char> key(reinterpret_cast<const char*>(tab.data()), reinterpret_cast<const char*>(tab.data()) + bytes);
    *changed = key != p->key_table;
    if (*changed) {
        p->table.ensure(bytes);
        GMR_CUDA(cudaStreamSynchronize(st));  // the table may be in use by an earlier launch
        GMR_CUDA(cudaMemcpy(p->table.p, tab.data(), bytes, cudaMemcpyHostToDevice));
        p->key_table = std::move(key);
    }
    return max_depth;
}

static void pack_persistent(gmr_pack* p, int semiring, const std::vector<Launch>& lcs, const void* const* dX,
                            void* const* dY, cudaStream_t st) {
    std::vector<PackGrammar> tab;
    bool changed = false;
    const int n = (int)p->engines.size();
    const int max_depth = pack_table(p, lcs, dX, dY, st, tab, &changed);
    const PackGrammar* table = static_cast<const PackGrammar*>(p->table.p);
    if (semiring == GMR_PLUS_TIMES) launch_pack<SPlus>(p, table, n, max_depth, st);
    else if (semiring == GMR_BOOLEAN) launch_pack<SBool>(p, table, n, max_depth, st);
    else launch_pack<STrop>(p, table, n, max_depth, st);
    p->launches = 1;
    p->last_persistent = true;
}

// Blocks of grammar g in the level-k launch: the engine's own grid sizing
// (emissions folded by the segmented chunk-16 fold, rules two per thread,
// at most 32 blocks per SM for each part, grid-stride beyond).
static void pack_level_blocks(const gmr_engine* e, const PackGrammar& g, int k, int sm_count, int* eb, int* ob) {
    auto blocks = [&](int64_t items) -> int {
        return (int)std::max<int64_t>(1, std::min<int64_t>((items + 255) / 256, (int64_t)sm_count * 32));
    };
    const int G = g.a.G;
    const bool lane_per_unit = g.kind == 0 || g.kind == 7 || g.kind == 8;  // warp-segmented fold
    *eb = *ob = 0;
    if (k == 0) {
        *ob = blocks((e->rows + e->n_terms) * (int64_t)G);
        return;
    }
    if (k > e->depth + 1) return;
    const int64_t ne = e->em_off[k] - e->em_off[k - 1];
    const int64_t no = k <= e->depth ? e->lvl_off[k] - e->lvl_off[k - 1] : 0;
    if (ne > 0) *eb = blocks(lane_per_unit ? (ne + 1) / 2 : (ne + 15) / 16 * G);
    if (no > 0) *ob = blocks((no * G + 1) / 2);
}

template <class S>
static void pack_level_chain(gmr_pack* p, int n, int max_depth, cudaStream_t st) {
    const PackGrammar* table = static_cast<const PackGrammar*>(p->table.p);
    int sms = 152;
    GMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
    std::vector<PackGrammar> host(n);
    std::memcpy(static_cast<void*>(host.data()), p->key_table.data(), sizeof(PackGrammar) * (size_t)n);
    int64_t launches = 0;
    for (int k = 0; k <= max_depth + 1; ++k) {
        PackLaunch P{};
        P.n = n;
        P.k = k;
        for (int i = 0; i < n; ++i) {
            int eb = 0, ob = 0;
            pack_level_blocks(p->engines[i], host[i], k, sms, &eb, &ob);
            P.em_blocks[i] = eb;
            P.blk[i + 1] = P.blk[i] + eb + ob;
        }
        if (P.blk[n] == 0) continue;
        k_pack_level<S, GMR_EMIT_SEGMENTED><<<P.blk[n], 256, 0, st>>>(table, P);
        ++launches;
    }
    GMR_CUDA(cudaGetLastError());
    p->launches = launches;
}

// The pack as one launch per level, captured once into a graph and replayed
// while the grammar table stays the same.
static void pack_levels(gmr_pack* p, int semiring, const std::vector<Launch>& lcs, const void* const* dX,
                        void* const* dY, cudaStream_t st) {
    std::vector<PackGrammar> tab;
    bool changed = false;
    const int n = (int)p->engines.size();
    const int max_depth = pack_table(p, lcs, dX, dY, st, tab, &changed);
    if (changed || !p->levels_exec || p->levels_semiring != semiring) {
        if (p->levels_exec) cudaGraphExecDestroy(p->levels_exec);
        p->levels_exec = nullptr;
        cudaGraph_t graph = nullptr;
        GMR_CUDA(cudaStreamBeginCapture(p->origin, cudaStreamCaptureModeThreadLocal));
        try {
            if (semiring == GMR_PLUS_TIMES) pack_level_chain<SPlus>(p, n, max_depth, p->origin);
            else if (semiring == GMR_BOOLEAN) pack_level_chain<SBool>(p, n, max_depth, p->origin);
            else pack_level_chain<STrop>(p, n, max_depth, p->origin);
        } catch (...) {
            cudaStreamEndCapture(p->origin, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        GMR_CUDA(cudaStreamEndCapture(p->origin, &graph));
        cudaError_t ie = cudaGraphInstantiate(&p->levels_exec, graph, 0);
        cudaGraphDestroy(graph);
        GMR_CUDA(ie);
        p->levels_semiring = semiring;
        p->levels_launches = p->launches;
    }
    GMR_CUDA(cudaGraphLaunch(p->levels_exec, st));
    p->launches = p->levels_launches;
}

}  // namespace gmr

extern "C" int gmr_pack_create(gmr_engine* const* engines, int n, gmr_pack** out) {
    return guarded([&] {
        if (!engines || n < 1 || !out) throw Error(GMR_ERR_ARG, "bad argument");
        auto p = std::make_unique<gmr_pack>();
        for (int i = 0; i < n; ++i) {
            if (!engines[i]) throw Error(GMR_ERR_ARG, "null engine");
            if (engines[i]->device != engines[0]->device) throw Error(GMR_ERR_ARG, "engines on different devices");
            for (int j = 0; j < i; ++j)
                if (engines[j] == engines[i]) throw Error(GMR_ERR_ARG, "an engine appears twice");
            p->engines.push_back(engines[i]);
        }
        p->device = engines[0]->device;
        DeviceGuard dg(p->device);
        GMR_CUDA(cudaStreamCreateWithFlags(&p->origin, cudaStreamNonBlocking));
        GMR_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
        p->join.resize(n);
        for (auto& ev : p->join) GMR_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        p->sync.ensure(16);
        GMR_CUDA(cudaMemset(p->sync.p, 0, 16));
        GMR_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&p->status_host), 16, cudaHostAllocDefault));
        std::memset(p->status_host, 0, 16);
        *out = p.release();
    });
}

extern "C" int gmr_pack_multiply(gmr_pack* p, const int* semirings, const void* const* dX, void* const* dY,
                                 const int* B, void* stream) {
    return guarded([&] {
        if (!p || !semirings || !dX || !dY || !B) throw Error(GMR_ERR_ARG, "null argument");
        const int n = (int)p->engines.size();
        std::vector<gmr_engine*> order(p->engines);
        std::sort(order.begin(), order.end());
        std::vector<std::unique_lock<std::mutex>> locks;
        for (auto* e : order) locks.emplace_back(e->mu);
        DeviceGuard dg(p->device);
        bool uniform = true, direct = false;
        for (int i = 0; i < n; ++i) {
            uniform = uniform && semirings[i] == semirings[0];
            direct = direct || p->engines[i]->direct_terms;
        }
        // the single-kernel packings instantiate lanes of up to 16 bytes; the
        // graph of per-engine branches runs each engine's own chain
        const bool one_kernel = uniform && !direct &&
                                (p->mode == GMR_PACK_PERSISTENT || (p->mode == GMR_PACK_LEVELS && n <= kMaxPackLevels));
        std::vector<Launch> lcs;
        for (int i = 0; i < n; ++i) {
            gmr_engine* e = p->engines[i];
            if (semirings[i] < 0 || semirings[i] > 2) throw Error(GMR_ERR_ARG, "unknown semiring");
            if (B[i] < 1) throw Error(GMR_ERR_ARG, "B must be >= 1");
            if (((uintptr_t)dX[i] | (uintptr_t)dY[i]) % 4 != 0) throw Error(GMR_ERR_ARG, "misaligned X or Y");
            Launch lc = resolve_launch(e, semirings[i], B[i], dX[i], dY[i], nullptr, one_kernel ? 4 : 8);
            ensure_scratch(e, lc.Bw);
            lcs.push_back(lc);
        }
        p->last_persistent = false;
        if (p->mode == GMR_PACK_PERSISTENT && uniform && !direct) {
            pack_persistent(p, semirings[0], lcs, dX, dY, static_cast<cudaStream_t>(stream));
            return;
        }
        if (p->mode == GMR_PACK_LEVELS && uniform && !direct && n <= kMaxPackLevels) {
            pack_levels(p, semirings[0], lcs, dX, dY, static_cast<cudaStream_t>(stream));
            return;
        }
        bool hit = p->exec != nullptr && p->key_lc.size() == (size_t)n;
        for (int i = 0; hit && i < n; ++i)
            hit = p->key_lc[i] == lcs[i] && p->key_x[i] == dX[i] && p->key_y[i] == dY[i] &&
                  p->key_arena[i] == p->engines[i]->arena.p;
        if (!hit) {
            if (p->exec) cudaGraphExecDestroy(p->exec);
            p->exec = nullptr;
            cudaGraph_t graph = nullptr;
            GMR_CUDA(cudaStreamBeginCapture(p->origin, cudaStreamCaptureModeThreadLocal));
            int64_t total = 0;
            try {
                GMR_CUDA(cudaEventRecord(p->fork, p->origin));
                for (int i = 0; i < n; ++i) {
                    gmr_engine* e = p->engines[i];
                    GMR_CUDA(cudaStreamWaitEvent(e->own_stream, p->fork, 0));
                    launch_chain(e, lcs[i], dX[i], dY[i], e->own_stream, total);
                    GMR_CUDA(cudaEventRecord(p->join[i], e->own_stream));
                    GMR_CUDA(cudaStreamWaitEvent(p->origin, p->join[i], 0));
                }
            } catch (...) {
                cudaStreamEndCapture(p->origin, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            GMR_CUDA(cudaStreamEndCapture(p->origin, &graph));
            cudaError_t ie = cudaGraphInstantiate(&p->exec, graph, 0);
            cudaGraphDestroy(graph);
            GMR_CUDA(ie);
            p->key_lc = lcs;
            p->key_x.assign(dX, dX + n);
            p->key_y.assign(dY, dY + n);
            p->key_arena.clear();
            for (auto* e : p->engines) p->key_arena.push_back(e->arena.p);
            p->launches = total;
        }
        GMR_CUDA(cudaGraphLaunch(p->exec, static_cast<cudaStream_t>(stream)));
    });
}

extern "C" int64_t gmr_pack_last_launches(const gmr_pack* p) { return p ? p->launches : -1; }

extern "C" int gmr_pack_set_mode(gmr_pack* p, int mode, int spin_limit) {
    return guarded([&] {
        if (!p) throw Error(GMR_ERR_ARG, "null pack");
        if (mode != GMR_PACK_GRAPH && mode != GMR_PACK_PERSISTENT && mode != GMR_PACK_LEVELS)
            throw Error(GMR_ERR_ARG, "unknown pack mode");
        p->mode = mode;
        p->spin_limit = spin_limit > 0 ? (unsigned long long)spin_limit : 20000000ull;
    });
}

extern "C" int gmr_pack_status(const gmr_pack* p, int* persistent, int* failed, int* phase) {
    return guarded([&] {
        if (!p) throw Error(GMR_ERR_ARG, "null pack");
        if (persistent) *persistent = p->last_persistent ? 1 : 0;
        if (failed) *failed = p->last_persistent ? p->status_host[0] : 0;
        if (phase) *phase = p->last_persistent ? p->status_host[1] : 0;
    });
}

extern "C" void gmr_pack_free(gmr_pack* p) {
    if (!p) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(p->device);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->levels_exec) cudaGraphExecDestroy(p->levels_exec);
    p->table.release();
    p->sync.release();
    if (p->status_host) cudaFreeHost(p->status_host);
    for (auto ev : p->join) cudaEventDestroy(ev);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->origin) cudaStreamDestroy(p->origin);
    if (prev >= 0) cudaSetDevice(prev);
    delete p;
}

// ------------------------------------------------------------------ gather-bandwidth calibration
// The sweep's dominant kernel gathers whole values (128 bytes at 32 fp32
// right-hand sides) at data-dependent addresses; its ceiling is the random
// gather bandwidth of the GPU, from L2 (a working set that fits) and from HBM
// (one that does not).  This calibration measures it with the same access
// pattern (unit indices hashed, taken modulo the buffer's unit count, so every
// access is in bounds) along three load paths:
//   * lane loads of 16 or 32 bytes, `depth` independent loads in flight per
//     thread (the sweep's own path; sequential mode reads the units in order);
//   * one bulk copy per unit into shared memory (cp.async.bulk completing on
//     an mbarrier), `depth` copies in flight per warp: the path a kernel that
//     stages values in shared memory would take.
namespace gmr {

__device__ __forceinline__ unsigned mix32(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

template <int W>
__device__ __forceinline__ float lane_load_sum(const unsigned char* p) {
    if constexpr (W == 16) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(p));
        return v.x + v.y + v.z + v.w;
    } else {
        float a0, a1, a2, a3, a4, a5, a6, a7;
        asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=f"(a0), "=f"(a1), "=f"(a2), "=f"(a3), "=f"(a4), "=f"(a5), "=f"(a6), "=f"(a7)
                     : "l"(p));
        return ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    }
}

// items units of (W << ushift) bytes; lane access ii reads part ii & (2^ushift - 1)
// of unit ii >> ushift.  DEPTH accesses per thread are issued before any is used.
template <int DEPTH, int W>
__global__ void __launch_bounds__(256) k_gather_units(const unsigned char* __restrict__ buf, unsigned nunits,
                                                      int ushift, int64_t items, bool sequential,
                                                      float* __restrict__ sink) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t total = items << ushift;
    const int64_t unit_bytes = (int64_t)W << ushift;
    const int64_t part_mask = ((int64_t)1 << ushift) - 1;
    float acc = 0.0f;
    for (int64_t i = t; i < total; i += DEPTH * stride) {
        float v[DEPTH];
#pragma unroll
        for (int j = 0; j < DEPTH; ++j) {
            const int64_t ii = i + j * stride;
            const unsigned ui = (unsigned)(ii >> ushift);
            const unsigned unit = (sequential ? ui : mix32(ui)) % nunits;
            v[j] = ii < total ? lane_load_sum<W>(buf + (int64_t)unit * unit_bytes + (ii & part_mask) * W) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < DEPTH; ++j) acc += v[j];
    }
    if (acc == 1.2345f) sink[t & 255] = acc;  // keeps the loads
}

static constexpr int kBulkMaxDepth = 64;

// Four warps per block; warp w of the grid gathers units gw, gw + nw, ...
// through two shared-memory stages of depth/2 units each.  One barrier phase
// covers a whole stage: lane 0 posts the stage's byte count, then lane j
// issues the bulk copy of the stage's unit j, so depth copies are in flight
// per warp and the barrier work is paid once per depth/2 copies.  A wait that
// gives up sets *err, drains the warp's copies still in flight (bounded) and
// returns.
__global__ void __launch_bounds__(128) k_gather_bulk(const unsigned char* __restrict__ buf, unsigned nunits,
                                                     int unit_bytes, int depth, int64_t items,
                                                     unsigned long long spin_limit, float* __restrict__ sink,
                                                     int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char ring_all[];
    __shared__ __align__(8) uint64_t bar[4][2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per = depth / 2;
    unsigned char* ring = ring_all + (size_t)warp * depth * unit_bytes;
    const int64_t gw = (int64_t)blockIdx.x * 4 + warp, nw = (int64_t)gridDim.x * 4;
    const int64_t mine = gw < items ? (items - gw + nw - 1) / nw : 0;
    const int64_t groups = (mine + per - 1) / per;
    if (lane == 0) {
        mbar_init(&bar[warp][0], 1);
        mbar_init(&bar[warp][1], 1);
        mbar_init_fence();
    }
    __syncwarp();
    auto issue = [&](int64_t g) {  // called by the whole warp
        const int s = (int)(g & 1);
        const int64_t k0 = g * per;
        const int n = (int)min((int64_t)per, mine - k0);
        if (lane == 0) mbar_arrive_expect_tx(&bar[warp][s], (uint32_t)(n * unit_bytes));
        __syncwarp();
        if (lane < n) {
            const unsigned unit = mix32((unsigned)(gw + (k0 + lane) * nw)) % nunits;
            bulk_g2s(ring + ((size_t)s * per + lane) * unit_bytes, buf + (int64_t)unit * unit_bytes,
                     (uint32_t)unit_bytes, &bar[warp][s]);
        }
    };
    int64_t issued = groups < 2 ? groups : 2;
    for (int64_t g = 0; g < issued; ++g) issue(g);
    float acc = 0.0f;
    for (int64_t g = 0; g < groups; ++g) {
        const int s = (int)(g & 1);
        const uint32_t parity = (uint32_t)((g >> 1) & 1);
        // lane 0 polls; __syncwarp then orders the other lanes' reads after
        // its observation of the completed phase
        int ok = 1;
        if (lane == 0) ok = mbar_wait(&bar[warp][s], parity, spin_limit) ? 1 : 0;
        __syncwarp();
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
            if (lane == 0) {
                atomicExch(err, 1);
                for (int64_t j = g; j < issued; ++j) mbar_wait(&bar[warp][j & 1], (uint32_t)((j >> 1) & 1), spin_limit);
            }
            __syncwarp();
            return;
        }
        const int n = (int)min((int64_t)per, mine - g * per);
        const float4* p = reinterpret_cast<const float4*>(ring + (size_t)s * per * unit_bytes);
        for (int q = lane; q < n * unit_bytes / 16; q += 32) {
            const float4 v = p[q];
            acc += v.x + v.y + v.z + v.w;
        }
        __syncwarp();  // every lane's reads of stage s have returned (they fed acc)
        if (g + 2 < groups) {
            issue(g + 2);
            ++issued;
        }
    }
    if (acc == 1.2345f) sink[(blockIdx.x * 128 + threadIdx.x) & 255] = acc;
}

template <int W>
static void launch_gather_units(int depth, int sms, const unsigned char* buf, unsigned nunits, int ushift,
                                int64_t items, bool seq, float* sink) {
    auto go = [&](auto kernel) {
        int per_sm = 0;
        GMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
        kernel<<<std::max(1, per_sm) * sms, 256>>>(buf, nunits, ushift, items, seq, sink);
    };
    switch (depth) {
        case 1: go(k_gather_units<1, W>); break;
        case 2: go(k_gather_units<2, W>); break;
        case 4: go(k_gather_units<4, W>); break;
        case 8: go(k_gather_units<8, W>); break;
        default: go(k_gather_units<16, W>); break;
    }
}

}  // namespace gmr

extern "C" int gmr_measure_gather(int device, int64_t buffer_bytes, int mode, int depth, int unit_bytes,
                                  float* gbs) {
    return guarded([&] {
        if (!gbs || buffer_bytes < 4096 || buffer_bytes > (int64_t)64 << 30) throw Error(GMR_ERR_ARG, "bad buffer size");
        if (mode < GMR_GATHER_LOAD16 || mode > GMR_GATHER_BULK) throw Error(GMR_ERR_ARG, "unknown gather mode");
        if (unit_bytes < 16 || (unit_bytes & (unit_bytes - 1)) || unit_bytes > 16384)
            throw Error(GMR_ERR_ARG, "unit_bytes must be a power of two in [16, 16384]");
        const bool bulk = mode == GMR_GATHER_BULK;
        const int W = mode == GMR_GATHER_LOAD32 ? 32 : 16;
        if (!bulk && (depth != 1 && depth != 2 && depth != 4 && depth != 8 && depth != 16))
            throw Error(GMR_ERR_ARG, "depth must be 1, 2, 4, 8 or 16 loads per thread");
        if (!bulk && unit_bytes < W) throw Error(GMR_ERR_ARG, "unit smaller than one lane access");
        if (bulk && (depth < 2 || depth > kBulkMaxDepth || depth % 2)) throw Error(GMR_ERR_ARG, "depth must be even, 2..64 copies");
        const size_t smem = bulk ? (size_t)4 * depth * unit_bytes : 0;
        if (smem > (size_t)200 * 1024) throw Error(GMR_ERR_RANGE, "4 warps x depth x unit_bytes beyond 200 KB");
        DeviceGuard dg(device);
        const int64_t units = buffer_bytes / unit_bytes;
        if (units < 1 || units > 0xffffffffLL) throw Error(GMR_ERR_ARG, "bad unit count");
        DevBuf buf, sink, errb;
        buf.ensure((size_t)units * unit_bytes);
        sink.ensure(1024);
        errb.ensure(16);
        GMR_CUDA(cudaMemset(buf.p, 0, (size_t)units * unit_bytes));
        GMR_CUDA(cudaMemset(errb.p, 0, 16));
        int sms = 152;
        GMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        const int64_t items = std::max<int64_t>(1, ((int64_t)6400 << 20) / unit_bytes);  // ~6.7 GB per timed run
        int ushift = 0;
        while ((W << ushift) < unit_bytes) ++ushift;
        const unsigned char* b = static_cast<const unsigned char*>(buf.p);
        float* sk = static_cast<float*>(sink.p);
        int* er = static_cast<int*>(errb.p);
        int bulk_blocks = 0;
        if (bulk) {
            GMR_CUDA(cudaFuncSetAttribute(k_gather_bulk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            GMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bulk_blocks, k_gather_bulk, 128, smem));
            if (bulk_blocks < 1) throw Error(GMR_ERR_RANGE, "bulk gather kernel cannot be resident");
            bulk_blocks *= sms;
        }
        auto run = [&](int64_t n) {
            if (bulk)
                k_gather_bulk<<<bulk_blocks, 128, smem>>>(b, (unsigned)units, unit_bytes, depth, n, 20000000ull, sk,
                                                           er);
            else if (W == 32)
                launch_gather_units<32>(depth, sms, b, (unsigned)units, ushift, n, mode == GMR_GATHER_SEQ16, sk);
            else
                launch_gather_units<16>(depth, sms, b, (unsigned)units, ushift, n, mode == GMR_GATHER_SEQ16, sk);
        };
        cudaEvent_t a, e;
        GMR_CUDA(cudaEventCreate(&a));
        GMR_CUDA(cudaEventCreate(&e));
        run(items / 10);
        float best = 0.0f;
        for (int r = 0; r < 3; ++r) {
            cudaEventRecord(a);
            run(items);
            cudaEventRecord(e);
            GMR_CUDA(cudaEventSynchronize(e));
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, a, e);
            best = std::max(best, (float)((double)items * unit_bytes / (ms * 1e6)));
        }
        cudaEventDestroy(a);
        cudaEventDestroy(e);
        GMR_CUDA(cudaGetLastError());
        int failed = 0;
        GMR_CUDA(cudaMemcpy(&failed, er, sizeof(int), cudaMemcpyDeviceToHost));
        if (failed) throw Error(GMR_ERR_TIMEOUT, "a bulk-copy wait gave up");
        *gbs = best;
    });
}

extern "C" int gmr_measure_gather_bandwidth(int device, int64_t buffer_bytes, int sequential, float* gbs) {
    return gmr_measure_gather(device, buffer_bytes, sequential ? GMR_GATHER_SEQ16 : GMR_GATHER_LOAD16, 4, 128, gbs);
}

// ------------------------------------------------------------------ no-allocation entry point
// For callers that may not allocate device memory while they run: the
// scratch values live in this statically sized device array instead of
// engine-owned cudaMalloc buffers; the schedule, X and Y are the caller's.
namespace gmr {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GMR_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device.  In host code the symbol
// name is only a host-side stand-in, so the address is looked up once per
// device with that device current.
static void* g_noalloc_addr[64] = {};
static std::mutex g_noalloc_mu;

// Every kernel the entry point can launch, for one semiring.  Querying a
// kernel's attributes loads its code onto the current device, so the set-up
// call below leaves nothing for a later call's first launch to load.
template <class S, int VEC, int GLOG>
static void noalloc_touch_one() {
    cudaFuncAttributes fa;
    GMR_CUDA(cudaFuncGetAttributes(&fa, k_prologue<S, VEC, GLOG>));
    GMR_CUDA(cudaFuncGetAttributes(&fa, k_level<S, VEC, GLOG, GMR_EMIT_ROWS>));
}
template <class S>
static void noalloc_touch() {
    noalloc_touch_one<S, 4, 0>();
    noalloc_touch_one<S, 4, 1>();
    noalloc_touch_one<S, 4, 2>();
    noalloc_touch_one<S, 4, 3>();
    noalloc_touch_one<S, 4, 4>();
    noalloc_touch_one<S, 4, 5>();
    noalloc_touch_one<S, 4, -1>();
    noalloc_touch_one<S, 2, 0>();
    noalloc_touch_one<S, 1, 0>();
    noalloc_touch_one<S, 1, -1>();
}

// Set-up, once per device with that device current: the array's device
// address, and the code of every kernel the entry point launches.
static void* noalloc_scratch_for_current_device() {
    int dev = -1;
    GMR_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw Error(GMR_ERR_RANGE, "device index beyond 63");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* ptr = nullptr;
        GMR_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        noalloc_touch<SPlus>();
        noalloc_touch<SBool>();
        noalloc_touch<STrop>();
        g_noalloc_addr[dev] = ptr;
    }
    return g_noalloc_addr[dev];
}

template <class S, int VEC, int GLOG>
static void noalloc_chain(const gmr_device_plan& p, void* arena, void* T, int Bw, int G, const void* X, void* Y,
                          cudaStream_t st, int sm_count) {
    SweepArgs a;
    a.arena = arena;
    a.T = T;
    a.Y = Y;
    a.X = X;
    a.V = p.V;
    a.term_val = p.term_val;
    a.term_col = p.term_col;
    a.n_terms = p.n_terms;
    a.n_ops = p.n_ops;
    a.rows = p.rows;
    a.ldx = Bw;
    a.ldy = Bw;
    a.Bt = Bw;
    a.G = G;
    a.t0 = 0;
    const int TPB = 256;
    auto blocks_for = [&](int64_t items) -> int {
        int64_t b = (items + TPB - 1) / TPB;
        return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm_count * 32));
    };
    k_prologue<S, VEC, GLOG><<<dim3(blocks_for((p.rows + p.n_terms) * (int64_t)G), 1), TPB, 0, st>>>(a);
    for (int k = 1; k <= p.depth + 1; ++k) {  // ops of level k (none for k = depth + 1), emissions of k - 1
        LevelArgs L{};
        L.ops = reinterpret_cast<const int2*>(p.ops);
        L.op_c = p.op_c;
        L.em_src = p.em_src;
        L.seg_row = p.seg_row;
        L.seg_start = p.seg_start;
        if (k <= p.depth) {
            L.op_first = p.lvl_off[k - 1];
            L.n_ops = p.lvl_off[k] - p.lvl_off[k - 1];
        }
        L.seg_first = p.seg_off[k - 1];
        L.n_seg = p.seg_off[k] - p.seg_off[k - 1];
        L.n_em = L.n_seg;
        if (L.n_ops == 0 && L.n_seg == 0) continue;
        const int eb = L.n_seg > 0 ? blocks_for(L.n_seg * G) : 0;
        const int ob = L.n_ops > 0 ? blocks_for((L.n_ops * G + 1) / 2) : 0;
        L.em_blocks = eb;
        k_level<S, VEC, GLOG, GMR_EMIT_ROWS><<<dim3(eb + ob, 1), TPB, 0, st>>>(a, L);
    }
    GMR_CUDA(cudaGetLastError());
}

template <class S>
static void noalloc_dispatch(const gmr_device_plan& p, void* arena, void* T, int Bw, const void* X, void* Y,
                             cudaStream_t st, int sm_count) {
    const bool a16 = ((uintptr_t)X % 16 == 0) && ((uintptr_t)Y % 16 == 0);
    const bool a8 = ((uintptr_t)X % 8 == 0) && ((uintptr_t)Y % 8 == 0);
    if (Bw % 4 == 0 && a16) {
        switch (Bw / 4) {
            case 1: return noalloc_chain<S, 4, 0>(p, arena, T, Bw, 1, X, Y, st, sm_count);
            case 2: return noalloc_chain<S, 4, 1>(p, arena, T, Bw, 2, X, Y, st, sm_count);
            case 4: return noalloc_chain<S, 4, 2>(p, arena, T, Bw, 4, X, Y, st, sm_count);
            case 8: return noalloc_chain<S, 4, 3>(p, arena, T, Bw, 8, X, Y, st, sm_count);
            case 16: return noalloc_chain<S, 4, 4>(p, arena, T, Bw, 16, X, Y, st, sm_count);
            case 32: return noalloc_chain<S, 4, 5>(p, arena, T, Bw, 32, X, Y, st, sm_count);
            default: return noalloc_chain<S, 4, -1>(p, arena, T, Bw, Bw / 4, X, Y, st, sm_count);
        }
    }
    if (Bw == 2 && a8) return noalloc_chain<S, 2, 0>(p, arena, T, Bw, 1, X, Y, st, sm_count);
    if (Bw == 1) return noalloc_chain<S, 1, 0>(p, arena, T, Bw, 1, X, Y, st, sm_count);
    return noalloc_chain<S, 1, -1>(p, arena, T, Bw, Bw, X, Y, st, sm_count);
}

}  // namespace gmr

extern "C" int gmr_multiply_noalloc(const gmr_device_plan* p, int semiring, const void* dX, void* dY, int B,
                                    void* stream) {
    return guarded([&] {
        if (!p) throw Error(GMR_ERR_ARG, "null plan");
        if (semiring < 0 || semiring > 2) throw Error(GMR_ERR_ARG, "unknown semiring");
        if (B < 1) throw Error(GMR_ERR_ARG, "B must be >= 1");
        if (p->depth < 0 || p->n_ops < 0 || p->n_terms < 1 || p->rows < 0 || p->cols < 1)
            throw Error(GMR_ERR_ARG, "bad plan sizes");
        if (!p->lvl_off || !p->seg_off || (p->n_ops > 0 && !p->ops) || !p->seg_start || (p->n_terms > 1 &&
            (!p->term_val || !p->term_col || !p->V)))
            throw Error(GMR_ERR_ARG, "null plan array");
        if ((!dX && p->cols > 0) || (!dY && p->rows > 0)) throw Error(GMR_ERR_ARG, "null X or Y");
        if (((uintptr_t)dX | (uintptr_t)dY) % 4 != 0 || (uintptr_t)p->ops % 8 != 0 || (uintptr_t)p->seg_start % 8 != 0)
            throw Error(GMR_ERR_ARG, "misaligned device pointer");
        if (p->lvl_off[0] != 0 || p->lvl_off[p->depth] != p->n_ops)
            throw Error(GMR_ERR_FORMAT, "level offsets do not cover the rules");
        for (int k = 1; k <= p->depth; ++k)
            if (p->lvl_off[k] < p->lvl_off[k - 1]) throw Error(GMR_ERR_FORMAT, "level offsets decrease");
        if (p->seg_off[0] != 0) throw Error(GMR_ERR_FORMAT, "row segment offsets do not start at 0");
        for (int k = 0; k <= p->depth; ++k)
            if (p->seg_off[k + 1] < p->seg_off[k]) throw Error(GMR_ERR_FORMAT, "row segment offsets decrease");
        if (p->seg_off[p->depth + 1] > 0 && (!p->em_src || !p->seg_row))
            throw Error(GMR_ERR_ARG, "null emission array (em_src or seg_row) with emissions present");
        if ((uintptr_t)p->op_c % 4 != 0 || (uintptr_t)p->em_src % 4 != 0 || (uintptr_t)p->seg_row % 4 != 0)
            throw Error(GMR_ERR_ARG, "misaligned device pointer");
        const int Bw = words_per_slot(semiring, B);
        const uint64_t arena_bytes = ((uint64_t)p->n_ops * Bw * 4 + 255) / 256 * 256;
        const uint64_t need = arena_bytes + (uint64_t)p->n_terms * Bw * 4;
        if (need > GMR_NOALLOC_SCRATCH_BYTES)
            throw Error(GMR_ERR_RANGE, "scratch of " + std::to_string(need) + " bytes ((n_ops + n_terms) x " +
                                           std::to_string(Bw) + " words x 4) exceeds the static " +
                                           std::to_string((unsigned long long)GMR_NOALLOC_SCRATCH_BYTES) +
                                           "-byte array; use gmr_engine_multiply");
        unsigned char* base = static_cast<unsigned char*>(noalloc_scratch_for_current_device());
        int dev = 0, sms = 152;
        GMR_CUDA(cudaGetDevice(&dev));
        GMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        void* arena = base;
        void* T = base + arena_bytes;
        if (semiring == GMR_PLUS_TIMES) noalloc_dispatch<SPlus>(*p, arena, T, Bw, dX, dY, st, sms);
        else if (semiring == GMR_BOOLEAN) noalloc_dispatch<SBool>(*p, arena, T, Bw, dX, dY, st, sms);
        else noalloc_dispatch<STrop>(*p, arena, T, Bw, dX, dY, st, sms);
    });
}

// ------------------------------------------------------------------ legacy ABI
// The reference's two entry points (gpu_engine.h:99-136).  Per call: relayout
// the given proper-layered schedule into a plan, upload, run `iters`
// multiplies timed with CUDA events, optionally measure energy with NVML,
// print the reference's stdout lines (gpu_engine.cu:279-280, 337-340, 546-547),
// copy Y back and free.  Semiring from SEMIRING (gpu_engine.cu:379-396).
// Errors print "CUDA Error: ..." and exit(1) like the reference's CUDA_CHECK.
namespace gmr {

static int semiring_from_env() {
    const char* s = std::getenv("SEMIRING");
    std::string v = s ? s : "plustimes";
    if (v == "boolean" || v == "bool") return GMR_BOOLEAN;
    if (v == "tropical" || v == "minplus") return GMR_TROPICAL;
    return GMR_PLUS_TIMES;
}

[[noreturn]] static void legacy_fail(const char* where, const std::string& msg) {
    std::cerr << "CUDA Error: " << msg << " at " << where << std::endl;
    std::exit(1);
}

// Converts the reference's float inputs to the engine's input words.
static void legacy_inputs(int semiring, const float* hx, int64_t n_vec, int B, std::vector<uint32_t>& words) {
    // hx layout: [cols][B] (B = 1 for the single-vector call)
    const int64_t cols = n_vec;
    if (semiring == GMR_PLUS_TIMES) {
        words.resize((size_t)(cols * B));
        std::memcpy(words.data(), hx, words.size() * 4);
    } else if (semiring == GMR_TROPICAL) {
        words.resize((size_t)(cols * B));
        for (int64_t i = 0; i < cols * B; ++i) {
            float f = hx[i];
            int32_t v = f >= 2147483647.0f ? INT32_MAX : (f <= -2147483648.0f ? INT32_MIN : (int32_t)f);
            words[i] = (uint32_t)v;
        }
    } else {
        const int W = (B + 31) / 32;
        words.assign((size_t)(cols * W), 0u);
        for (int64_t j = 0; j < cols; ++j)
            for (int b = 0; b < B; ++b)
                if (hx[j * B + b] != 0.0f) words[j * W + b / 32] |= 1u << (b % 32);
    }
}

static void legacy_outputs(int semiring, const std::vector<uint32_t>& words, int64_t rows, int B, float* hy) {
    if (semiring == GMR_BOOLEAN) {
        const int W = (B + 31) / 32;
        int32_t* y = reinterpret_cast<int32_t*>(hy);
        for (int64_t r = 0; r < rows; ++r)
            for (int b = 0; b < B; ++b) y[r * B + b] = (words[r * W + b / 32] >> (b % 32)) & 1u;
    } else {
        std::memcpy(hy, words.data(), (size_t)(rows * B) * 4);
    }
}

static void run_legacy(int rows, int cols, int alpha, int total_layered_rules, const LayeredRule* h_rules,
                       const int* h_val_indices, const int* h_col_indices, const float* h_V, int num_distinct_vals,
                       const float* h_X, const GPUSchedule& h_sched, float* h_Y, int B, int iters, bool batched) {
    const int semiring = semiring_from_env();
    if (!batched) {
        std::cout << "[GPU Setup Debug] rows=" << rows << ", cols=" << cols << ", alpha=" << alpha
                  << ", total_rules=" << total_layered_rules << ", distinct_vals=" << num_distinct_vals
                  << ", sched_max_depth=" << h_sched.max_depth << ", sched_max_width=" << h_sched.max_width
                  << ", emit_total=" << h_sched.emit_total << ", num_term_emit=" << h_sched.num_term_emit
                  << std::endl;
    }
    gmr_plan* plan = nullptr;
    if (gmr_plan_from_layered(rows, cols, alpha, total_layered_rules, h_rules, h_val_indices, h_col_indices, h_V,
                              num_distinct_vals, &h_sched, &plan) != GMR_OK)
        legacy_fail("gmr_plan_from_layered", gmr_last_error());
    size_t free0 = 0, total0 = 0;
    if (cudaMemGetInfo(&free0, &total0) != cudaSuccess) legacy_fail("cudaMemGetInfo", "no device");
    gmr_engine* eng = nullptr;
    if (gmr_engine_create(plan, 0, &eng) != GMR_OK) legacy_fail("gmr_engine_create", gmr_last_error());
    gmr_plan_free(plan);

    const int Bw = words_per_slot(semiring, B);
    std::vector<uint32_t> xw, yw((size_t)rows * Bw);
    legacy_inputs(semiring, h_X, cols, B, xw);
    DevBuf dX, dY;
    try {
        dX.ensure(xw.size() * 4);
        dY.ensure(yw.size() * 4);
        GMR_CUDA(cudaMemcpy(dX.p, xw.data(), xw.size() * 4, cudaMemcpyHostToDevice));
    } catch (const Error& e) {
        legacy_fail("setup", e.what());
    }
    // the reference's analytic device bytes (gpu_engine.cu:174-184)
    const size_t es = 4;
    size_t mem_analytic = (size_t)alpha * es + (size_t)total_layered_rules * 12 + (size_t)(alpha - 1) * 8 +
                          (size_t)num_distinct_vals * 4 + (size_t)cols * 4 + (size_t)rows * es +
                          (size_t)h_sched.max_width * es * 2 + (size_t)h_sched.emit_total * 8 +
                          (size_t)h_sched.num_term_emit * 8;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    gmr_config cfg{};
    // warm-up: builds the graph outside the timed window
    if (gmr_engine_multiply(eng, semiring, dX.p, dY.p, B, &cfg, nullptr) != GMR_OK)
        legacy_fail("gmr_engine_multiply", gmr_last_error());
    cudaEventRecord(t0, 0);
    for (int it = 0; it < iters; ++it)
        if (gmr_engine_multiply(eng, semiring, dX.p, dY.p, B, &cfg, nullptr) != GMR_OK)
            legacy_fail("gmr_engine_multiply", gmr_last_error());
    cudaEventRecord(t1, 0);
    if (cudaEventSynchronize(t1) != cudaSuccess) legacy_fail("cudaEventSynchronize", cudaGetErrorString(cudaGetLastError()));
    float total_ms = 0;
    cudaEventElapsedTime(&total_ms, t0, t1);
    if (!batched) {
        std::cout << "GPU kernel: " << total_ms << " ms total over " << iters << " vectors = "
                  << (total_ms / iters) << " ms/vector." << std::endl;
        size_t free1 = 0, total1 = 0;
        cudaMemGetInfo(&free1, &total1);
        size_t mem_peak = free0 > free1 ? free0 - free1 : 0;
        double mj = -1.0, mw = -1.0;
        const char* en = std::getenv("GMR_ENERGY");
        if (!(en && en[0] == '0')) {
            Nvml nv;
            if (nv.load() && nv.init() == 0) {
                void* dev = nullptr;
                if (nv.by_index(0, &dev) == 0) {
                    unsigned long long e0 = 0, e1 = 0;
                    int r0 = nv.energy(dev, &e0);
                    auto w0 = std::chrono::steady_clock::now();
                    long count = 0;
                    double el = 0;
                    do {  // re-run the multiply for >= 1.5 s (gpu_engine.cu:286-335)
                        for (int r = 0; r < 10; ++r, ++count)
                            gmr_engine_multiply(eng, semiring, dX.p, dY.p, B, &cfg, nullptr);
                        cudaDeviceSynchronize();
                        el = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
                    } while (el < 1.5);
                    int r1 = nv.energy(dev, &e1);
                    if (r0 == 0 && r1 == 0 && count > 0) {
                        mj = (double)(e1 - e0) / (double)count;
                        mw = (double)(e1 - e0) / el;
                    }
                }
                nv.shutdown();
            }
        }
        std::cout << "MEM analytic bytes: " << mem_analytic << std::endl;
        std::cout << "MEM peak bytes: " << mem_peak << std::endl;
        std::cout << "ENERGY mJ/vector: " << mj << std::endl;
        std::cout << "ENERGY avg power mW: " << mw << std::endl;
    } else {
        double per_batch = total_ms / iters, per_vec = per_batch / B;
        std::cout << "GPU batched (B=" << B << "): " << per_batch << " ms/batch, " << per_vec
                  << " ms/vector over " << iters << " batches." << std::endl;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (cudaMemcpy(yw.data(), dY.p, yw.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        legacy_fail("cudaMemcpy", cudaGetErrorString(cudaGetLastError()));
    legacy_outputs(semiring, yw, rows, B, h_Y);
    dX.release();
    dY.release();
    gmr_engine_free(eng);
}

}  // namespace gmr

extern "C" void run_gpu_right_multiply_layered(int rows, int cols, int alpha, int total_layered_rules,
                                               const LayeredRule* h_rules, const int* h_val_indices,
                                               const int* h_col_indices, const float* h_V, int num_distinct_vals,
                                               const float* h_x, const GPUSchedule& h_sched, float* h_y,
                                               int iters) {
    gmr::run_legacy(rows, cols, alpha, total_layered_rules, h_rules, h_val_indices, h_col_indices, h_V,
                    num_distinct_vals, h_x, h_sched, h_y, 1, iters < 1 ? 1 : iters, false);
}

extern "C" void run_gpu_right_multiply_batched(int rows, int cols, int alpha, int total_layered_rules,
                                               const LayeredRule* h_rules, const int* h_val_indices,
                                               const int* h_col_indices, const float* h_V, int num_distinct_vals,
                                               const float* h_X, const GPUSchedule& h_sched, float* h_Y, int B,
                                               int iters) {
    gmr::run_legacy(rows, cols, alpha, total_layered_rules, h_rules, h_val_indices, h_col_indices, h_V,
                    num_distinct_vals, h_X, h_sched, h_Y, B < 1 ? 1 : B, iters < 1 ? 1 : iters, true);
}
