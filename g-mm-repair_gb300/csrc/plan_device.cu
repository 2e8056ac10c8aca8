// Schedule builder on the GPU: the same plan as gmr_plan_build (plan.cpp),
// array for array, built with device-wide passes instead of host loops.
//
// Steps (each mirrors the host builder, which follows the reference's
// build_schedule.cpp:42-227):
//   1. levels lvl(N -> A B) = 1 + max(lvl A, lvl B) (build_schedule.cpp:57-71)
//      by relaxation rounds: rules are numbered children-first, every round
//      only raises a level towards its final value, so at most depth + 1
//      rounds run (the last finds nothing to change);
//   2. the reference's layered figures (pass-throughs, widths, E, E_T, U)
//      from one pass over the rules and one over C;
//   3. liveness (reachable from C), top-down level by level;
//   4. terminal compaction (ascending code) by an exclusive scan of flags;
//   5. per level, the live rules sorted by (left ref, right ref, rule index)
//      with a stable radix sort of packed 64-bit keys, which assigns the
//      arena slots the next level's keys refer to;
//   6. emissions: every C entry becomes one key (level, row, source) where
//      the row is a scan of the row delimiters; one radix sort puts them in
//      plan order; the row segments come from a scan of key changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "device_util.cuh"
#include "gmr_internal.h"
#include "sort.cuh"

namespace gmr {
namespace {

using dev::grid_for;
using dev::kThreads;

int bits_for(uint64_t x) { return x == 0 ? 0 : 64 - __builtin_clzll(x); }

#define GRID_STRIDE(i, n) \
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_fill_i32(int32_t* a, int64_t n, int32_t v) {
    GRID_STRIDE(i, n) a[i] = v;
}

// One relaxation round of the levels; *changed is set when a level rose.
__global__ void k_relax_levels(const int2* __restrict__ R, const int32_t* __restrict__ kind, int32_t alpha, int64_t n,
                              int32_t* lvl, int32_t* changed) {
    GRID_STRIDE(i, n) {
        const int2 c = R[i];
        int32_t l = c.x >= alpha ? lvl[c.x - alpha] : 0;
        if (kind[i] == 0 && c.y >= alpha) l = max(l, lvl[c.y - alpha]);
        if (l + 1 != lvl[i]) {
            lvl[i] = l + 1;
            *changed = 1;
        }
    }
}

__global__ void k_max_i32(const int32_t* __restrict__ a, int64_t n, int32_t* out) {
    int32_t m = 0;
    GRID_STRIDE(i, n) m = max(m, a[i]);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Highest level among the parents of each rule (starts as its own level).
__global__ void k_ref_parents(const int2* __restrict__ R, const int32_t* __restrict__ kind, int32_t alpha, int64_t n,
                              const int32_t* __restrict__ lvl, int32_t* mref, uint8_t* used_t) {
    GRID_STRIDE(i, n) {
        const int2 c = R[i];
        if (c.x >= alpha) atomicMax(&mref[c.x - alpha], lvl[i]);
        else used_t[c.x] = 1;
        if (kind[i] == 0) {
            if (c.y >= alpha) atomicMax(&mref[c.y - alpha], lvl[i]);
            else used_t[c.y] = 1;
        }
    }
}

// Level histograms: raw[k] rules of level k; carried symbols enter the
// reference's level lvl+1 and leave after mref (dp / dm); pt = sum of carries.
__global__ void k_ref_hist(const int32_t* __restrict__ lvl, const int32_t* __restrict__ mref, int64_t n, int nb,
                           unsigned long long* raw, unsigned long long* dp, unsigned long long* dm,
                           unsigned long long* pt) {
    extern __shared__ unsigned long long sh[];
    unsigned long long *hr = sh, *hp = sh + nb, *hm = sh + 2 * nb;
    for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    unsigned long long s = 0;
    GRID_STRIDE(i, n) {
        const int32_t a = lvl[i], m = mref[i];
        atomicAdd(&hr[a], 1ull);
        if (m > a) {
            atomicAdd(&hp[a + 1], 1ull);
            atomicAdd(&hm[m + 1], 1ull);
            s += (unsigned long long)(m - a);
        }
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(pt, s);
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        if (hr[b]) atomicAdd(&raw[b], hr[b]);
        if (hp[b]) atomicAdd(&dp[b], hp[b]);
        if (hm[b]) atomicAdd(&dm[b], hm[b]);
    }
}

// One pass over C: counts (E, E_T), terminal flags, live roots, delimiters.
__global__ void k_scan_c(const int32_t* __restrict__ C, int64_t nc, int32_t alpha, uint8_t* used_t, uint8_t* live,
                         uint32_t* tflag, uint32_t* delim, unsigned long long* counts) {
    unsigned long long e = 0, et = 0;
    GRID_STRIDE(p, nc) {
        const int32_t c = C[p];
        delim[p] = c == 0;
        if (c == 0) continue;
        if (c < alpha) {
            ++et;
            used_t[c] = 1;
            tflag[c] = 1;
        } else {
            ++e;
            live[c - alpha] = 1;
        }
    }
    for (int o = 16; o; o >>= 1) {
        e += __shfl_xor_sync(0xffffffffu, e, o);
        et += __shfl_xor_sync(0xffffffffu, et, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (e) atomicAdd(&counts[0], e);
        if (et) atomicAdd(&counts[1], et);
    }
}

__global__ void k_count_flags(const uint8_t* __restrict__ f, int64_t lo, int64_t hi, unsigned long long* out) {
    unsigned long long s = 0;
    GRID_STRIDE(i, hi - lo) s += f[lo + i] != 0;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

__global__ void k_keys_by_level(const int32_t* __restrict__ lvl, int64_t n, uint64_t* key, uint32_t* val) {
    GRID_STRIDE(i, n) {
        key[i] = (uint64_t)lvl[i];
        val[i] = (uint32_t)i;
    }
}

// Marks the children of the live rules of one level.
__global__ void k_live_level(const uint32_t* __restrict__ ids, int64_t cnt, const int2* __restrict__ R,
                             const int32_t* __restrict__ kind, int32_t alpha, uint8_t* live) {
    GRID_STRIDE(j, cnt) {
        const uint32_t i = ids[j];
        if (!live[i]) continue;
        const int2 c = R[i];
        if (c.x >= alpha) live[c.x - alpha] = 1;
        if (kind[i] == 0 && c.y >= alpha) live[c.y - alpha] = 1;
    }
}

// Live rules keyed by level (dead ones after the deepest level); terminal
// children of live rules flagged for the compaction.
__global__ void k_live_keys(const int32_t* __restrict__ lvl, const uint8_t* __restrict__ live, const int2* __restrict__ R,
                            const int32_t* __restrict__ kind, int32_t alpha, int64_t n, int32_t dead, uint64_t* key,
                            uint32_t* val, uint32_t* tflag) {
    GRID_STRIDE(i, n) {
        const bool L = live[i] != 0;
        key[i] = (uint64_t)(L ? lvl[i] : dead);
        val[i] = (uint32_t)i;
        if (L) {
            const int2 c = R[i];
            if (c.x < alpha) tflag[c.x] = 1;
            if (kind[i] == 0 && c.y < alpha) tflag[c.y] = 1;
        }
    }
}

// Compacted terminal q = tpos[t] + 1 for each flagged code t >= 1.
__global__ void k_terms(const uint32_t* __restrict__ tflag, const uint32_t* __restrict__ tpos, int32_t alpha,
                        int32_t cols, int64_t nv, int32_t* tmap, int32_t* term_val, int32_t* term_col, int32_t* bad_t) {
    GRID_STRIDE(t, (int64_t)alpha) {
        if (t == 0 || !tflag[t]) {
            tmap[t] = 0;
            continue;
        }
        const uint32_t q = tpos[t];
        tmap[t] = (int32_t)q + 1;
        const int64_t vi = (t - 1) / cols, ci = (t - 1) % cols;
        term_val[q] = (int32_t)vi;
        term_col[q] = (int32_t)ci;
        if (vi >= nv) atomicMin(bad_t, (int32_t)t);
    }
}

__device__ __forceinline__ int32_t sym_ref(int32_t s, int32_t alpha, const int32_t* slot, const int32_t* tmap) {
    return s >= alpha ? slot[s - alpha] : -tmap[s] - 1;
}

// Keys (left ref, right ref) of the live rules of one level.
__global__ void k_slot_keys(const uint32_t* __restrict__ ids, int64_t cnt, const int2* __restrict__ R,
                            const int32_t* __restrict__ kind, int32_t alpha, const int32_t* __restrict__ slot,
                            const int32_t* __restrict__ tmap, int64_t off, int b, uint64_t* key, uint32_t* val) {
    GRID_STRIDE(j, cnt) {
        const uint32_t i = ids[j];
        const int2 c = R[i];
        const int64_t L = sym_ref(c.x, alpha, slot, tmap), Rr = kind[i] == 0 ? sym_ref(c.y, alpha, slot, tmap) : -1;
        key[j] = ((uint64_t)(L + off) << b) | (uint64_t)(Rr + off);
        val[j] = i;
    }
}

__global__ void k_slot_assign(const uint64_t* __restrict__ key, const uint32_t* __restrict__ val, int64_t cnt,
                              int64_t base, int64_t off, int b, const int32_t* __restrict__ kind,
                              const int32_t* __restrict__ reps, int32_t* slot, int32_t* op_l, int32_t* op_r,
                              float* op_c) {
    const uint64_t mask = (1ull << b) - 1;
    GRID_STRIDE(j, cnt) {
        const uint32_t i = val[j];
        const uint64_t k = key[j];
        slot[i] = (int32_t)(base + j);
        op_l[base + j] = (int32_t)((int64_t)(k >> b) - off);
        op_r[base + j] = (int32_t)((int64_t)(k & mask) - off);
        if (op_c) op_c[base + j] = kind[i] ? (float)reps[i] : 1.0f;
    }
}

// first[v] = position of the first key whose bits [shift, 64) equal v, for
// keys sorted ascending (first[] starts at -1: values that do not occur).
__global__ void k_firsts(const uint64_t* __restrict__ key, int64_t n, int shift, int64_t nfirst, int64_t* first) {
    GRID_STRIDE(j, n) {
        const uint64_t v = key[j] >> shift;
        if ((j == 0 || (key[j - 1] >> shift) != v) && v < (uint64_t)nfirst) first[v] = j;
    }
}

// Offsets of groups 0..m-1 of sorted keys from their first positions: group v
// covers [off[v], off[v+1]); absent groups are empty; off[m] = end.
std::vector<int64_t> group_offsets(const std::vector<int64_t>& first, int64_t m, int64_t end) {
    std::vector<int64_t> off(m + 1, end);
    for (int64_t v = m - 1; v >= 0; --v) off[v] = first[v] >= 0 ? first[v] : off[v + 1];
    return off;
}

// One key per C entry: (level, row, source); row delimiters sort last.
__global__ void k_emit_keys(const int32_t* __restrict__ C, int64_t nc, int32_t alpha, const int32_t* __restrict__ lvl,
                            const int32_t* __restrict__ slot, const int32_t* __restrict__ tmap,
                            const uint32_t* __restrict__ rowpos, int32_t rows, int32_t dead, int sr, int sl,
                            int64_t off, uint64_t* key, int32_t* bad_row) {
    GRID_STRIDE(p, nc) {
        const int32_t c = C[p];
        if (c == 0) {
            key[p] = (uint64_t)dead << sl;
            continue;
        }
        const uint32_t row = rowpos[p];
        if ((int64_t)row >= rows) *bad_row = 1;
        const int32_t level = c < alpha ? 0 : lvl[c - alpha];
        const int64_t src = c < alpha ? -(int64_t)tmap[c] - 1 : (int64_t)slot[c - alpha];
        key[p] = ((uint64_t)level << sl) | ((uint64_t)row << sr) | (uint64_t)(src + off);
    }
}

// Unpacks sorted emission keys and flags the first emission of each
// (level, row) segment.
__global__ void k_emit_unpack(const uint64_t* __restrict__ key, int64_t ne, int sr, int sl, int64_t off,
                              int32_t* em_src, int32_t* em_row, uint32_t* segflag) {
    const uint64_t mr = (1ull << (sl - sr)) - 1, ms = (1ull << sr) - 1;
    GRID_STRIDE(e, ne) {
        const uint64_t k = key[e];
        em_src[e] = (int32_t)((int64_t)(k & ms) - off);
        em_row[e] = (int32_t)((k >> sr) & mr);
        segflag[e] = e == 0 || (k >> sr) != (key[e - 1] >> sr);
    }
}

__global__ void k_seg_fill(const uint64_t* __restrict__ key, const uint32_t* __restrict__ segflag,
                           const uint32_t* __restrict__ segidx, int64_t ne, int sr, int sl, int32_t* seg_row,
                           int64_t* seg_start) {
    const uint64_t mr = (1ull << (sl - sr)) - 1;
    GRID_STRIDE(e, ne) {
        if (!segflag[e]) continue;
        const uint32_t s = segidx[e];
        seg_row[s] = (int32_t)((key[e] >> sr) & mr);
        seg_start[s] = e;
    }
}

// out[j] = a[idx[j]] (idx and out may be the same array).
__global__ void k_gather_u32(const uint32_t* __restrict__ a, const int64_t* idx, int64_t n, int64_t* out) {
    GRID_STRIDE(j, n) out[j] = (int64_t)a[idx[j]];
}

template <class T>
void to_device(DevArray<T>& d, const T* h, int64_t n, cudaStream_t st) {
    d.alloc(n);
    if (n) GMR_CUDA(cudaMemcpyAsync(d.p, h, (size_t)n * sizeof(T), cudaMemcpyHostToDevice, st));
}

template <class T>
void to_host(std::vector<T>& h, const T* d, int64_t n, cudaStream_t st) {
    h.resize((size_t)n);
    if (n) GMR_CUDA(cudaMemcpyAsync(h.data(), d, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, st));
}

template <class T>
T read1(const T* d, cudaStream_t st) {
    T v;
    GMR_CUDA(cudaMemcpyAsync(&v, d, sizeof(T), cudaMemcpyDeviceToHost, st));
    GMR_CUDA(cudaStreamSynchronize(st));
    return v;
}

template <class T>
std::vector<T> read_n(const T* d, int64_t n, cudaStream_t st) {
    std::vector<T> v((size_t)n);
    if (n) GMR_CUDA(cudaMemcpyAsync(v.data(), d, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, st));
    GMR_CUDA(cudaStreamSynchronize(st));
    return v;
}

// Holds the stream of one build; destroys it on scope exit.
struct Stream {
    cudaStream_t s = nullptr;
    Stream() { GMR_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~Stream() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

#define LAUNCH(kernel, n, smem, ...)                                                   \
    do {                                                                               \
        kernel<<<grid_for(n), kThreads, (smem), st>>>(__VA_ARGS__);                    \
        GMR_CUDA(cudaGetLastError());                                                  \
    } while (0)

std::unique_ptr<gmr_plan> build_on_device(const gmr_grammar& g, int rows, int cols, cudaStream_t st) {
    const int32_t alpha = g.alpha;
    const int64_t n = g.n_rules(), nc = (int64_t)g.C.size(), nv = (int64_t)g.V.size();
    if (n >= (int64_t)INT32_MAX || nc >= (int64_t)UINT32_MAX - 1)
        throw Error(GMR_ERR_RANGE, "device schedule build: grammar too large");
    auto p = std::make_unique<gmr_plan>();
    p->rows = rows;
    p->cols = cols;
    p->V.assign(g.V.begin(), g.V.end());

    DevArray<int2> R;
    DevArray<int32_t> kind, reps, C;
    to_device(R, reinterpret_cast<const int2*>(g.rules.data()), n, st);
    to_device(kind, g.kinds.data(), n, st);
    if (g.has_runlen) to_device(reps, g.reps.data(), n, st);
    to_device(C, g.C.data(), nc, st);

    DevArray<unsigned long long> acc(8);  // changed/max, E, E_T, pt, U_ref
    DevArray<int32_t> flag(4);
    // (1) levels
    DevArray<int32_t> lvl(n);
    LAUNCH(k_fill_i32, n, 0, lvl.p, n, 1);
    for (int64_t round = 0;; ++round) {
        if (round > n + 1) throw Error(GMR_ERR_FORMAT, "device schedule build: levels do not settle");
        GMR_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int32_t), st));
        LAUNCH(k_relax_levels, n, 0, R.p, kind.p, alpha, n, lvl.p, flag.p);
        if (read1(flag.p, st) == 0) break;
    }
    GMR_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int32_t), st));
    LAUNCH(k_max_i32, n, 0, lvl.p, n, flag.p);
    const int depth = read1(flag.p, st);
    p->depth = depth;
    const int nb = depth + 2;

    // (2) the reference's layered figures
    DevArray<uint8_t> used_t(alpha), live(n);
    DevArray<uint32_t> tflag(alpha), delim(nc + 1);
    GMR_CUDA(cudaMemsetAsync(used_t.p, 0, (size_t)alpha, st));
    GMR_CUDA(cudaMemsetAsync(live.p, 0, (size_t)std::max<int64_t>(n, 1), st));
    GMR_CUDA(cudaMemsetAsync(tflag.p, 0, (size_t)alpha * 4, st));
    GMR_CUDA(cudaMemsetAsync(acc.p, 0, 8 * sizeof(unsigned long long), st));
    DevArray<unsigned long long> hist(3 * (int64_t)nb);
    GMR_CUDA(cudaMemsetAsync(hist.p, 0, 3 * (size_t)nb * 8, st));
    {
        DevArray<int32_t> mref(n);
        if (n) GMR_CUDA(cudaMemcpyAsync(mref.p, lvl.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
        LAUNCH(k_ref_parents, n, 0, R.p, kind.p, alpha, n, lvl.p, mref.p, used_t.p);
        const size_t smem = 3 * (size_t)nb * 8;
        if (smem > 96 * 1024) throw Error(GMR_ERR_RANGE, "device schedule build: grammar too deep");
        if (smem > 48 * 1024)
            GMR_CUDA(cudaFuncSetAttribute(k_ref_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        LAUNCH(k_ref_hist, n, smem, lvl.p, mref.p, n, nb, hist.p, hist.p + nb, hist.p + 2 * nb, acc.p + 3);
    }
    LAUNCH(k_scan_c, nc, 0, C.p, nc, alpha, used_t.p, live.p, tflag.p, delim.p, acc.p + 1);
    if (alpha > 1) LAUNCH(k_count_flags, alpha - 1, 0, used_t.p, 1, alpha, acc.p + 4);
    {
        const auto a = read_n(acc.p, 8, st);
        const auto h = read_n(hist.p, 3 * (int64_t)nb, st);
        int64_t run = 0, wmax = 0;
        for (int k = 1; k <= depth; ++k) {
            run += (int64_t)h[nb + k] - (int64_t)h[2 * nb + k];
            wmax = std::max<int64_t>(wmax, (int64_t)h[k] + run);
        }
        auto& s = p->stats;
        s.ref_raw = n;
        s.ref_passthrough = (int64_t)a[3];
        s.ref_layered = n + (int64_t)a[3];
        s.ref_max_width = wmax;
        s.ref_emit = (int64_t)a[1];
        s.ref_term_emit = (int64_t)a[2];
        s.ref_alpha = 1 + (int64_t)a[4];
    }
    used_t.alloc(0);

    // levels of all rules, ascending rule index within a level
    const int64_t sort_words = dev::sort_scratch(std::max<int64_t>(n, nc));
    DevArray<uint32_t> tmp(std::max<int64_t>(sort_words, dev::scan_scratch(std::max<int64_t>(nc, alpha)) + 1));
    DevArray<uint64_t> ka(n), kb(n);
    DevArray<uint32_t> va(n), vb(n);
    uint64_t *k1 = ka.p, *k2 = kb.p;
    uint32_t *v1 = va.p, *v2 = vb.p;
    std::vector<int64_t> raw_off(depth + 1, 0);
    {
        const auto h = read_n(hist.p, nb, st);
        for (int k = 1; k <= depth; ++k) raw_off[k] = raw_off[k - 1] + (int64_t)h[k];
    }
    LAUNCH(k_keys_by_level, n, 0, lvl.p, n, k1, v1);
    dev::radix_sort(k1, k2, v1, v2, n, bits_for((uint64_t)depth), tmp.p, st);
    // (3) liveness, deepest level first
    for (int k = depth; k >= 1; --k) {
        const int64_t cnt = raw_off[k] - raw_off[k - 1];
        if (cnt) LAUNCH(k_live_level, cnt, 0, v1 + raw_off[k - 1], cnt, R.p, kind.p, alpha, live.p);
    }
    // live rules by level; terminal flags of live rules
    k1 = ka.p, k2 = kb.p, v1 = va.p, v2 = vb.p;
    LAUNCH(k_live_keys, n, 0, lvl.p, live.p, R.p, kind.p, alpha, n, depth + 1, k1, v1, tflag.p);
    dev::radix_sort(k1, k2, v1, v2, n, bits_for((uint64_t)depth + 1), tmp.p, st);
    DevArray<int64_t> first(nb + 1);
    GMR_CUDA(cudaMemsetAsync(first.p, 0xff, (size_t)(nb + 1) * 8, st));
    LAUNCH(k_firsts, n, 0, k1, n, 0, (int64_t)nb, first.p);
    std::vector<int64_t> lvl_off;
    {
        // live levels are 1..depth; key depth + 1 marks the dead rules
        const auto f = read_n(first.p, nb, st);
        int64_t nlive = f[depth + 1] >= 0 ? f[depth + 1] : n;
        auto o = group_offsets(f, depth + 1, nlive);  // o[k] = start of level k
        lvl_off.assign(depth + 1, 0);
        for (int k = 1; k <= depth; ++k) lvl_off[k] = o[k + 1];
    }
    live.alloc(0);

    // (4) compacted terminals
    DevArray<uint32_t> tpos(alpha + 1);
    dev::exclusive_scan(tflag.p, tpos.p, alpha, tmp.p, st);
    const int64_t U = 1 + (int64_t)read1(tpos.p + alpha, st);
    DevArray<int32_t> tmap(alpha), term_val(U), term_col(U);
    GMR_CUDA(cudaMemsetAsync(flag.p, 0x7f, sizeof(int32_t), st));
    LAUNCH(k_terms, alpha, 0, tflag.p, tpos.p, alpha, cols, nv, tmap.p, term_val.p, term_col.p, flag.p);
    {
        const int32_t bad = read1(flag.p, st);
        if (bad != 0x7f7f7f7f) throw Error(GMR_ERR_FORMAT, "terminal " + std::to_string(bad) + " has no value");
    }
    tflag.alloc(0);
    tpos.alloc(0);

    // (5) arena slots, level by level
    const int64_t n_ops = lvl_off[depth];
    if (n_ops > INT32_MAX) throw Error(GMR_ERR_RANGE, "more than 2^31 ops");
    const int64_t off = U + 1;
    const int b = bits_for((uint64_t)(n_ops + U));
    if (2 * b > 64) throw Error(GMR_ERR_RANGE, "device schedule build: rule keys exceed 64 bits");
    DevArray<int32_t> slot(n), op_l(n_ops), op_r(n_ops);
    DevArray<float> op_c(g.has_runlen ? n_ops : 0);
    GMR_CUDA(cudaMemsetAsync(slot.p, 0xff, (size_t)std::max<int64_t>(n, 1) * 4, st));
    {
        // live rule ids grouped by level; ka/kb and va/vb become sort buffers
        DevArray<uint32_t> ids(n_ops);
        if (n_ops) GMR_CUDA(cudaMemcpyAsync(ids.p, v1, (size_t)n_ops * 4, cudaMemcpyDeviceToDevice, st));
        for (int k = 1; k <= depth; ++k) {
            const int64_t base = lvl_off[k - 1], cnt = lvl_off[k] - base;
            if (!cnt) continue;
            uint64_t *x1 = ka.p, *x2 = kb.p;
            uint32_t *y1 = va.p, *y2 = vb.p;
            LAUNCH(k_slot_keys, cnt, 0, ids.p + base, cnt, R.p, kind.p, alpha, slot.p, tmap.p, off, b, x1, y1);
            dev::radix_sort(x1, x2, y1, y2, cnt, 2 * b, tmp.p, st);
            LAUNCH(k_slot_assign, cnt, 0, x1, y1, cnt, base, off, b, kind.p, reps.p, slot.p, op_l.p, op_r.p,
                   g.has_runlen ? op_c.p : nullptr);
        }
    }
    ka.alloc(0);
    kb.alloc(0);
    va.alloc(0);
    vb.alloc(0);
    p->lvl_off = lvl_off;
    to_host(p->op_l, op_l.p, n_ops, st);
    to_host(p->op_r, op_r.p, n_ops, st);
    if (g.has_runlen) to_host(p->op_c, op_c.p, n_ops, st);
    to_host(p->term_val, term_val.p, U - 1, st);
    to_host(p->term_col, term_col.p, U - 1, st);

    // (6) emissions
    const int sr = b, br = bits_for((uint64_t)std::max(rows, 0)), sl = sr + br;
    const int bd = bits_for((uint64_t)depth + 1);
    if (sl + bd > 64) throw Error(GMR_ERR_RANGE, "device schedule build: emission keys exceed 64 bits");
    dev::exclusive_scan(delim.p, delim.p, nc, tmp.p, st);  // row of each entry
    const int64_t nzero = (int64_t)read1(delim.p + nc, st);
    const int64_t ne = nc - nzero;
    DevArray<uint64_t> ea(nc), eb(nc);
    GMR_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int32_t), st));
    LAUNCH(k_emit_keys, nc, 0, C.p, nc, alpha, lvl.p, slot.p, tmap.p, delim.p, rows, depth + 1, sr, sl, off, ea.p,
           flag.p);
    if (read1(flag.p, st)) throw Error(GMR_ERR_FORMAT, "C holds more rows than rows=" + std::to_string(rows));
    delim.alloc(0);
    C.alloc(0);
    uint64_t *e1 = ea.p, *e2 = eb.p;
    uint32_t *nv1 = nullptr, *nv2 = nullptr;
    dev::radix_sort(e1, e2, nv1, nv2, nc, sl + bd, tmp.p, st);
    DevArray<int32_t> em_src(ne), em_row(ne);
    DevArray<uint32_t> segflag(ne + 1);
    LAUNCH(k_emit_unpack, ne, 0, e1, ne, sr, sl, off, em_src.p, em_row.p, segflag.p);
    to_host(p->em_src, em_src.p, ne, st);
    to_host(p->em_row, em_row.p, ne, st);
    DevArray<uint32_t> segidx(ne + 1);
    dev::exclusive_scan(segflag.p, segidx.p, ne, tmp.p, st);
    const int64_t nseg = (int64_t)read1(segidx.p + ne, st);
    DevArray<int32_t> seg_row(nseg);
    DevArray<int64_t> seg_start(nseg + 1);
    LAUNCH(k_seg_fill, ne, 0, e1, segflag.p, segidx.p, ne, sr, sl, seg_row.p, seg_start.p);
    to_host(p->seg_row, seg_row.p, nseg, st);
    to_host(p->seg_start, seg_start.p, nseg, st);
    p->seg_start.push_back(ne);
    // level k's emissions start at the first key of level k; its segments at
    // the segment index of that emission
    GMR_CUDA(cudaMemsetAsync(first.p, 0xff, (size_t)(nb + 1) * 8, st));
    LAUNCH(k_firsts, ne, 0, e1, ne, sl, (int64_t)depth + 1, first.p);
    const auto f = read_n(first.p, depth + 1, st);
    p->em_off = group_offsets(f, depth + 1, ne);
    DevArray<int64_t> pos(depth + 2);
    GMR_CUDA(cudaMemcpyAsync(pos.p, p->em_off.data(), (size_t)(depth + 2) * 8, cudaMemcpyHostToDevice, st));
    LAUNCH(k_gather_u32, depth + 2, 0, segidx.p, pos.p, depth + 2, pos.p);
    p->seg_off = read_n(pos.p, depth + 2, st);
    GMR_CUDA(cudaStreamSynchronize(st));
    fill_common_stats(*p);
    return p;
}

}  // namespace
}  // namespace gmr

using namespace gmr;

extern "C" int gmr_plan_build_device(const gmr_grammar* g, int rows, int cols, int device, int validate,
                                     gmr_plan** out) {
    return guarded([&] {
        if (!g || !out || rows < 0 || cols < 1) throw Error(GMR_ERR_ARG, "bad argument");
        DeviceGuard dg(device);
        std::unique_ptr<gmr_plan> p;
        {
            Stream s;
            p = build_on_device(*g, rows, cols, s.s);
        }
        if (validate) validate_plan(*p);
        *out = p.release();
    });
}
