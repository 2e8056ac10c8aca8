// RePair on the GPU: the same rounds as gmr_repair_compress (repair.cpp), and
// the same grammar, rule for rule, built with device-wide scans and sorts.
//
// One round over the current string s (row delimiter 0 is a barrier):
//   1. pair keys (x, y) at every position; the counted occurrences skip every
//      second pair of a run "aaa" (RePair counts non-overlapping ones): a
//      pair inside a run of equal symbols is counted when its distance to the
//      run's first symbol is even (run starts by a running-maximum scan);
//      after the first round only pairs that hold a symbol of the previous
//      round or were candidates then can reach a count of two, and only they
//      go on (a compaction);
//   2. one stable radix sort of (key, position) groups the occurrences of each
//      pair; per distinct pair, its count is a difference of a prefix sum;
//   3. candidates (count >= 2) ranked by (count desc, key asc) with a second
//      radix sort; the rank is scattered back to every position;
//   4. the host's left-to-right greedy scan ("replace at i when rank(i) is at
//      least as good as rank(i+1), then skip i+1") resolves in parallel: in a
//      maximal run of positions that want to replace, the choices alternate
//      from the run's first position (running maximum of run starts again);
//   5. pairs chosen at least twice become rules numbered in rank order; the
//      string is rewritten by one compaction.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "device_util.cuh"
#include "gmr_internal.h"
#include "sort.cuh"

namespace gmr {
namespace {

using dev::grid_for;
using dev::kThreads;

constexpr uint32_t NONE = 0xffffffffu;

int bits_of(uint64_t x) { return x == 0 ? 0 : 64 - __builtin_clzll(x); }

#define GRID_STRIDE(i, n) \
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// First index of the run of equal symbols containing i (candidate: i when a
// run starts there, else 0; a running maximum completes it).
__global__ void k_eq_run_marks(const int32_t* __restrict__ s, int64_t n, uint32_t* mark) {
    GRID_STRIDE(i, n) mark[i] = (i == 0 || s[i] != s[i - 1]) ? (uint32_t)i : 0u;
}

// Key of the pair at every position, whether it is a counted
// (non-overlapping) occurrence, and whether it can reach a count of two this
// round (rel).  After the first round a pair can only do so when it holds a
// symbol made by the previous round (>= fresh) or was a candidate then
// (cand): occurrences of an older pair only ever disappear.
__global__ void k_pair_keys(const int32_t* __restrict__ s, int64_t n, const uint32_t* __restrict__ eq_start, int b,
                            int32_t fresh, const uint8_t* __restrict__ cand, uint64_t* key, uint8_t* counted,
                            uint32_t* rel) {
    GRID_STRIDE(i, n) {
        bool valid = false, cnt = false, r = false;
        if (i + 1 < n) {
            const int32_t x = s[i], y = s[i + 1];
            valid = x != 0 && y != 0;
            cnt = valid && (x != y || ((i - (int64_t)eq_start[i]) & 1) == 0);
            r = valid && (cand == nullptr || x >= fresh || y >= fresh || cand[i]);
            key[i] = ((uint64_t)(uint32_t)x << b) | (uint32_t)y;
        }
        counted[i] = cnt;
        rel[i] = r;
    }
}

// The relevant pairs, compacted (keys and positions) in position order.
__global__ void k_pick_pairs(const uint64_t* __restrict__ key, const uint32_t* __restrict__ rel,
                             const uint32_t* __restrict__ rpos, int64_t n, uint64_t* ko, uint32_t* po) {
    GRID_STRIDE(i, n) {
        if (!rel[i]) continue;
        ko[rpos[i]] = key[i];
        po[rpos[i]] = (uint32_t)i;
    }
}

// Over the sorted occurrences [0, nv): start of each distinct pair, and the
// counted flag in sorted order.
__global__ void k_groups(const uint64_t* __restrict__ key, const uint32_t* __restrict__ pos,
                         const uint8_t* __restrict__ counted, int64_t nv, uint32_t* start_flag, uint32_t* cflag) {
    GRID_STRIDE(j, nv) {
        start_flag[j] = j == 0 || key[j] != key[j - 1];
        cflag[j] = counted[pos[j]];
    }
}

// Distinct pair u: first occurrence ustart[u], key ukey[u].
__global__ void k_group_fill(const uint64_t* __restrict__ key, const uint32_t* __restrict__ start_flag,
                             const uint32_t* __restrict__ gidx, int64_t nv, uint32_t* ustart, uint64_t* ukey) {
    GRID_STRIDE(j, nv) {
        if (!start_flag[j]) continue;
        const uint32_t u = gidx[j];
        ustart[u] = (uint32_t)j;
        ukey[u] = key[j];
    }
}

// Ranking key of each distinct pair: (count desc, key asc) for candidates
// (count >= 2), all ones otherwise.  Distinct pairs are in ascending key order,
// so u stands for the key.
__global__ void k_rank_keys(const uint32_t* __restrict__ ustart, const uint32_t* __restrict__ cpre, int64_t nu,
                            int64_t nv, int bu, uint64_t* rkey, uint32_t* rval, unsigned long long* n_cand) {
    unsigned long long nc = 0;
    GRID_STRIDE(u, nu) {
        const uint32_t a = ustart[u], b = u + 1 < nu ? ustart[u + 1] : (uint32_t)nv;
        const uint32_t c = cpre[b] - cpre[a];
        const bool cand = c >= 2;
        rkey[u] = cand ? (((uint64_t)(0x80000000u - c) << bu) | (uint64_t)u) : ~0ull;
        rval[u] = (uint32_t)u;
        nc += cand;
    }
    for (int o = 16; o; o >>= 1) nc += __shfl_xor_sync(0xffffffffu, nc, o);
    if ((threadIdx.x & 31) == 0 && nc) atomicAdd(n_cand, nc);
}

__global__ void k_fill_u32(uint32_t* a, int64_t n, uint32_t v) {
    GRID_STRIDE(i, n) a[i] = v;
}

__global__ void k_rank_of(const uint32_t* __restrict__ rval, int64_t ncand, uint32_t* rank_of) {
    GRID_STRIDE(r, ncand) rank_of[rval[r]] = (uint32_t)r;
}

// Rank of the pair at every position (positions without a candidate keep NONE).
__global__ void k_rank_at(const uint32_t* __restrict__ pos, const uint32_t* __restrict__ start_flag,
                          const uint32_t* __restrict__ gidx, const uint32_t* __restrict__ rank_of, int64_t nv,
                          uint32_t* rank_pos) {
    GRID_STRIDE(j, nv) {
        const uint32_t u = gidx[j] + start_flag[j] - 1;
        rank_pos[pos[j]] = rank_of[u];
    }
}

// Positions that want to replace, and the start candidates of their runs.
__global__ void k_want(const uint32_t* __restrict__ rank_pos, int64_t n, uint8_t* want, uint32_t* mark) {
    GRID_STRIDE(i, n) {
        const uint32_t r = rank_pos[i], rn = i + 1 < n ? rank_pos[i + 1] : NONE;
        const bool w = r != NONE && r <= rn;
        bool wp = false;
        if (i > 0) {
            const uint32_t rp = rank_pos[i - 1];
            wp = rp != NONE && rp <= r;
        }
        want[i] = w;
        mark[i] = (w && !wp) ? (uint32_t)i : 0u;
    }
}

// chosen[i]: the greedy scan replaces the pair at i.
__global__ void k_choose(const uint8_t* __restrict__ want, const uint32_t* __restrict__ wstart, int64_t n,
                         uint8_t* chosen) {
    GRID_STRIDE(i, n) chosen[i] = want[i] && ((i - (int64_t)wstart[i]) & 1) == 0;
}

__global__ void k_chosen_sorted(const uint32_t* __restrict__ pos, const uint8_t* __restrict__ chosen, int64_t nv,
                                uint32_t* f) {
    GRID_STRIDE(j, nv) f[j] = chosen[pos[j]];
}

// Candidates (in rank order) chosen at least twice are accepted.
__global__ void k_accept(const uint32_t* __restrict__ rval, const uint32_t* __restrict__ ustart,
                         const uint32_t* __restrict__ upre, int64_t ncand, int64_t nu, int64_t nv, uint32_t* acc) {
    GRID_STRIDE(r, ncand) {
        const uint32_t u = rval[r];
        const uint32_t a = ustart[u], b = u + 1 < nu ? ustart[u + 1] : (uint32_t)nv;
        acc[r] = upre[b] - upre[a] >= 2;
    }
}

// Rules of the accepted candidates, in rank order.
__global__ void k_new_rules(const uint32_t* __restrict__ rval, const uint64_t* __restrict__ ukey,
                            const uint32_t* __restrict__ acc, const uint32_t* __restrict__ apre, int64_t ncand, int b,
                            int32_t* rules) {
    const uint64_t mask = (1ull << b) - 1;
    GRID_STRIDE(r, ncand) {
        if (!acc[r]) continue;
        const uint64_t k = ukey[rval[r]];
        rules[2 * (int64_t)apre[r]] = (int32_t)(k >> b);
        rules[2 * (int64_t)apre[r] + 1] = (int32_t)(k & mask);
    }
}

// Rewritten symbol at each position and whether it survives.
__global__ void k_rewrite(const int32_t* __restrict__ s, int64_t n, const uint8_t* __restrict__ chosen,
                          const uint32_t* __restrict__ rank_pos, const uint32_t* __restrict__ acc,
                          const uint32_t* __restrict__ apre, int32_t next, int32_t* sym, uint32_t* keep) {
    GRID_STRIDE(i, n) {
        const bool here = chosen[i] && acc[rank_pos[i]];
        const bool gone = i > 0 && chosen[i - 1] && acc[rank_pos[i - 1]];
        sym[i] = here ? next + (int32_t)apre[rank_pos[i]] : s[i];
        keep[i] = !gone;
    }
}

// Compaction of the rewritten string; the candidate flag of each surviving
// position goes along (for the next round's relevant pairs).
__global__ void k_compact(const int32_t* __restrict__ sym, const uint32_t* __restrict__ keep,
                          const uint32_t* __restrict__ kpre, const uint32_t* __restrict__ rank_pos, int64_t n,
                          int32_t* out, uint8_t* cand_out) {
    GRID_STRIDE(i, n) {
        if (!keep[i]) continue;
        out[kpre[i]] = sym[i];
        cand_out[kpre[i]] = rank_pos[i] != NONE;
    }
}

template <class T>
T read1(const T* d, cudaStream_t st) {
    T v;
    GMR_CUDA(cudaMemcpyAsync(&v, d, sizeof(T), cudaMemcpyDeviceToHost, st));
    GMR_CUDA(cudaStreamSynchronize(st));
    return v;
}

#define LAUNCH(kernel, n, ...)                                          \
    do {                                                                \
        kernel<<<grid_for(n), kThreads, 0, st>>>(__VA_ARGS__);          \
        GMR_CUDA(cudaGetLastError());                                   \
    } while (0)

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

}  // namespace
}  // namespace gmr

using namespace gmr;

extern "C" int gmr_repair_compress_device(const gmr_csrv* m, int device, gmr_grammar** out) {
    return guarded([&] {
        if (!m || !out) throw Error(GMR_ERR_ARG, "null argument");
        const int64_t alpha64 = (int64_t)m->V.size() * m->cols + 1;
        if (alpha64 > INT32_MAX) throw Error(GMR_ERR_RANGE, "terminal space exceeds int32");
        const int32_t alpha = (int32_t)alpha64;
        int64_t n = (int64_t)m->codes.size();
        if (n >= (int64_t)UINT32_MAX - 1) throw Error(GMR_ERR_RANGE, "device RePair: string longer than 2^32");
        DeviceGuard dg(device);
        Stream stream;
        cudaStream_t st = stream.s;
        const bool verbose = std::getenv("GMR_VERBOSE") != nullptr;

        const int64_t cap = std::max<int64_t>(n, 1);
        DevArray<int32_t> s(cap), s2(cap);
        if (n) GMR_CUDA(cudaMemcpyAsync(s.p, m->codes.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
        DevArray<uint64_t> ka(cap), kb(cap);
        DevArray<uint32_t> pa(cap), pb(cap), w1(cap + 1), w2(cap + 1), w3(cap + 1);
        DevArray<uint8_t> counted(cap), chosen(cap), want(cap), cand(cap), cand2(cap);
        int32_t fresh = alpha;  // first symbol made by the previous round
        DevArray<uint32_t> tmp(std::max(dev::sort_scratch(cap), dev::scan_scratch(cap + 1)) + 1);
        DevArray<unsigned long long> cnt(4);
        std::vector<int32_t> rules;           // host copy, appended per round
        DevArray<int32_t> new_rules(0);

        for (int round = 0; round < 100000 && n > 1; ++round) {
            auto t0 = std::chrono::steady_clock::now();
            const int64_t maxsym = (int64_t)alpha + (int64_t)rules.size() / 2;
            const int b = bits_of((uint64_t)maxsym + 1);
            if (2 * b > 64) throw Error(GMR_ERR_RANGE, "device RePair: pair keys exceed 64 bits");
            // (1) run starts of equal symbols, pair keys, counted occurrences,
            // and the pairs that can be candidates, compacted
            LAUNCH(k_eq_run_marks, n, s.p, n, w1.p);
            dev::inclusive_max_scan(w1.p, w1.p, n, tmp.p, st);
            GMR_CUDA(cudaMemsetAsync(cnt.p, 0, 4 * 8, st));
            LAUNCH(k_pair_keys, n, s.p, n, w1.p, b, fresh, round == 0 ? nullptr : cand.p, ka.p, counted.p, w2.p);
            dev::exclusive_scan(w2.p, w3.p, n, tmp.p, st);
            const int64_t nv = (int64_t)read1(w3.p + n, st);
            if (nv < 2) break;
            LAUNCH(k_pick_pairs, n, ka.p, w2.p, w3.p, n, kb.p, pb.p);
            // (2) group occurrences of each pair
            uint64_t *k1 = kb.p, *k2 = ka.p;
            uint32_t *p1 = pb.p, *p2 = pa.p;
            dev::radix_sort(k1, k2, p1, p2, nv, 2 * b, tmp.p, st);
            // w1 = group start flags, w2 = group index (exclusive), w3 = counted prefix
            LAUNCH(k_groups, nv, k1, p1, counted.p, nv, w1.p, w3.p);
            dev::exclusive_scan(w1.p, w2.p, nv, tmp.p, st);
            dev::exclusive_scan(w3.p, w3.p, nv, tmp.p, st);
            const int64_t nu = (int64_t)read1(w2.p + nv, st);
            // distinct pairs: start and key (in the spare key / position buffers)
            uint64_t* ukey = k2;
            uint32_t* ustart = p2;
            LAUNCH(k_group_fill, nv, k1, w1.p, w2.p, nv, ustart, ukey);
            // (3) rank the candidates
            DevArray<uint64_t> rk(nu), rk2(nu);
            DevArray<uint32_t> rv(nu), rv2(nu), rank_of(nu);
            const int bu = bits_of((uint64_t)nu);
            LAUNCH(k_rank_keys, nu, ustart, w3.p, nu, nv, bu, rk.p, rv.p, cnt.p + 1);
            const int64_t ncand = (int64_t)read1(cnt.p + 1, st);
            if (ncand == 0) break;
            if (ncand + maxsym > INT32_MAX) throw Error(GMR_ERR_RANGE, "grammar exceeds the int32 symbol space");
            uint64_t *r1 = rk.p, *r2 = rk2.p;
            uint32_t *q1 = rv.p, *q2 = rv2.p;
            dev::radix_sort(r1, r2, q1, q2, nu, 32 + bu, tmp.p, st);
            LAUNCH(k_fill_u32, nu, rank_of.p, nu, NONE);
            LAUNCH(k_rank_of, ncand, q1, ncand, rank_of.p);
            // rank at every position (w3 is free again after this)
            uint32_t* rank_pos = w3.p;
            LAUNCH(k_fill_u32, n, rank_pos, n, NONE);
            LAUNCH(k_rank_at, nv, p1, w1.p, w2.p, rank_of.p, nv, rank_pos);
            // (4) the greedy choices
            uint32_t* mark = w1.p;
            LAUNCH(k_want, n, rank_pos, n, want.p, mark);
            dev::inclusive_max_scan(mark, mark, n, tmp.p, st);
            LAUNCH(k_choose, n, want.p, mark, n, chosen.p);
            // (5) uses per distinct pair -> accepted candidates
            uint32_t* f = w1.p;
            LAUNCH(k_chosen_sorted, nv, p1, chosen.p, nv, f);
            dev::exclusive_scan(f, f, nv, tmp.p, st);
            DevArray<uint32_t> acc(ncand + 1);
            LAUNCH(k_accept, ncand, q1, ustart, f, ncand, nu, nv, acc.p);
            uint32_t* apre = w2.p;  // group indices no longer needed
            dev::exclusive_scan(acc.p, apre, ncand, tmp.p, st);
            const int64_t nacc = (int64_t)read1(apre + ncand, st);
            if (nacc == 0) break;
            new_rules.alloc(2 * nacc);
            LAUNCH(k_new_rules, ncand, q1, ukey, acc.p, apre, ncand, b, new_rules.p);
            const size_t r0 = rules.size();
            rules.resize(r0 + 2 * (size_t)nacc);
            GMR_CUDA(cudaMemcpyAsync(rules.data() + r0, new_rules.p, (size_t)nacc * 8, cudaMemcpyDeviceToHost, st));
            // rewrite and compact (positions read ranks at rank_pos, acc by rank)
            uint32_t* keep = f;
            LAUNCH(k_rewrite, n, s.p, n, chosen.p, rank_pos, acc.p, apre, (int32_t)maxsym, s2.p, keep);
            dev::exclusive_scan(keep, w2.p, n, tmp.p, st);
            const int64_t n2 = (int64_t)read1(w2.p + n, st);
            LAUNCH(k_compact, n, s2.p, keep, w2.p, rank_pos, n, s.p, cand2.p);
            cand.swap(cand2);
            fresh = (int32_t)maxsym;  // symbols made this round start here
            GMR_CUDA(cudaStreamSynchronize(st));
            if (verbose)
                std::fprintf(stderr, "device repair round %d: %lld -> %lld symbols, %lld candidates, %zu rules, %.3fs\n",
                             round, (long long)n, (long long)n2, (long long)ncand, rules.size() / 2,
                             std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            n = n2;
        }
        auto g = std::make_unique<gmr_grammar>();
        g->alpha = alpha;
        g->rules.swap(rules);
        const size_t nr = g->rules.size() / 2;
        g->kinds.assign(nr, 0);
        g->reps.assign(nr, 1);
        g->C.resize((size_t)n);
        if (n) GMR_CUDA(cudaMemcpyAsync(g->C.data(), s.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
        GMR_CUDA(cudaStreamSynchronize(st));
        g->V = m->V;
        *out = g.release();
    });
}
