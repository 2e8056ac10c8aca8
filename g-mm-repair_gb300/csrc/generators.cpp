// Seeded synthetic matrices in CSRV form.
//
// Random numbers come from a counter-based hash: u(stream, index) =
// splitmix64_finalizer(seed * K1 + stream * K2 + index), the SplitMix64
// output function of Steele, Lea & Flood, "Fast splittable pseudorandom
// number generators" (OOPSLA 2014).  Every draw is a pure function of
// (seed, stream, index), so the output does not depend on the thread count.
//
// Mosaic genotype matrix (rows = sites, columns = haplotypes, value 1):
//   p_r ~ Beta(1/2, 1/2) per site, drawn as sin^2(pi/2 * U) (the arcsine law);
//   founder f carries allele 1 at site r with probability p_r;
//   haplotype j starts on a uniform founder and at every later site switches
//   to a uniformly chosen founder with probability switch_rate (geometric
//   gaps); every (site, haplotype) bit flips with probability mutation.
//
// Copy-model graph (row = node): node u >= 1 picks a prototype v uniform in
// [0, u); each of its `degree` entries copies entry i of v's raw list with
// probability copy_prob, else draws a uniform target (and, if weighted, a
// uniform weight 1..100; a copied entry keeps its weight).  Lists are sorted
// by target and deduplicated (smallest weight kept).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "gmr_internal.h"

namespace gmr {

static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Hasher {
    uint64_t seed;
    uint64_t h(uint64_t stream, uint64_t idx) const {
        return mix64(mix64(seed * 0xD1B54A32D192ED03ULL + stream) ^ (idx * 0xABC98388FB8FAC03ULL));
    }
    double u01(uint64_t stream, uint64_t idx) const {
        return (double)(h(stream, idx) >> 11) * (1.0 / 9007199254740992.0);
    }
};

// Sequential per-stream generator for event gaps.
struct Stream {
    uint64_t state;
    uint64_t next() {
        state += 0x9E3779B97F4A7C15ULL;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // Gap to the next success of a Bernoulli(p) process (>= 1); huge if p == 0.
    int64_t gap(double p) {
        if (p <= 0.0) return INT64_MAX / 4;
        if (p >= 1.0) return 1;
        double u = u01();
        if (u <= 0.0) u = 1e-300;
        return 1 + (int64_t)std::floor(std::log(u) / std::log1p(-p));
    }
};

enum : uint64_t { S_P = 1, S_ALLELE = 2, S_F0 = 3, S_SWITCH = 4, S_FLIP = 5,
                  S_PROTO = 11, S_COPY = 12, S_TARGET = 13, S_WEIGHT = 14 };

}  // namespace gmr

using namespace gmr;

extern "C" int gmr_gen_mosaic(int rows, int cols, int founders, double switch_rate, double mutation,
                              uint64_t seed, int n_threads, gmr_csrv** out) {
    return guarded([&] {
        if (!out || rows < 0 || cols < 1 || founders < 1) throw Error(GMR_ERR_ARG, "bad argument");
        if (switch_rate < 0 || switch_rate > 1 || mutation < 0 || mutation > 1)
            throw Error(GMR_ERR_ARG, "rates must lie in [0, 1]");
        const int T = default_threads(n_threads);
        Hasher H{seed};

        // Per-haplotype event lists: (site, founder) switches and flip sites.
        std::vector<std::vector<std::pair<int, int>>> sw(cols);
        std::vector<std::vector<int>> fl(cols);
        parallel_for_threads(T, [&](int t) {
            for (int j = t; j < cols; j += T) {
                Stream s{mix64(seed ^ (0x5157ULL << 40) ^ (uint64_t)j * 0x9E37ULL)};
                int f0 = (int)(H.u01(S_F0, (uint64_t)j) * founders);
                if (f0 >= founders) f0 = founders - 1;
                sw[j].push_back({0, f0});
                for (int64_t r = s.gap(switch_rate); r < rows; r += s.gap(switch_rate)) {
                    int f = (int)(s.u01() * founders);
                    if (f >= founders) f = founders - 1;
                    sw[j].push_back({(int)r, f});
                }
                Stream m{mix64(seed ^ (0xF11AULL << 40) ^ (uint64_t)j * 0x7F4AULL)};
                for (int64_t r = m.gap(mutation) - 1; r < rows; r += m.gap(mutation))
                    fl[j].push_back((int)r);
            }
        });

        // Rows in blocks; each thread writes its block's codes.
        const int nblk = std::max(1, std::min(rows, T * 8));
        std::vector<std::vector<int32_t>> blk(nblk);
        std::atomic_int counter{0};
        parallel_for_threads(T, [&](int) {
            std::vector<uint8_t> allele(founders);
            std::vector<int> cur(cols), swp(cols), flp(cols);
            for (;;) {
                int b = counter.fetch_add(1);
                if (b >= nblk) break;
                int r0 = (int)((int64_t)rows * b / nblk), r1 = (int)((int64_t)rows * (b + 1) / nblk);
                for (int j = 0; j < cols; ++j) {
                    auto& e = sw[j];
                    int k = (int)(std::upper_bound(e.begin(), e.end(), std::make_pair(r0, INT32_MAX)) - e.begin()) - 1;
                    swp[j] = k + 1;
                    cur[j] = e[k].second;
                    flp[j] = (int)(std::lower_bound(fl[j].begin(), fl[j].end(), r0) - fl[j].begin());
                }
                auto& o = blk[b];
                for (int r = r0; r < r1; ++r) {
                    double u = H.u01(S_P, (uint64_t)r);
                    double sn = std::sin(1.5707963267948966 * u);
                    double p = sn * sn;
                    for (int f = 0; f < founders; ++f)
                        allele[f] = H.u01(S_ALLELE, (uint64_t)r * founders + f) < p;
                    for (int j = 0; j < cols; ++j) {
                        if (swp[j] < (int)sw[j].size() && sw[j][swp[j]].first == r) cur[j] = sw[j][swp[j]++].second;
                        int bit = allele[cur[j]];
                        if (flp[j] < (int)fl[j].size() && fl[j][flp[j]] == r) {
                            bit ^= 1;
                            ++flp[j];
                        }
                        if (bit) o.push_back(j + 1);
                    }
                    o.push_back(0);
                }
            }
        });
        auto m = new gmr_csrv();
        m->rows = rows;
        m->cols = cols;
        m->V = {1.0};
        size_t tot = 0;
        for (auto& b : blk) tot += b.size();
        m->codes.reserve(tot);
        for (auto& b : blk) {
            m->codes.insert(m->codes.end(), b.begin(), b.end());
            std::vector<int32_t>().swap(b);
        }
        *out = m;
    });
}

extern "C" int gmr_gen_copy_graph(int nodes, int degree, double copy_prob, int weighted, uint64_t seed,
                                  int n_threads, gmr_csrv** out) {
    return guarded([&] {
        if (!out || nodes < 1 || degree < 1 || copy_prob < 0 || copy_prob > 1)
            throw Error(GMR_ERR_ARG, "bad argument");
        const int nv = weighted ? 100 : 1;
        if ((int64_t)nv * nodes + 1 > (int64_t)INT32_MAX)
            throw Error(GMR_ERR_RANGE, "100 * nodes exceeds the int32 terminal space");
        const int T = default_threads(n_threads);
        Hasher H{seed};
        // Entry (u, i): follow the copy chain to the node that drew it.
        auto origin = [&](uint64_t u, uint64_t i) -> uint64_t {
            while (u > 0 && H.u01(S_COPY, u * (uint64_t)degree + i) < copy_prob)
                u = H.h(S_PROTO, u) % u;
            return u;
        };
        const int nblk = std::max(1, std::min(nodes, T * 16));
        std::vector<std::vector<int32_t>> blk(nblk);
        std::atomic_int counter{0};
        parallel_for_threads(T, [&](int) {
            std::vector<std::pair<int32_t, int32_t>> ent(degree);
            for (;;) {
                int b = counter.fetch_add(1);
                if (b >= nblk) break;
                int u0 = (int)((int64_t)nodes * b / nblk), u1 = (int)((int64_t)nodes * (b + 1) / nblk);
                auto& o = blk[b];
                for (int u = u0; u < u1; ++u) {
                    for (int i = 0; i < degree; ++i) {
                        uint64_t w = origin((uint64_t)u, (uint64_t)i);
                        uint64_t key = w * (uint64_t)degree + (uint64_t)i;
                        int32_t tgt = (int32_t)(H.h(S_TARGET, key) % (uint64_t)nodes);
                        int32_t wt = weighted ? (int32_t)(H.h(S_WEIGHT, key) % 100) : 0;  // value index
                        ent[i] = {tgt, wt};
                    }
                    std::sort(ent.begin(), ent.end());
                    int32_t last = -1;
                    for (auto& e : ent) {
                        if (e.first == last) continue;  // dedup; the smallest weight sorts first
                        last = e.first;
                        o.push_back((int32_t)((int64_t)e.second * nodes + e.first + 1));
                    }
                    o.push_back(0);
                }
            }
        });
        auto m = new gmr_csrv();
        m->rows = nodes;
        m->cols = nodes;
        m->V.resize(nv);
        for (int k = 0; k < nv; ++k) m->V[k] = weighted ? (double)(k + 1) : 1.0;
        size_t tot = 0;
        for (auto& b : blk) tot += b.size();
        m->codes.reserve(tot);
        for (auto& b : blk) {
            m->codes.insert(m->codes.end(), b.begin(), b.end());
            std::vector<int32_t>().swap(b);
        }
        *out = m;
    });
}
