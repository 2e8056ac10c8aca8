// RePair grammar compression of a CSRV string, in rounds.
//
// RePair (Larsson & Moffat, "Off-line dictionary-based compression",
// Proc. IEEE 88(11), 2000) repeatedly replaces the most frequent adjacent
// pair of symbols by a new non-terminal.  mm-repair (the producer of the
// reference's .vc.R/.vc.C files) applies it to the CSRV string with the row
// delimiter 0 acting as a barrier, so no rule spans two rows.
//
// This implementation processes pairs in rounds so that rows can be
// handled by many threads:
//   1. count every adjacent pair inside a row (runs "aaa" count
//      non-overlapping occurrences, as RePair does);
//   2. rank the pairs that occur at least twice by (count desc, key asc);
//   3. scan each row left to right and replace the pair at i when its rank
//      is at least as good as the overlapping pair at i+1 (most frequent
//      pair first, as in RePair);
//   4. keep only pairs that were replaced at least twice (the others are
//      left in place), number the kept pairs as new rules in rank order.
// Rounds repeat until no pair occurs twice.  Rules are numbered in creation
// order, so children always precede parents (the topological numbering the
// schedule builder relies on, grammar.h:37-40).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "gmr_internal.h"

namespace gmr {
namespace {

inline uint64_t hkey(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

// Open-addressing map uint64 key (never 0) -> uint32 value.
struct PairMap {
    std::vector<uint64_t> keys;
    std::vector<uint32_t> vals;
    size_t mask = 0, used = 0;
    explicit PairMap(size_t cap = 1024) { reset(cap); }
    void reset(size_t cap) {
        size_t c = 16;
        while (c < cap * 2) c <<= 1;
        keys.assign(c, 0);
        vals.assign(c, 0);
        mask = c - 1;
        used = 0;
    }
    void grow() {
        std::vector<uint64_t> ok;
        std::vector<uint32_t> ov;
        ok.swap(keys);
        ov.swap(vals);
        size_t c = (mask + 1) * 2;
        keys.assign(c, 0);
        vals.assign(c, 0);
        mask = c - 1;
        used = 0;
        for (size_t i = 0; i < ok.size(); ++i)
            if (ok[i]) add(ok[i], ov[i]);
    }
    void add(uint64_t k, uint32_t v) {
        if ((used + 1) * 2 > mask + 1) grow();
        size_t i = hkey(k) & mask;
        while (keys[i] && keys[i] != k) i = (i + 1) & mask;
        if (!keys[i]) {
            keys[i] = k;
            ++used;
        }
        vals[i] += v;
    }
    void put(uint64_t k, uint32_t v) {
        if ((used + 1) * 2 > mask + 1) grow();
        size_t i = hkey(k) & mask;
        while (keys[i] && keys[i] != k) i = (i + 1) & mask;
        if (!keys[i]) {
            keys[i] = k;
            ++used;
        }
        vals[i] = v;
    }
    // Returns UINT32_MAX when absent.
    uint32_t get(uint64_t k) const {
        size_t i = hkey(k) & mask;
        while (keys[i]) {
            if (keys[i] == k) return vals[i];
            i = (i + 1) & mask;
        }
        return UINT32_MAX;
    }
};

inline uint64_t pkey(int32_t a, int32_t b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

}  // namespace
}  // namespace gmr

using namespace gmr;

extern "C" int gmr_repair_compress(const gmr_csrv* m, int n_threads, gmr_grammar** out) {
    return guarded([&] {
        if (!m || !out) throw Error(GMR_ERR_ARG, "null argument");
        const int T = default_threads(n_threads);
        const int64_t alpha64 = (int64_t)m->V.size() * m->cols + 1;
        if (alpha64 > INT32_MAX) throw Error(GMR_ERR_RANGE, "terminal space exceeds int32");
        const int32_t alpha = (int32_t)alpha64;
        std::vector<int32_t> s(m->codes);
        int64_t n = (int64_t)s.size();

        // Chunks of whole rows, balanced by length.
        auto make_chunks = [&](int64_t len) {
            std::vector<int64_t> cs(T + 1, len);
            cs[0] = 0;
            int64_t p = 0;
            for (int t = 1; t < T; ++t) {
                int64_t target = len * t / T;
                if (target < p) target = p;
                while (target < len && (target == 0 || s[target - 1] != 0)) ++target;
                cs[t] = target;
                p = target;
            }
            return cs;
        };

        std::vector<int32_t> rules;
        // After the first round only pairs that hold a symbol made by the
        // previous round (>= fresh) or were candidates in it (was_cand, one flag
        // per position) can reach a count of two: an older pair's occurrences
        // only disappear.  Only those are counted.
        std::vector<uint8_t> was_cand;
        int32_t fresh = alpha;
        const int P = T;  // shards
        const uint32_t NONE = UINT32_MAX;
        const bool verbose = std::getenv("GMR_VERBOSE") != nullptr;
        for (int round = 0; round < 100000; ++round) {
            auto t_round = std::chrono::steady_clock::now();
            std::vector<int64_t> cs = make_chunks(n);
            const int32_t round_first = alpha + (int32_t)(rules.size() / 2);  // first symbol made this round
            // (1) count
            std::vector<std::vector<PairMap>> local(T);
            parallel_for_threads(T, [&](int t) {
                local[t].assign(P, PairMap(1024));
                int64_t a = cs[t], b = cs[t + 1];
                bool prev_eq_counted = false;
                for (int64_t i = a; i + 1 < b; ++i) {
                    int32_t x = s[i], y = s[i + 1];
                    if (x == 0 || y == 0) {
                        prev_eq_counted = false;
                        continue;
                    }
                    if (x == y) {
                        if (prev_eq_counted && s[i - 1] == x) {
                            prev_eq_counted = false;
                            continue;
                        }
                        prev_eq_counted = true;
                    } else {
                        prev_eq_counted = false;
                    }
                    if (round > 0 && x < fresh && y < fresh && !was_cand[i]) continue;
                    uint64_t k = pkey(x, y);
                    local[t][hkey(k) % P].add(k, 1);
                }
            });
            // merge shards; collect candidates
            std::vector<std::vector<std::pair<uint32_t, uint64_t>>> cand(P);
            parallel_for_threads(T, [&](int p) {
                size_t est = 0;
                for (int t = 0; t < T; ++t) est += local[t][p].used;
                PairMap mp(est / 2 + 16);
                for (int t = 0; t < T; ++t) {
                    const PairMap& L = local[t][p];
                    for (size_t i = 0; i < L.keys.size(); ++i)
                        if (L.keys[i]) mp.add(L.keys[i], L.vals[i]);
                    PairMap().keys.swap(local[t][p].keys);
                }
                for (size_t i = 0; i < mp.keys.size(); ++i)
                    if (mp.keys[i] && mp.vals[i] >= 2) cand[p].push_back({mp.vals[i], mp.keys[i]});
            });
            std::vector<std::pair<uint32_t, uint64_t>> all;
            for (auto& c : cand) {
                all.insert(all.end(), c.begin(), c.end());
                std::vector<std::pair<uint32_t, uint64_t>>().swap(c);
            }
            if (all.empty()) break;
            std::sort(all.begin(), all.end(), [](const auto& u, const auto& v) {
                return u.first != v.first ? u.first > v.first : u.second < v.second;
            });
            const size_t nc = all.size();
            if ((int64_t)nc + alpha + (int64_t)rules.size() / 2 > INT32_MAX)
                throw Error(GMR_ERR_RANGE, "grammar exceeds the int32 symbol space");
            // rank maps per shard
            std::vector<PairMap> rank(P);
            {
                std::vector<size_t> per(P, 0);
                for (auto& c : all) per[hkey(c.second) % P]++;
                parallel_for_threads(T, [&](int p) {
                    rank[p].reset(per[p] + 16);
                    for (size_t r = 0; r < nc; ++r)
                        if ((int)(hkey(all[r].second) % P) == p) rank[p].put(all[r].second, (uint32_t)r);
                });
            }
            auto rank_at = [&](int64_t i, int64_t end) -> uint32_t {
                if (i + 1 >= end) return NONE;
                int32_t x = s[i], y = s[i + 1];
                if (x == 0 || y == 0) return NONE;
                uint64_t k = pkey(x, y);
                return rank[hkey(k) % P].get(k);
            };
            // (3) pass A: greedy decisions, usage counts
            std::vector<std::vector<uint32_t>> use(T);
            parallel_for_threads(T, [&](int t) {
                use[t].assign(nc, 0);
                int64_t a = cs[t], b = cs[t + 1];
                int64_t i = a;
                uint32_t ri = rank_at(i, b);
                while (i < b) {
                    uint32_t rn = rank_at(i + 1, b);
                    if (ri != NONE && ri <= rn) {
                        use[t][ri]++;
                        i += 2;
                        ri = rank_at(i, b);
                    } else {
                        i += 1;
                        ri = rn;
                    }
                }
            });
            // (4) accept pairs replaced at least twice
            std::vector<int32_t> newsym(nc, -1);
            {
                std::vector<uint32_t> tot(nc, 0);
                parallel_for_threads(T, [&](int t) {
                    size_t lo = nc * t / T, hi = nc * (t + 1) / T;
                    for (int u = 0; u < T; ++u)
                        for (size_t r = lo; r < hi; ++r) tot[r] += use[u][r];
                });
                std::vector<std::vector<uint32_t>>().swap(use);
                int32_t next = alpha + (int32_t)(rules.size() / 2);
                for (size_t r = 0; r < nc; ++r) {
                    if (tot[r] >= 2) {
                        newsym[r] = next++;
                        rules.push_back((int32_t)(all[r].second >> 32));
                        rules.push_back((int32_t)(all[r].second & 0xffffffffu));
                    }
                }
            }
            bool any = false;
            for (size_t r = 0; r < nc && !any; ++r) any = newsym[r] >= 0;
            if (!any) break;
            // pass B: same traversal, write accepted replacements in place; each
            // written position keeps whether its pair was a candidate
            std::vector<int64_t> outlen(T, 0);
            std::vector<uint8_t> cnew((size_t)n);
            parallel_for_threads(T, [&](int t) {
                int64_t a = cs[t], b = cs[t + 1];
                int64_t i = a, w = a;
                uint32_t ri = rank_at(i, b);
                while (i < b) {
                    uint32_t rn = rank_at(i + 1, b);
                    if (ri != NONE && ri <= rn) {
                        int32_t ns = newsym[ri];
                        if (ns >= 0) {
                            cnew[w] = 0;
                            s[w++] = ns;
                        } else {
                            cnew[w] = 1;
                            s[w++] = s[i];
                            cnew[w] = rn != NONE;
                            s[w++] = s[i + 1];
                        }
                        i += 2;
                        ri = rank_at(i, b);
                    } else {
                        cnew[w] = ri != NONE;
                        s[w++] = s[i];
                        i += 1;
                        ri = rn;
                    }
                }
                outlen[t] = w - a;
            });
            // compact chunks
            int64_t w = outlen[0];
            for (int t = 1; t < T; ++t) {
                std::memmove(&s[w], &s[cs[t]], (size_t)outlen[t] * sizeof(int32_t));
                std::memmove(&cnew[w], &cnew[cs[t]], (size_t)outlen[t]);
                w += outlen[t];
            }
            cnew.resize((size_t)w);
            was_cand.swap(cnew);
            fresh = round_first;
            if (verbose)
                std::fprintf(stderr, "repair round %d: %lld -> %lld symbols, %zu candidates, %zu rules, %.3fs\n",
                             round, (long long)n, (long long)w, nc, rules.size() / 2,
                             std::chrono::duration<double>(std::chrono::steady_clock::now() - t_round).count());
            n = w;
            s.resize((size_t)n);
        }
        auto g = new gmr_grammar();
        g->alpha = alpha;
        g->rules.swap(rules);
        size_t nr = g->rules.size() / 2;
        g->kinds.assign(nr, 0);
        g->reps.assign(nr, 1);
        s.shrink_to_fit();
        g->C.swap(s);
        g->V = m->V;
        *out = g;
    });
}
