// Schedule builder: grammar (or the reference's proper-layered schedule) ->
// level-major, child-sorted plan for the GB300 sweep.
//
// The reference lays a grammar out in levels (build_schedule.cpp:57-71:
// lvl(N -> A B) = 1 + max(lvl A, lvl B), terminals at 0), inserts identity
// pass-through nodes so every child sits in the frontier directly below its
// parent (build_schedule.cpp:119-135), emits each non-terminal occurrence
// of C at the symbol's own level (build_schedule.cpp:138-155) and compacts
// the terminal alphabet to the referenced ones (build_schedule.cpp:187-224).
//
// The plan keeps the levels, the emit-at-own-level rule and the compacted
// terminals, and changes the layout:
//   * all values of one multiply live in one arena (one slot per evaluated
//     rule, level-major), so a pass-through is a reference to its source
//     slot instead of a copied value: no pass-through work at run time;
//   * within a level, rules are sorted by (left child, right child), so the
//     left-child gathers of consecutive threads are monotone;
//   * emissions of a level are sorted by (row, source), so a warp reduces a
//     row segment in registers and issues one atomic per segment;
//   * ops and emissions are structure-of-arrays (8 bytes per binary rule,
//     the coefficient array exists only when a run-length rule does).
// The reference's own layered figures (L, w*, |R|, +pt, E, E_T, U) are
// computed alongside for reporting and for the roofline byte count.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>

#include "gmr_internal.h"

namespace gmr {

namespace {

// Level index of an arena slot (binary search over level offsets).
int level_of_slot(const std::vector<int64_t>& lvl_off, int64_t slot) {
    // lvl_off[k] = end of level k; level k covers [lvl_off[k-1], lvl_off[k]).
    auto it = std::upper_bound(lvl_off.begin(), lvl_off.end(), slot);
    return (int)(it - lvl_off.begin());
}

// Sort ops of one level by (left, right) and return the permutation.
std::vector<int64_t> child_sort(const std::vector<int32_t>& L, const std::vector<int32_t>& R) {
    std::vector<int64_t> perm(L.size());
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) {
        if (L[a] != L[b]) return L[a] < L[b];
        if (R[a] != R[b]) return R[a] < R[b];
        return a < b;
    });
    return perm;
}

void build_segments(gmr_plan& p);

// Group emissions by level, then sort each level's segment by (row, src).
void finish_emissions(gmr_plan& p, std::vector<int32_t>& lvl_of_em, std::vector<int32_t>& src,
                      std::vector<int32_t>& row) {
    const int D = p.depth;
    std::vector<int64_t> cnt(D + 2, 0);
    for (int32_t l : lvl_of_em) cnt[l + 1]++;
    for (int k = 0; k <= D; ++k) cnt[k + 1] += cnt[k];
    p.em_off = cnt;
    const int64_t E = (int64_t)src.size();
    p.em_src.assign(E, 0);
    p.em_row.assign(E, 0);
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int64_t e = 0; e < E; ++e) {
        int64_t d = pos[lvl_of_em[e]]++;
        p.em_src[d] = src[e];
        p.em_row[d] = row[e];
    }
    // rows are visited in order, so each level segment is row-nondecreasing;
    // sort sources within each (level, row) group.
    std::vector<uint64_t> key;
    for (int k = 0; k <= D; ++k) {
        int64_t a = p.em_off[k], b = p.em_off[k + 1];
        int64_t i = a;
        while (i < b) {
            int64_t j = i + 1;
            while (j < b && p.em_row[j] == p.em_row[i]) ++j;
            if (j - i > 1) std::sort(p.em_src.begin() + i, p.em_src.begin() + j);
            i = j;
        }
        // guard: rows must be non-decreasing inside the level
        for (int64_t e = a + 1; e < b; ++e)
            if (p.em_row[e] < p.em_row[e - 1]) {
                // not row-sorted (caller-supplied emission order): full sort
                key.resize((size_t)(b - a));
                for (int64_t q = a; q < b; ++q)
                    key[q - a] = ((uint64_t)(uint32_t)p.em_row[q] << 32) | (uint32_t)p.em_src[q];
                std::sort(key.begin(), key.end());
                for (int64_t q = a; q < b; ++q) {
                    p.em_row[q] = (int32_t)(key[q - a] >> 32);
                    p.em_src[q] = (int32_t)(key[q - a] & 0xffffffffu);
                }
                break;
            }
    }
    build_segments(p);
}

// Row segments of the (level-major, row-sorted) emission arrays.
void build_segments(gmr_plan& p) {
    const int D = p.depth;
    p.seg_off.assign(D + 2, 0);
    p.seg_row.clear();
    p.seg_start.clear();
    for (int k = 0; k <= D; ++k) {
        p.seg_off[k] = (int64_t)p.seg_row.size();
        for (int64_t e = p.em_off[k]; e < p.em_off[k + 1]; ++e) {
            if (e == p.em_off[k] || p.em_row[e] != p.em_row[e - 1]) {
                p.seg_row.push_back(p.em_row[e]);
                p.seg_start.push_back(e);
            }
        }
    }
    p.seg_off[D + 1] = (int64_t)p.seg_row.size();
    p.seg_start.push_back((int64_t)p.em_src.size());
}

}  // namespace

void fill_common_stats(gmr_plan& p) {
    auto& s = p.stats;
    s.rows = p.rows;
    s.cols = p.cols;
    s.depth = p.depth;
    s.n_vals = (int)p.V.size();
    s.has_coeff = p.has_coeff() ? 1 : 0;
    s.n_ops = p.n_ops();
    s.n_terms = p.n_terms();
    s.n_term_emit = p.em_off.size() > 1 ? p.em_off[1] - p.em_off[0] : 0;
    s.n_emit = (int64_t)p.em_src.size() - s.n_term_emit;
    int64_t mx = 0;
    for (int k = 1; k <= p.depth; ++k) mx = std::max(mx, p.lvl_off[k] - p.lvl_off[k - 1]);
    s.max_level_ops = mx;
}

void validate_plan(const gmr_plan& p) {
    const int D = p.depth;
    if ((int)p.lvl_off.size() != D + 1 || p.lvl_off[0] != 0 || p.lvl_off[D] != p.n_ops())
        throw Error(GMR_ERR_FORMAT, "plan: bad level offsets");
    if ((int)p.em_off.size() != D + 2 || p.em_off[0] != 0 || p.em_off[D + 1] != (int64_t)p.em_src.size())
        throw Error(GMR_ERR_FORMAT, "plan: bad emission offsets");
    const int64_t U = p.n_terms();
    for (int k = 1; k <= D; ++k) {
        if (p.lvl_off[k] < p.lvl_off[k - 1]) throw Error(GMR_ERR_FORMAT, "plan: level offsets decrease");
        for (int64_t i = p.lvl_off[k - 1]; i < p.lvl_off[k]; ++i) {
            for (int32_t c : {p.op_l[i], p.op_r[i]}) {
                if (c >= 0 ? (int64_t)c >= p.lvl_off[k - 1] : (int64_t)(-(int64_t)c - 1) >= U)
                    throw Error(GMR_ERR_FORMAT, "plan: op " + std::to_string(i) + " child " +
                                                    std::to_string(c) + " out of range");
            }
        }
    }
    for (int k = 0; k <= D; ++k) {
        int64_t lo = k == 0 ? 0 : p.lvl_off[k - 1], hi = k == 0 ? 0 : p.lvl_off[k];
        for (int64_t e = p.em_off[k]; e < p.em_off[k + 1]; ++e) {
            int32_t c = p.em_src[e];
            bool ok = c >= 0 ? (c >= lo && c < hi) : (int64_t)(-(int64_t)c - 1) < U;
            if (k == 0 && c >= 0) ok = false;
            if (!ok) throw Error(GMR_ERR_FORMAT, "plan: emission source out of range");
            if (p.em_row[e] < 0 || p.em_row[e] >= p.rows) throw Error(GMR_ERR_FORMAT, "plan: emission row out of range");
        }
    }
    if ((int)p.seg_off.size() != D + 2 || p.seg_start.size() != p.seg_row.size() + 1 ||
        p.seg_off[D + 1] != (int64_t)p.seg_row.size() || p.seg_start.back() != (int64_t)p.em_src.size())
        throw Error(GMR_ERR_FORMAT, "plan: bad row segments");
    for (int k = 0; k <= D; ++k) {
        for (int64_t q = p.seg_off[k]; q < p.seg_off[k + 1]; ++q) {
            if (p.seg_start[q] < p.em_off[k] || p.seg_start[q + 1] > p.em_off[k + 1] || p.seg_start[q + 1] <= p.seg_start[q])
                throw Error(GMR_ERR_FORMAT, "plan: row segment out of its level");
            if (q > p.seg_off[k] && p.seg_row[q] <= p.seg_row[q - 1])
                throw Error(GMR_ERR_FORMAT, "plan: row segments not strictly increasing");
            for (int64_t e = p.seg_start[q]; e < p.seg_start[q + 1]; ++e)
                if (p.em_row[e] != p.seg_row[q]) throw Error(GMR_ERR_FORMAT, "plan: row segment mixes rows");
        }
    }
    for (size_t q = 0; q < p.term_val.size(); ++q) {
        if (p.term_val[q] < 0 || p.term_val[q] >= (int32_t)p.V.size())
            throw Error(GMR_ERR_FORMAT, "plan: terminal value index out of range");
        if (p.term_col[q] < 0 || p.term_col[q] >= p.cols)
            throw Error(GMR_ERR_FORMAT, "plan: terminal column out of range");
    }
}

}  // namespace gmr

using namespace gmr;

extern "C" int gmr_plan_build(const gmr_grammar* g, int rows, int cols, gmr_plan** out) {
    return guarded([&] {
        if (!g || !out || rows < 0 || cols < 1) throw Error(GMR_ERR_ARG, "bad argument");
        const int32_t alpha = g->alpha;
        const int64_t n = g->n_rules();
        const int64_t nv = (int64_t)g->V.size();
        const int32_t* R = g->rules.data();
        auto is_rl = [&](int64_t i) { return g->kinds[i] == 1; };

        // (1) levels (build_schedule.cpp:57-71)
        std::vector<int32_t> lvl((size_t)n, 0);
        int depth = 0;
        auto clvl = [&](int32_t s) { return s >= alpha ? lvl[s - alpha] : 0; };
        for (int64_t i = 0; i < n; ++i) {
            int l = clvl(R[2 * i]);
            if (!is_rl(i)) l = std::max(l, clvl(R[2 * i + 1]));
            lvl[i] = l + 1;
            depth = std::max(depth, l + 1);
        }

        auto p = std::make_unique<gmr_plan>();
        p->rows = rows;
        p->cols = cols;
        p->depth = depth;
        p->V.assign(g->V.begin(), g->V.end());

        // (2) reference-equivalent layered figures on the full grammar
        {
            std::vector<int32_t> mref(lvl);
            for (int64_t i = 0; i < n; ++i) {
                int32_t l = R[2 * i], r = R[2 * i + 1];
                if (l >= alpha) mref[l - alpha] = std::max(mref[l - alpha], lvl[i]);
                if (!is_rl(i) && r >= alpha) mref[r - alpha] = std::max(mref[r - alpha], lvl[i]);
            }
            int64_t pt = 0;
            for (int64_t i = 0; i < n; ++i) pt += mref[i] - lvl[i];
            // width of reference level k = raw rules of level k + symbols carried
            // through it (present at levels lvl+1 .. mref as pass-throughs)
            std::vector<int64_t> raw(depth + 2, 0), diff(depth + 2, 0);
            for (int64_t i = 0; i < n; ++i) raw[lvl[i]]++;
            for (int64_t i = 0; i < n; ++i)
                if (mref[i] > lvl[i]) {
                    diff[lvl[i] + 1]++;
                    diff[mref[i] + 1]--;
                }
            int64_t run = 0, wmax = 0;
            for (int k = 1; k <= depth; ++k) {
                run += diff[k];
                wmax = std::max(wmax, raw[k] + run);
            }
            std::vector<uint8_t> used_t((size_t)alpha, 0);
            for (int64_t i = 0; i < n; ++i) {
                if (R[2 * i] < alpha) used_t[R[2 * i]] = 1;
                if (!is_rl(i) && R[2 * i + 1] < alpha) used_t[R[2 * i + 1]] = 1;
            }
            int64_t e = 0, et = 0;
            for (int32_t c : g->C) {
                if (c == 0) continue;
                if (c < alpha) {
                    ++et;
                    used_t[c] = 1;
                } else {
                    ++e;
                }
            }
            int64_t U = 1;
            for (int32_t t = 1; t < alpha; ++t) U += used_t[t];
            auto& s = p->stats;
            s.ref_raw = n;
            s.ref_passthrough = pt;
            s.ref_layered = n + pt;
            s.ref_max_width = wmax;
            s.ref_emit = e;
            s.ref_term_emit = et;
            s.ref_alpha = U;
        }

        // (3) live rules: reachable from C
        std::vector<uint8_t> live((size_t)n, 0);
        for (int32_t c : g->C)
            if (c >= alpha) live[c - alpha] = 1;
        for (int64_t i = n - 1; i >= 0; --i) {
            if (!live[i]) continue;
            int32_t l = R[2 * i], r = R[2 * i + 1];
            if (l >= alpha) live[l - alpha] = 1;
            if (!is_rl(i) && r >= alpha) live[r - alpha] = 1;
        }

        // (4) compacted terminals (ascending original code, zero terminal = 0)
        std::vector<int32_t> tmap((size_t)alpha, 0);
        for (int64_t i = 0; i < n; ++i) {
            if (!live[i]) continue;
            if (R[2 * i] < alpha) tmap[R[2 * i]] = 1;
            if (!is_rl(i) && R[2 * i + 1] < alpha) tmap[R[2 * i + 1]] = 1;
        }
        for (int32_t c : g->C)
            if (c > 0 && c < alpha) tmap[c] = 1;
        int32_t U = 1;
        for (int32_t t = 1; t < alpha; ++t) {
            if (!tmap[t]) continue;
            tmap[t] = U++;
            int64_t vi = (int64_t)(t - 1) / cols, ci = (int64_t)(t - 1) % cols;
            if (vi >= nv) throw Error(GMR_ERR_FORMAT, "terminal " + std::to_string(t) + " has no value");
            p->term_val.push_back((int32_t)vi);
            p->term_col.push_back((int32_t)ci);
        }

        // (5) slots, level by level, child-sorted
        std::vector<std::vector<int64_t>> by_level(depth + 1);
        for (int64_t i = 0; i < n; ++i)
            if (live[i]) by_level[lvl[i]].push_back(i);
        std::vector<int32_t> slot((size_t)n, -1);
        auto ref = [&](int32_t s) -> int32_t { return s >= alpha ? slot[s - alpha] : -tmap[s] - 1; };
        p->lvl_off.assign(depth + 1, 0);
        bool coeff = g->has_runlen;
        int64_t next = 0;
        for (int k = 1; k <= depth; ++k) {
            auto& ids = by_level[k];
            std::vector<int32_t> L(ids.size()), Rr(ids.size());
            for (size_t j = 0; j < ids.size(); ++j) {
                int64_t i = ids[j];
                L[j] = ref(R[2 * i]);
                Rr[j] = is_rl(i) ? -1 : ref(R[2 * i + 1]);
            }
            auto perm = child_sort(L, Rr);
            if (next + (int64_t)ids.size() > INT32_MAX) throw Error(GMR_ERR_RANGE, "more than 2^31 ops");
            for (size_t j = 0; j < perm.size(); ++j) {
                int64_t i = ids[perm[j]];
                slot[i] = (int32_t)(next + (int64_t)j);
                p->op_l.push_back(L[perm[j]]);
                p->op_r.push_back(Rr[perm[j]]);
                if (coeff) p->op_c.push_back(is_rl(i) ? (float)g->reps[i] : 1.0f);
            }
            next += (int64_t)ids.size();
            p->lvl_off[k] = next;
            std::vector<int64_t>().swap(ids);
        }

        // (6) emissions from C at the symbol's own level
        std::vector<int32_t> el, es, er;
        el.reserve(g->C.size());
        es.reserve(g->C.size());
        er.reserve(g->C.size());
        int32_t row = 0;
        for (int32_t c : g->C) {
            if (c == 0) {
                ++row;
                continue;
            }
            if (row >= rows) throw Error(GMR_ERR_FORMAT, "C holds more rows than rows=" + std::to_string(rows));
            if (c < alpha) {
                el.push_back(0);
                es.push_back(-tmap[c] - 1);
            } else {
                el.push_back(lvl[c - alpha]);
                es.push_back(slot[c - alpha]);
            }
            er.push_back(row);
        }
        finish_emissions(*p, el, es, er);
        fill_common_stats(*p);
        validate_plan(*p);
        *out = p.release();
    });
}

extern "C" int gmr_plan_from_layered(int rows, int cols, int alpha, int total_layered_rules,
                                     const LayeredRule* rules, const int* val_indices,
                                     const int* col_indices, const float* V, int n_vals,
                                     const GPUSchedule* sched, gmr_plan** out) {
    return guarded([&] {
        if (!out || !sched || rows < 0 || cols < 1 || alpha < 1 || total_layered_rules < 0 || n_vals < 0)
            throw Error(GMR_ERR_ARG, "bad argument");
        if (total_layered_rules > 0 && !rules) throw Error(GMR_ERR_ARG, "null rules");
        if (alpha > 1 && (!val_indices || !col_indices)) throw Error(GMR_ERR_ARG, "null terminal tables");
        const int D = sched->max_depth;
        if (D < 0 || (D > 0 && !sched->level_offsets)) throw Error(GMR_ERR_FORMAT, "bad schedule depth");
        auto p = std::make_unique<gmr_plan>();
        p->rows = rows;
        p->cols = cols;
        p->depth = D;
        p->V.assign(V, V + n_vals);
        for (int q = 1; q < alpha; ++q) {
            p->term_val.push_back(val_indices[q - 1]);
            p->term_col.push_back(col_indices[q - 1]);
        }
        const int* lo = sched->level_offsets;
        if (D > 0 && (lo[0] != 0 || lo[D] != total_layered_rules))
            throw Error(GMR_ERR_FORMAT, "level offsets do not cover the rules");
        const int* eo = sched->emit_offsets;
        if (sched->emit_total > 0 && (!eo || !sched->emit_pos || !sched->emit_row))
            throw Error(GMR_ERR_FORMAT, "null emit lists");

        std::vector<int32_t> el, es, er;
        for (int e = 0; e < sched->num_term_emit; ++e) {
            int s = sched->term_emit_sym[e];
            if (s < 0 || s >= alpha) throw Error(GMR_ERR_FORMAT, "terminal emission symbol out of range");
            el.push_back(0);
            es.push_back(-s - 1);
            er.push_back(sched->term_emit_row[e]);
        }
        p->lvl_off.assign(D + 1, 0);
        std::vector<int32_t> prev, cur;  // frontier slot -> plan reference
        bool coeff = false;
        for (int64_t i = 0; i < total_layered_rules; ++i)
            if (rules[i].coeff != 1.0f) coeff = true;
        int64_t next = 0, identities = 0;
        auto resolve = [&](int c, int k) -> int32_t {
            if (c >= 0) {
                if (c >= (int)prev.size())
                    throw Error(GMR_ERR_FORMAT, "level " + std::to_string(k) + ": child slot " + std::to_string(c) +
                                                    " beyond the previous frontier");
                return prev[c];
            }
            if ((int64_t)(-(int64_t)c - 1) >= alpha) throw Error(GMR_ERR_FORMAT, "terminal child out of range");
            return c;
        };
        for (int k = 1; k <= D; ++k) {
            int a = lo[k - 1], b = lo[k];
            if (b < a) throw Error(GMR_ERR_FORMAT, "level offsets decrease");
            cur.assign((size_t)(b - a), 0);
            std::vector<int32_t> L, Rr, idx;
            std::vector<float> Cf;
            for (int j = a; j < b; ++j) {
                int32_t l = resolve(rules[j].left, k), r = resolve(rules[j].right, k);
                float c = rules[j].coeff;
                if (c == 1.0f && r == -1) {
                    cur[j - a] = l;  // identity (pass-through): alias
                    ++identities;
                } else if (c == 1.0f && l == -1) {
                    cur[j - a] = r;
                    ++identities;
                } else {
                    L.push_back(l);
                    Rr.push_back(r);
                    Cf.push_back(c);
                    idx.push_back(j - a);
                }
            }
            auto perm = child_sort(L, Rr);
            for (size_t q = 0; q < perm.size(); ++q) {
                cur[idx[perm[q]]] = (int32_t)(next + (int64_t)q);
                p->op_l.push_back(L[perm[q]]);
                p->op_r.push_back(Rr[perm[q]]);
                if (coeff) p->op_c.push_back(Cf[perm[q]]);
            }
            next += (int64_t)perm.size();
            p->lvl_off[k] = next;
            // emissions of level k
            if (sched->emit_total > 0) {
                for (int e = eo[k - 1]; e < eo[k]; ++e) {
                    int pos = sched->emit_pos[e];
                    if (pos < 0 || pos >= (int)cur.size()) throw Error(GMR_ERR_FORMAT, "emission position out of range");
                    el.push_back(0);  // level of the source, fixed once all slots exist
                    es.push_back(cur[pos]);
                    er.push_back(sched->emit_row[e]);
                }
            }
            prev.swap(cur);
        }
        // levels of emission sources (slots are final now)
        for (size_t e = 0; e < es.size(); ++e) el[e] = es[e] < 0 ? 0 : level_of_slot(p->lvl_off, es[e]);
        for (size_t e = 0; e < er.size(); ++e)
            if (er[e] < 0 || er[e] >= rows) throw Error(GMR_ERR_FORMAT, "emission row out of range");
        finish_emissions(*p, el, es, er);
        fill_common_stats(*p);
        auto& s = p->stats;
        s.ref_layered = total_layered_rules;
        s.ref_passthrough = identities;
        s.ref_raw = total_layered_rules - identities;
        s.ref_max_width = sched->max_width;
        s.ref_emit = sched->emit_total;
        s.ref_term_emit = sched->num_term_emit;
        s.ref_alpha = alpha;
        validate_plan(*p);
        *out = p.release();
    });
}


// Per-slot statistics: [ops_k, em_{k-1}, seg_{k-1}, distinct sources_{k-1},
// children from k-1, k-2, <= k-3, terminals] for slots k = 0 .. depth+1.
static const std::vector<double>& slot_stats(const gmr_plan& p) {
    if (!p.slot_stats.empty()) return p.slot_stats;
    const int D = p.depth, NS = 8;
    std::vector<double> st((size_t)(D + 2) * NS, 0.0);
    std::vector<uint32_t> seen((size_t)(p.n_ops() + p.n_terms()), 0);
    for (int k = 1; k <= D + 1; ++k) {
        double* s = st.data() + (size_t)k * NS;
        if (k <= D) {
            s[0] = (double)(p.lvl_off[k] - p.lvl_off[k - 1]);
            for (int64_t i = p.lvl_off[k - 1]; i < p.lvl_off[k]; ++i) {
                for (int32_t c : {p.op_l[i], p.op_r[i]}) {
                    if (c < 0) {
                        s[7] += 1;
                        continue;
                    }
                    const int lc = level_of_slot(p.lvl_off, c);
                    const int dist = k - lc;
                    s[dist == 1 ? 4 : (dist == 2 ? 5 : 6)] += 1;
                }
            }
        }
        const int ke = k - 1;
        s[1] = (double)(p.em_off[ke + 1] - p.em_off[ke]);
        s[2] = (double)(p.seg_off[ke + 1] - p.seg_off[ke]);
        double distinct = 0;
        for (int64_t e = p.em_off[ke]; e < p.em_off[ke + 1]; ++e) {
            const int32_t c = p.em_src[e];
            const size_t key = c >= 0 ? (size_t)c : (size_t)(p.n_ops() + (-(int64_t)c - 1));
            if (seen[key] != (uint32_t)k) {
                seen[key] = (uint32_t)k;
                distinct += 1;
            }
        }
        s[3] = distinct;
    }
    p.slot_stats.swap(st);
    return p.slot_stats;
}

extern "C" int gmr_plan_launch_features(const gmr_plan* p, int semiring, int B, float* out, int cap, int* n_slots) {
    return guarded([&] {
        if (!p || !out || !n_slots || B < 1) throw Error(GMR_ERR_ARG, "bad argument");
        const int D = p->depth, NF = GMR_N_BASE_FEATURES, slots = D + 2;
        if (cap < slots * NF) throw Error(GMR_ERR_RANGE, "feature buffer too small");
        const auto& st = slot_stats(*p);
        const double words = semiring == GMR_BOOLEAN ? (double)((B + 31) / 32) : (double)B;
        std::fill(out, out + (size_t)slots * NF, 0.0f);
        // the engine evaluates terminals in place (no terminal table) when
        // there are more than 4 terminals per column and codes fit 31 bits
        const int64_t n_te = p->em_off.size() > 1 ? p->em_off[1] - p->em_off[0] : 0;
        const bool direct = n_te > 0 && p->n_terms() > 4 * (int64_t)p->cols &&
                            (int64_t)p->V.size() * p->cols <= INT32_MAX;
        for (int k = 1; k < slots; ++k) {
            const double* s = st.data() + (size_t)k * 8;
            float* f = out + (size_t)k * NF;
            const double children = s[4] + s[5] + s[6] + s[7];
            const double prev_ops = k >= 2 ? (double)(p->lvl_off[k - 1] - p->lvl_off[k - 2]) : (double)p->n_terms();
            f[0] = (float)std::log1p(s[0]);
            f[1] = (float)std::log1p(s[1]);
            f[2] = (float)std::log1p(s[2]);
            f[3] = (float)std::log1p(s[2] > 0 ? s[1] / s[2] : 0.0);
            f[4] = (float)std::log1p(s[3] > 0 ? s[1] / s[3] : 0.0);
            for (int j = 0; j < 4; ++j) f[5 + j] = (float)(children > 0 ? s[4 + j] / children : 0.0);
            f[9] = (float)std::log1p(prev_ops * words * 4.0 / 1048576.0);
            f[10] = (float)std::log2(words);
            f[11] = semiring == GMR_BOOLEAN ? 1.0f : 0.0f;
            f[12] = semiring == GMR_TROPICAL ? 1.0f : 0.0f;
            f[13] = (float)std::log1p((double)p->rows);
            f[14] = (float)std::log1p((double)p->n_ops());
            f[15] = (float)k / (float)(D + 1);
            f[16] = direct ? 1.0f : 0.0f;
        }
        *n_slots = slots;
    });
}


extern "C" int gmr_plan_prepare_left(gmr_plan* p) {
    return guarded([&] {
        if (!p) throw Error(GMR_ERR_ARG, "null plan");
        if (!p->par_off.empty()) return;
        const int64_t n = p->n_ops(), U = p->n_terms(), N = n + U;
        auto node = [&](int32_t ref) -> int64_t { return ref >= 0 ? (int64_t)ref : n + (-(int64_t)ref - 1); };
        std::vector<int64_t> po(N + 1, 0), eo(N + 1, 0), co((size_t)p->cols + 1, 0);
        for (int64_t i = 0; i < n; ++i) {
            po[node(p->op_l[i]) + 1]++;
            po[node(p->op_r[i]) + 1]++;
        }
        for (size_t e = 0; e < p->em_src.size(); ++e) eo[node(p->em_src[e]) + 1]++;
        for (size_t q = 0; q < p->term_col.size(); ++q) co[p->term_col[q] + 1]++;
        for (int64_t u = 0; u < N; ++u) {
            po[u + 1] += po[u];
            eo[u + 1] += eo[u];
        }
        for (int c = 0; c < p->cols; ++c) co[c + 1] += co[c];
        std::vector<int32_t> ps((size_t)po[N]), er((size_t)eo[N]), tq(p->term_col.size());
        std::vector<int64_t> fp(po.begin(), po.end() - 1), fe(eo.begin(), eo.end() - 1), fc(co.begin(), co.end() - 1);
        for (int64_t i = 0; i < n; ++i) {  // parents in increasing slot order
            ps[fp[node(p->op_l[i])]++] = (int32_t)i;
            ps[fp[node(p->op_r[i])]++] = ~(int32_t)i;
        }
        for (size_t e = 0; e < p->em_src.size(); ++e) er[fe[node(p->em_src[e])]++] = p->em_row[e];
        for (size_t q = 0; q < p->term_col.size(); ++q) tq[fc[p->term_col[q]]++] = (int32_t)(q + 1);
        // flat edge lists for the chunked left fold
        if (n + (int64_t)p->rows > (int64_t)INT32_MAX) throw Error(GMR_ERR_RANGE, "left product: rules + rows exceed 2^31");
        const int64_t tot = (po[n] - po[0]) + (eo[n] - eo[0]) + (po[N] - po[n + 1]) + (eo[N] - eo[n + 1]);
        std::vector<int32_t> src((size_t)tot), tgt((size_t)tot);
        std::vector<int64_t> start((size_t)N + 1, 0);  // first edge of each node
        int64_t w = 0;
        auto emit_node = [&](int64_t u, int32_t t) {
            start[u] = w;
            for (int64_t j = po[u]; j < po[u + 1]; ++j, ++w) {
                src[w] = ps[j];
                tgt[w] = t;
            }
            for (int64_t j = eo[u]; j < eo[u + 1]; ++j, ++w) {
                src[w] = (int32_t)(n + er[j]);
                tgt[w] = t;
            }
        };
        for (int64_t u = 0; u < n; ++u) emit_node(u, (int32_t)u);
        for (int64_t q = 1; q < U; ++q) emit_node(n + q, (int32_t)q);
        const int D = p->depth;
        std::vector<int64_t> lo((size_t)D + 2, 0);
        for (int k = 1; k <= D; ++k) lo[k] = p->lvl_off[k] < n ? start[p->lvl_off[k]] : (po[n] - po[0]) + (eo[n] - eo[0]);
        lo[D + 1] = tot;
        std::vector<int32_t> split;
        for (int k = 1; k <= D + 1; ++k) {
            const int64_t a = lo[k - 1], b = lo[k];
            for (int64_t e = a; e < b;) {
                int64_t f = e + 1;
                while (f < b && tgt[f] == tgt[e]) ++f;
                if ((e - a) / kLeftChunk != (f - 1 - a) / kLeftChunk)
                    split.push_back(k <= D ? tgt[e] : (int32_t)(n + tgt[e]));
                e = f;
            }
        }
        p->par_off.swap(po);
        p->erow_off.swap(eo);
        p->tcol_off.swap(co);
        p->par_src.swap(ps);
        p->erow_row.swap(er);
        p->tcol_q.swap(tq);
        p->le_off.swap(lo);
        p->le_src.swap(src);
        p->le_tgt.swap(tgt);
        p->le_split.swap(split);
    });
}

extern "C" int gmr_plan_get_stats(const gmr_plan* p, gmr_plan_stats* s) {
    return guarded([&] {
        if (!p || !s) throw Error(GMR_ERR_ARG, "null argument");
        *s = p->stats;
    });
}

extern "C" int gmr_plan_level_ops(const gmr_plan* p, int64_t* out, int n) {
    return guarded([&] {
        if (!p || !out || n < p->depth + 1) throw Error(GMR_ERR_ARG, "bad argument");
        out[0] = 0;
        for (int k = 1; k <= p->depth; ++k) out[k] = p->lvl_off[k] - p->lvl_off[k - 1];
    });
}

extern "C" int gmr_plan_level_emits(const gmr_plan* p, int64_t* out, int n) {
    return guarded([&] {
        if (!p || !out || n < p->depth + 1) throw Error(GMR_ERR_ARG, "bad argument");
        for (int k = 0; k <= p->depth; ++k) out[k] = p->em_off[k + 1] - p->em_off[k];
    });
}

extern "C" double gmr_plan_alg_bytes(const gmr_plan* p, int semiring, int B) {
    if (!p || B < 1) return -1.0;
    const auto& s = p->stats;
    double Bp = semiring == GMR_BOOLEAN ? (double)((B + 31) / 32) : (double)B;
    return 12.0 * (double)s.ref_layered + 8.0 * (double)s.ref_emit + 8.0 * (double)s.ref_term_emit +
           8.0 * (double)(s.ref_alpha - 1) + 4.0 * (double)s.n_vals + 4.0 * (double)s.cols * Bp +
           4.0 * (double)s.rows * Bp;
}

// Left-child windows of shared-memory staging: within a level the rules are
// sorted by left child, so the arena slots that the left children of a run of
// consecutive rules (one CTA's rules) reference form one contiguous window
// [first slot child, last child].  Per level k (row k-1 of out): fractions of
// the level's runs of rules_per_cta rules whose window holds at most 64 KB,
// 128 KB and 200 KB of values of `words` 4-byte words; the mean density of
// the windows (distinct referenced slots / window slots); and the fraction of
// left children that are slots (the rest are terminals).
static void window_stats(const gmr_plan& p, int rules_per_cta, int words, double* out) {
    const double budget[3] = {64.0 * 1024, 128.0 * 1024, 200.0 * 1024};
    for (int k = 1; k <= p.depth; ++k) {
        double* o = out + (size_t)(k - 1) * GMR_WINDOW_STATS;
        std::fill(o, o + GMR_WINDOW_STATS, 0.0);
        const int64_t a = p.lvl_off[k - 1], b = p.lvl_off[k];
        int64_t runs = 0, slot_refs = 0, dens_runs = 0;
        double dens = 0.0;
        for (int64_t r0 = a; r0 < b; r0 += rules_per_cta) {
            const int64_t r1 = std::min<int64_t>(r0 + rules_per_cta, b);
            ++runs;
            int64_t lo = -1, hi = -1, distinct = 0;
            int32_t prev = INT32_MIN;
            for (int64_t i = r0; i < r1; ++i) {
                const int32_t c = p.op_l[(size_t)i];
                if (c < 0) continue;
                ++slot_refs;
                if (lo < 0) lo = c;
                hi = c;
                distinct += c != prev;
                prev = c;
            }
            const double bytes = lo < 0 ? 0.0 : (double)(hi - lo + 1) * words * 4.0;
            for (int j = 0; j < 3; ++j) o[j] += bytes <= budget[j];
            if (lo >= 0) {
                dens += (double)distinct / (double)(hi - lo + 1);
                ++dens_runs;
            }
        }
        if (runs) for (int j = 0; j < 3; ++j) o[j] /= (double)runs;
        o[3] = dens_runs ? dens / (double)dens_runs : 0.0;
        o[4] = b > a ? (double)slot_refs / (double)(b - a) : 0.0;
    }
}

extern "C" int gmr_plan_window_stats(const gmr_plan* p, int rules_per_cta, int words, double* out, int cap, int* n) {
    return guarded([&] {
        if (!p || !out || !n || rules_per_cta < 1 || words < 1) throw Error(GMR_ERR_ARG, "bad argument");
        if (cap < p->depth * GMR_WINDOW_STATS) throw Error(GMR_ERR_RANGE, "need depth x GMR_WINDOW_STATS doubles");
        window_stats(*p, rules_per_cta, words, out);
        *n = p->depth;
    });
}

extern "C" int gmr_plan_describe(const gmr_plan* p, char* buf, size_t cap) {
    return guarded([&] {
        if (!p || !buf || cap == 0) throw Error(GMR_ERR_ARG, "bad argument");
        std::string o;
        char line[256];
        const auto& s = p->stats;
        std::snprintf(line, sizeof line,
                      "Max depth (L): %d, Max width (w*): %lld, Total layered rules: %lld (raw NTs: %lld, +pt: %lld), "
                      "emissions: %lld+%lld term\n",
                      p->depth, (long long)s.ref_max_width, (long long)s.ref_layered, (long long)s.ref_raw,
                      (long long)s.ref_passthrough, (long long)s.ref_emit, (long long)s.ref_term_emit);
        o += line;
        std::snprintf(line, sizeof line, "Plan: ops=%lld (pass-throughs elided), terminals U=%lld, coeff=%d\n",
                      (long long)s.n_ops, (long long)s.n_terms, s.has_coeff);
        o += line;
        o += "Level\tOps\tEmits\n";
        std::snprintf(line, sizeof line, "0\t0\t%lld\n", (long long)(p->em_off[1] - p->em_off[0]));
        o += line;
        for (int k = 1; k <= p->depth; ++k) {
            std::snprintf(line, sizeof line, "%d\t%lld\t%lld\n", k, (long long)(p->lvl_off[k] - p->lvl_off[k - 1]),
                          (long long)(p->em_off[k + 1] - p->em_off[k]));
            o += line;
        }
        std::vector<double> ws((size_t)std::max(p->depth, 1) * GMR_WINDOW_STATS);
        window_stats(*p, 128, 32, ws.data());
        o += "Left-child windows of 128 rules at 32 words per value: level, share fitting 64/128/200 KB, "
             "density, slot share\n";
        for (int k = 1; k <= p->depth; ++k) {
            const double* w = ws.data() + (size_t)(k - 1) * GMR_WINDOW_STATS;
            std::snprintf(line, sizeof line, "%d\t%.2f\t%.2f\t%.2f\t%.2f\t%.2f\n", k, w[0], w[1], w[2], w[3], w[4]);
            o += line;
        }
        std::snprintf(buf, cap, "%s", o.c_str());
        if (o.size() + 1 > cap) throw Error(GMR_ERR_RANGE, "buffer too small: need " + std::to_string(o.size() + 1));
    });
}

extern "C" int gmr_plan_array(const gmr_plan* p, int which, const void** ptr, int64_t* n) {
    return guarded([&] {
        if (!p || !ptr || !n) throw Error(GMR_ERR_ARG, "null argument");
        switch (which) {
            case 0: *ptr = p->op_l.data(); *n = (int64_t)p->op_l.size(); break;
            case 1: *ptr = p->op_r.data(); *n = (int64_t)p->op_r.size(); break;
            case 2: *ptr = p->op_c.data(); *n = (int64_t)p->op_c.size(); break;
            case 3: *ptr = p->lvl_off.data(); *n = (int64_t)p->lvl_off.size(); break;
            case 4: *ptr = p->em_off.data(); *n = (int64_t)p->em_off.size(); break;
            case 5: *ptr = p->em_src.data(); *n = (int64_t)p->em_src.size(); break;
            case 6: *ptr = p->em_row.data(); *n = (int64_t)p->em_row.size(); break;
            case 7: *ptr = p->term_val.data(); *n = (int64_t)p->term_val.size(); break;
            case 8: *ptr = p->term_col.data(); *n = (int64_t)p->term_col.size(); break;
            case 9: *ptr = p->V.data(); *n = (int64_t)p->V.size(); break;
            case 10: *ptr = p->seg_off.data(); *n = (int64_t)p->seg_off.size(); break;
            case 11: *ptr = p->seg_row.data(); *n = (int64_t)p->seg_row.size(); break;
            case 12: *ptr = p->seg_start.data(); *n = (int64_t)p->seg_start.size(); break;
            case 13: *ptr = p->par_off.data(); *n = (int64_t)p->par_off.size(); break;
            case 14: *ptr = p->par_src.data(); *n = (int64_t)p->par_src.size(); break;
            case 15: *ptr = p->erow_off.data(); *n = (int64_t)p->erow_off.size(); break;
            case 16: *ptr = p->erow_row.data(); *n = (int64_t)p->erow_row.size(); break;
            case 17: *ptr = p->tcol_off.data(); *n = (int64_t)p->tcol_off.size(); break;
            case 18: *ptr = p->tcol_q.data(); *n = (int64_t)p->tcol_q.size(); break;
            case 19: *ptr = p->le_off.data(); *n = (int64_t)p->le_off.size(); break;
            case 20: *ptr = p->le_src.data(); *n = (int64_t)p->le_src.size(); break;
            case 21: *ptr = p->le_tgt.data(); *n = (int64_t)p->le_tgt.size(); break;
            case 22: *ptr = p->le_split.data(); *n = (int64_t)p->le_split.size(); break;
            default: throw Error(GMR_ERR_ARG, "unknown plan array");
        }
    });
}

extern "C" void gmr_plan_free(gmr_plan* p) { delete p; }
