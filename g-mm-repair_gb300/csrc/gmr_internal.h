// Host-side data structures shared by the grammar I/O, the generators, the
// RePair compressor, the schedule builder and the CUDA engine.
#pragma once

#include <cstdint>
#include <string>
#include <vector>
#include <stdexcept>

#include "gmr.h"

namespace gmr {

// Error carrying a gmr status code; caught at the C-ABI boundary.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

// Runs `f` and converts exceptions into a status code + last-error message.
template <class F>
int guarded(F&& f) {
    try {
        f();
        return GMR_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return GMR_ERR_OOM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GMR_ERR_ARG;
    }
}

int default_threads(int requested);

// Run f(t) for t in [0, n_threads) on std::threads.
template <class F>
void parallel_for_threads(int n_threads, F&& f);

}  // namespace gmr

// RePair grammar (reference: gpu-engine/grammar.h:41-63).  Symbol s < alpha
// is a terminal (0 is the row delimiter), s >= alpha is rule s - alpha.
struct gmr_grammar {
    int alpha = 0;
    std::vector<int32_t> rules;  // 2 per rule: left, right
    std::vector<int32_t> kinds;  // 0 binary, 1 run-length
    std::vector<int32_t> reps;   // run-length count (1 for binary)
    std::vector<int32_t> C;      // top sequence, 0 = row end
    std::vector<double> V;       // distinct values
    bool has_runlen = false;
    int64_t n_rules() const { return (int64_t)kinds.size(); }
};

// Uncompressed CSRV string.
struct gmr_csrv {
    int rows = 0, cols = 0;
    std::vector<int32_t> codes;
    std::vector<double> V;
};

// Level-major, child-sorted schedule.  Values live in one arena of n_ops
// slots; a reference (int32) >= 0 is an arena slot, < 0 is terminal
// T[-ref-1] (T[0] is the semiring zero).  Ops of level k occupy slots
// [lvl_off[k-1], lvl_off[k]); level-k emissions [em_off[k], em_off[k+1])
// (k = 0: terminal occurrences), sorted by (row, source).
struct gmr_plan {
    int rows = 0, cols = 0, depth = 0;
    std::vector<float> V;
    std::vector<int32_t> term_val, term_col;  // for terminals q = 1..U-1
    std::vector<int64_t> lvl_off;             // depth + 1
    std::vector<int32_t> op_l, op_r;
    std::vector<float> op_c;                  // empty unless has_coeff
    std::vector<int64_t> em_off;              // depth + 2
    std::vector<int32_t> em_src, em_row;
    // Row segments: the emissions of one (level, row) pair are contiguous;
    // segment s covers [seg_start[s], seg_start[s+1]) of em_src and folds
    // into row seg_row[s].  Level k's segments are [seg_off[k], seg_off[k+1]).
    std::vector<int64_t> seg_off;             // depth + 2
    std::vector<int32_t> seg_row;             // n_seg
    std::vector<int64_t> seg_start;           // n_seg + 1
    gmr_plan_stats stats{};
    // B-independent per-slot statistics for the cost-model features (lazy)
    mutable std::vector<double> slot_stats;
    // Transpose (left product) structures, built by gmr_plan_prepare_left.
    // Node u = arena slot (u < n_ops) or terminal n_ops + q.  Parents of u:
    // par_src[par_off[u] .. par_off[u+1]), p >= 0 when u is p's left child,
    // ~p when it is the right child.  Rows emitting u: erow_row[erow_off[u]..).
    // Terminals of column c: tcol_q[tcol_off[c] .. tcol_off[c+1]) (q >= 1).
    std::vector<int64_t> par_off, erow_off, tcol_off;
    std::vector<int32_t> par_src, erow_row, tcol_q;
    // The same edges flattened for the chunked left fold: edge e adds source
    // le_src[e] into target le_tgt[e].  Sources: p >= 0 (down value of parent
    // p, u its left child, times p's coefficient), ~p (parent p, right child),
    // n_ops + r (x row r).  Targets: arena slot u (levels 1..depth), or
    // compacted terminal q (level 0).  Level k's edges are [le_off[k-1],
    // le_off[k]), terminals' [le_off[depth], le_off[depth+1]); targets are
    // ascending within each range.  le_split: targets whose edges straddle a
    // chunk of kLeftChunk edges (counted from the start of their range),
    // encoded u or n_ops + q; they are folded with atomics into a zeroed value.
    std::vector<int64_t> le_off;
    std::vector<int32_t> le_src, le_tgt, le_split;

    int64_t n_ops() const { return (int64_t)op_l.size(); }
    int64_t n_terms() const { return (int64_t)term_val.size() + 1; }
    bool has_coeff() const { return !op_c.empty(); }
};

namespace gmr {
constexpr int64_t kLeftChunk = 16;  // edges per lane group in the left fold
void validate_plan(const gmr_plan& p);  // throws Error(GMR_ERR_FORMAT)
void fill_common_stats(gmr_plan& p);    // stats derived from the plan arrays
}

#include <thread>
namespace gmr {
template <class F>
void parallel_for_threads(int n_threads, F&& f) {
    if (n_threads <= 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(n_threads);
    for (int t = 0; t < n_threads; ++t) th.emplace_back([&f, t] { f(t); });
    for (auto& x : th) x.join();
}
}  // namespace gmr
