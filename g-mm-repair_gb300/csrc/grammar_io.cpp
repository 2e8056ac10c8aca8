// Grammar and CSRV objects, the mm-repair file format, and error plumbing.
//
// File format (as read by the reference driver, gpu-engine/gpu_engine_test.cu:291-345):
//   <base>.vc.R  int32 alpha, then int32 (left, right) per rule, rule i being
//                symbol alpha + i; children always precede their parent.
//   <base>.vc.C  int32 top sequence C; 0 ends a row.
//   <base>.val   float64 distinct values; terminal t >= 1 decodes to value
//                index (t-1)/cols and column (t-1)%cols.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <thread>

#include "gmr_internal.h"

namespace gmr {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

int default_threads(int requested) {
    if (requested > 0) return requested;
    unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1 : (int)n;
}

template <class T>
static std::vector<T> read_file(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error(GMR_ERR_IO, "cannot open " + path);
    std::fseek(f, 0, SEEK_END);
    long long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0 || sz % (long long)sizeof(T) != 0) {
        std::fclose(f);
        throw Error(GMR_ERR_FORMAT, path + ": size is not a multiple of the element size");
    }
    std::vector<T> v((size_t)(sz / (long long)sizeof(T)));
    if (!v.empty() && std::fread(v.data(), sizeof(T), v.size(), f) != v.size()) {
        std::fclose(f);
        throw Error(GMR_ERR_IO, "short read on " + path);
    }
    std::fclose(f);
    return v;
}

template <class T>
static void write_file(const std::string& path, const T* data, size_t n, const int32_t* head = nullptr) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error(GMR_ERR_IO, "cannot create " + path);
    bool ok = true;
    if (head) ok = std::fwrite(head, sizeof(int32_t), 1, f) == 1;
    if (ok && n) ok = std::fwrite(data, sizeof(T), n, f) == n;
    if (std::fclose(f) != 0) ok = false;
    if (!ok) throw Error(GMR_ERR_IO, "short write on " + path);
}

// Structural checks shared by load/create: children of rule i are symbols
// in [1, alpha + i) (topological numbering; 0 is the row delimiter and never
// a child), C symbols in [0, alpha + n_rules).
static void check_grammar(const gmr_grammar& g) {
    if (g.alpha < 1) throw Error(GMR_ERR_FORMAT, "alpha must be >= 1");
    const int64_t n = g.n_rules();
    if ((int64_t)g.alpha + n > (int64_t)INT32_MAX)
        throw Error(GMR_ERR_RANGE, "alpha + rules exceeds the int32 symbol space");
    for (int64_t i = 0; i < n; ++i) {
        const int64_t lim = (int64_t)g.alpha + i;
        int32_t l = g.rules[2 * i], r = g.rules[2 * i + 1];
        if (l < 1 || l >= lim)
            throw Error(GMR_ERR_FORMAT, "rule " + std::to_string(i) + ": left child " +
                                            std::to_string(l) + " out of range");
        if (g.kinds[i] == 0) {
            if (r < 1 || r >= lim)
                throw Error(GMR_ERR_FORMAT, "rule " + std::to_string(i) + ": right child " +
                                                std::to_string(r) + " out of range");
        } else if (g.kinds[i] == 1) {
            if (g.reps[i] < 1)
                throw Error(GMR_ERR_FORMAT, "rule " + std::to_string(i) + ": run-length count < 1");
        } else {
            throw Error(GMR_ERR_FORMAT, "rule " + std::to_string(i) + ": unknown kind");
        }
    }
    const int64_t top = (int64_t)g.alpha + n;
    for (size_t j = 0; j < g.C.size(); ++j)
        if (g.C[j] < 0 || g.C[j] >= top)
            throw Error(GMR_ERR_FORMAT, "C[" + std::to_string(j) + "] = " + std::to_string(g.C[j]) +
                                            " out of range");
}

}  // namespace gmr

using namespace gmr;

extern "C" {

const char* gmr_last_error(void) { return g_last_error.c_str(); }
const char* gmr_version(void) { return "gmr-gb300 1.0"; }

int gmr_grammar_load(const char* base, gmr_grammar** out) {
    return guarded([&] {
        if (!base || !out) throw Error(GMR_ERR_ARG, "null argument");
        std::string b(base);
        auto R = read_file<int32_t>(b + ".vc.R");
        if (R.empty()) throw Error(GMR_ERR_FORMAT, b + ".vc.R: missing alpha");
        if ((R.size() - 1) % 2 != 0) throw Error(GMR_ERR_FORMAT, b + ".vc.R: truncated rule pair");
        auto g = new gmr_grammar();
        try {
            g->alpha = R[0];
            g->rules.assign(R.begin() + 1, R.end());
            int64_t n = (int64_t)g->rules.size() / 2;
            g->kinds.assign((size_t)n, 0);
            g->reps.assign((size_t)n, 1);
            g->C = read_file<int32_t>(b + ".vc.C");
            g->V = read_file<double>(b + ".val");
            check_grammar(*g);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

int gmr_grammar_save(const gmr_grammar* g, const char* base) {
    return guarded([&] {
        if (!g || !base) throw Error(GMR_ERR_ARG, "null argument");
        if (g->has_runlen) throw Error(GMR_ERR_FORMAT, "the .vc.R format holds binary rules only");
        std::string b(base);
        int32_t a = g->alpha;
        write_file<int32_t>(b + ".vc.R", g->rules.data(), g->rules.size(), &a);
        write_file<int32_t>(b + ".vc.C", g->C.data(), g->C.size());
        write_file<double>(b + ".val", g->V.data(), g->V.size());
    });
}

int gmr_grammar_create(int alpha, int64_t n_rules, const int32_t* rules, const int32_t* kinds,
                       const int32_t* reps, int64_t c_len, const int32_t* C, int n_vals,
                       const double* V, gmr_grammar** out) {
    return guarded([&] {
        if (!out || n_rules < 0 || c_len < 0 || n_vals < 0) throw Error(GMR_ERR_ARG, "bad argument");
        if ((n_rules && !rules) || (c_len && !C) || (n_vals && !V)) throw Error(GMR_ERR_ARG, "null array");
        auto g = new gmr_grammar();
        try {
            g->alpha = alpha;
            g->rules.assign(rules, rules + 2 * n_rules);
            g->kinds.assign((size_t)n_rules, 0);
            g->reps.assign((size_t)n_rules, 1);
            for (int64_t i = 0; i < n_rules; ++i) {
                if (kinds) g->kinds[i] = kinds[i];
                if (reps) g->reps[i] = reps[i];
                if (g->kinds[i] == 1) g->has_runlen = true;
                else g->reps[i] = 1;
            }
            g->C.assign(C, C + c_len);
            g->V.assign(V, V + n_vals);
            check_grammar(*g);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

int gmr_grammar_get_info(const gmr_grammar* g, gmr_grammar_info* info) {
    return guarded([&] {
        if (!g || !info) throw Error(GMR_ERR_ARG, "null argument");
        info->alpha = g->alpha;
        info->n_rules = g->n_rules();
        info->c_len = (int64_t)g->C.size();
        info->n_vals = (int)g->V.size();
        info->has_runlen = g->has_runlen ? 1 : 0;
    });
}

const int32_t* gmr_grammar_rules(const gmr_grammar* g) { return g ? g->rules.data() : nullptr; }
const int32_t* gmr_grammar_kinds(const gmr_grammar* g) { return g ? g->kinds.data() : nullptr; }
const int32_t* gmr_grammar_reps(const gmr_grammar* g) { return g ? g->reps.data() : nullptr; }
const int32_t* gmr_grammar_C(const gmr_grammar* g) { return g ? g->C.data() : nullptr; }
const double* gmr_grammar_V(const gmr_grammar* g) { return g ? g->V.data() : nullptr; }
void gmr_grammar_free(gmr_grammar* g) { delete g; }

int gmr_csrv_create(int rows, int cols, int64_t len, const int32_t* codes, int n_vals,
                    const double* V, gmr_csrv** out) {
    return guarded([&] {
        if (!out || rows < 0 || cols < 1 || len < 0 || n_vals < 1) throw Error(GMR_ERR_ARG, "bad argument");
        if ((len && !codes) || !V) throw Error(GMR_ERR_ARG, "null array");
        if ((int64_t)n_vals * cols + 1 > (int64_t)INT32_MAX)
            throw Error(GMR_ERR_RANGE, "n_vals * cols exceeds the int32 terminal space");
        auto m = new gmr_csrv();
        m->rows = rows;
        m->cols = cols;
        m->codes.assign(codes, codes + len);
        m->V.assign(V, V + n_vals);
        int64_t zeros = 0;
        const int64_t alpha = (int64_t)n_vals * cols + 1;
        for (int64_t i = 0; i < len; ++i) {
            if (codes[i] == 0) ++zeros;
            else if (codes[i] < 0 || codes[i] >= alpha) {
                delete m;
                throw Error(GMR_ERR_FORMAT, "code out of range at " + std::to_string(i));
            }
        }
        if (zeros > rows) {
            delete m;
            throw Error(GMR_ERR_FORMAT, "more row delimiters than rows");
        }
        *out = m;
    });
}

int gmr_csrv_from_dense(int rows, int cols, const double* M, gmr_csrv** out) {
    return guarded([&] {
        if (!out || !M || rows < 0 || cols < 1) throw Error(GMR_ERR_ARG, "bad argument");
        std::vector<double> vals;
        for (int64_t i = 0; i < (int64_t)rows * cols; ++i)
            if (M[i] != 0.0) vals.push_back(M[i]);
        std::sort(vals.begin(), vals.end());
        vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
        if (vals.empty()) vals.push_back(1.0);
        auto m = new gmr_csrv();
        m->rows = rows;
        m->cols = cols;
        m->V = vals;
        for (int r = 0; r < rows; ++r) {
            for (int c = 0; c < cols; ++c) {
                double v = M[(int64_t)r * cols + c];
                if (v == 0.0) continue;
                int vi = (int)(std::lower_bound(vals.begin(), vals.end(), v) - vals.begin());
                m->codes.push_back((int32_t)((int64_t)vi * cols + c + 1));
            }
            m->codes.push_back(0);
        }
        *out = m;
    });
}

int gmr_csrv_get_info(const gmr_csrv* m, gmr_csrv_info* info) {
    return guarded([&] {
        if (!m || !info) throw Error(GMR_ERR_ARG, "null argument");
        info->rows = m->rows;
        info->cols = m->cols;
        info->len = (int64_t)m->codes.size();
        int64_t z = 0;
        for (int32_t c : m->codes) z += (c == 0);
        info->nnz = info->len - z;
        info->n_vals = (int)m->V.size();
    });
}

const int32_t* gmr_csrv_codes(const gmr_csrv* m) { return m ? m->codes.data() : nullptr; }
const double* gmr_csrv_V(const gmr_csrv* m) { return m ? m->V.data() : nullptr; }
void gmr_csrv_free(gmr_csrv* m) { delete m; }

}  // extern "C"
