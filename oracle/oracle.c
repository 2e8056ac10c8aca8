/*
 * oracle.c -- CPU restatement of the reference's algorithm for the grammar
 * sweep.  TEST INFRASTRUCTURE ONLY: it is called by tests/, by the smoke
 * check in __graft_entry__.py and by the CPU-baseline leg of bench.py, as
 * the checker and as the timed CPU baseline.  The product path never links,
 * loads or calls it.
 *
 * What it restates (file:line in the reference project, g-mm-repair):
 *   orc_build_schedule   gpu-engine/build_schedule.cpp:42-227
 *                        levels (:57-71), highest referencing level (:73-84),
 *                        layering with pass-through completion (:86-136),
 *                        emit lists from C (:138-155), flattening (:157-185),
 *                        terminal compaction (:187-224)
 *   orc_sweep_f64        gpu-engine/cpu_selftest.cpp:67-102 (cpu_sweep, FP64)
 *                        with the semirings of cpu_selftest.cpp:39-63
 *   orc_cpu_reference    gpu-engine/gpu_engine_test.cu:49-104
 *                        (run_cpu_reference_layered: float / int semirings of
 *                        gpu-engine/gpu_engine.h:46-97, OpenMP per level)
 *   orc_expand           gpu-engine/cpu_selftest.cpp:119-156 (re-expansion)
 *   orc_brute_force      gpu-engine/cpu_selftest.cpp:104-117
 * Terminal decoding follows gpu-engine/gpu_engine_test.cu:373-380:
 * value index (t-1)/cols, column (t-1)%cols.
 *
 * Pinned against the reference itself: the recipe in oracle/Makefile builds
 * the reference's own sources into oracle/_ref, and tests/golden holds the
 * outputs they produced (tests/golden/make_golden.py).
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_TROP_INF 1000000000

enum { ORC_PLUS = 0, ORC_BOOL = 1, ORC_TROP = 2 };

typedef struct {
    int alpha;          /* compacted U */
    int depth, max_width;
    long num_raw, num_layered, num_pt;
    int *left, *right;  /* flattened layered rules */
    float *coeff;
    int *level_offsets; /* depth + 1 */
    int *level_widths;  /* depth + 1 */
    int *emit_offsets;  /* depth + 1 */
    int *emit_pos, *emit_row;
    long emit_total;
    int *term_sym, *term_row;
    long num_term;
    int *term_orig;     /* alpha */
} orc_sched;

static void* xmalloc(size_t n) {
    void* p = malloc(n ? n : 1);
    return p;
}

void orc_sched_free(orc_sched* s) {
    if (!s) return;
    free(s->left); free(s->right); free(s->coeff);
    free(s->level_offsets); free(s->level_widths); free(s->emit_offsets);
    free(s->emit_pos); free(s->emit_row); free(s->term_sym); free(s->term_row);
    free(s->term_orig);
    free(s);
}

/* kinds: NULL = all binary; 1 = run-length left^reps[i]. Returns 0 on success. */
int orc_build_schedule(int alpha, long n, const int* rules, const int* kinds, const int* reps,
                       long c_len, const int* C, orc_sched** out) {
    orc_sched* s = (orc_sched*)calloc(1, sizeof(orc_sched));
    int* lvl = (int*)xmalloc(sizeof(int) * (size_t)n);
    int* mref = (int*)xmalloc(sizeof(int) * (size_t)n);
    int depth = 0;
    long i;
    for (i = 0; i < n; ++i) {
        int l = rules[2 * i], r = rules[2 * i + 1];
        int ll = l >= alpha ? lvl[l - alpha] : 0;
        if (kinds && kinds[i] == 1) {
            lvl[i] = 1 + ll;
        } else {
            int rl = r >= alpha ? lvl[r - alpha] : 0;
            lvl[i] = 1 + (ll > rl ? ll : rl);
        }
        if (lvl[i] > depth) depth = lvl[i];
    }
    for (i = 0; i < n; ++i) mref[i] = lvl[i];
    for (i = 0; i < n; ++i) {
        int l = rules[2 * i], r = rules[2 * i + 1];
        if (l >= alpha && mref[l - alpha] < lvl[i]) mref[l - alpha] = lvl[i];
        if (!(kinds && kinds[i] == 1) && r >= alpha && mref[r - alpha] < lvl[i]) mref[r - alpha] = lvl[i];
    }
    /* sizes per level: raw rules of level k + pass-throughs of level-(k-1)
     * entries whose symbol is referenced above k-1 */
    long* width = (long*)calloc((size_t)depth + 2, sizeof(long));
    for (i = 0; i < n; ++i) {
        int k;
        width[lvl[i]]++;
        for (k = lvl[i] + 1; k <= mref[i]; ++k) width[k]++;
    }
    long total = 0;
    int k;
    s->level_offsets = (int*)xmalloc(sizeof(int) * ((size_t)depth + 1));
    s->level_widths = (int*)xmalloc(sizeof(int) * ((size_t)depth + 1));
    s->level_offsets[0] = 0;
    s->level_widths[0] = 0;
    s->max_width = 0;
    for (k = 1; k <= depth; ++k) {
        total += width[k];
        s->level_offsets[k] = (int)total;
        s->level_widths[k] = (int)width[k];
        if (width[k] > s->max_width) s->max_width = (int)width[k];
    }
    s->depth = depth;
    s->num_raw = n;
    s->num_layered = total;
    s->num_pt = total - n;
    s->left = (int*)xmalloc(sizeof(int) * (size_t)total);
    s->right = (int*)xmalloc(sizeof(int) * (size_t)total);
    s->coeff = (float*)xmalloc(sizeof(float) * (size_t)total);
    /* orig symbol of every slot (for pass-through decisions), slot of each
     * symbol in the latest level it is present in, and at its own level */
    int* orig = (int*)xmalloc(sizeof(int) * (size_t)total);
    int* cur_slot = (int*)xmalloc(sizeof(int) * (size_t)n);
    int* own_slot = (int*)xmalloc(sizeof(int) * (size_t)n);
    int* nxt_slot = (int*)xmalloc(sizeof(int) * (size_t)n);
    /* raw rules grouped by level, in index order */
    long* lstart = (long*)calloc((size_t)depth + 2, sizeof(long));
    long* byl = (long*)xmalloc(sizeof(long) * (size_t)n);
    for (i = 0; i < n; ++i) lstart[lvl[i] + 1]++;
    for (k = 0; k <= depth; ++k) lstart[k + 1] += lstart[k];
    {
        long* fill = (long*)xmalloc(sizeof(long) * ((size_t)depth + 2));
        memcpy(fill, lstart, sizeof(long) * ((size_t)depth + 2));
        for (i = 0; i < n; ++i) byl[fill[lvl[i]]++] = i;
        free(fill);
    }
    for (k = 1; k <= depth; ++k) {
        long base = s->level_offsets[k - 1], idx = 0, j;
        /* raw rules of level k; children as seen in frontier k-1 */
        for (j = lstart[k]; j < lstart[k + 1]; ++j) {
            long r = byl[j];
            int l = rules[2 * r], rr = rules[2 * r + 1];
            s->left[base + idx] = l < alpha ? -l - 1 : cur_slot[l - alpha];
            if (kinds && kinds[r] == 1) {
                s->right[base + idx] = -1;
                s->coeff[base + idx] = (float)reps[r];
            } else {
                s->right[base + idx] = rr < alpha ? -rr - 1 : cur_slot[rr - alpha];
                s->coeff[base + idx] = 1.0f;
            }
            orig[base + idx] = (int)r;
            own_slot[r] = (int)idx;
            nxt_slot[r] = (int)idx;
            ++idx;
        }
        /* pass-throughs of level k-1 entries still referenced above k-1 */
        if (k > 1) {
            long pb = s->level_offsets[k - 2], pw = s->level_widths[k - 1];
            for (j = 0; j < pw; ++j) {
                int o = orig[pb + j];
                if (mref[o] > k - 1) {
                    s->left[base + idx] = (int)j;
                    s->right[base + idx] = -1;
                    s->coeff[base + idx] = 1.0f;
                    orig[base + idx] = o;
                    nxt_slot[o] = (int)idx;
                    ++idx;
                }
            }
        }
        for (j = 0; j < idx; ++j) cur_slot[orig[base + j]] = nxt_slot[orig[base + j]];
    }
    /* emit lists from C: non-terminals at their own level, terminals once */
    long ne_total = 0, nt_total = 0, j;
    long* ecount = (long*)calloc((size_t)depth + 2, sizeof(long));
    for (j = 0; j < c_len; ++j) {
        int c = C[j];
        if (c == 0) continue;
        if (c < alpha) ++nt_total;
        else { ++ne_total; ecount[lvl[c - alpha]]++; }
    }
    s->emit_offsets = (int*)xmalloc(sizeof(int) * ((size_t)depth + 1));
    s->emit_offsets[0] = 0;
    for (k = 1; k <= depth; ++k) s->emit_offsets[k] = s->emit_offsets[k - 1] + (int)ecount[k];
    s->emit_pos = (int*)xmalloc(sizeof(int) * (size_t)ne_total);
    s->emit_row = (int*)xmalloc(sizeof(int) * (size_t)ne_total);
    s->term_sym = (int*)xmalloc(sizeof(int) * (size_t)nt_total);
    s->term_row = (int*)xmalloc(sizeof(int) * (size_t)nt_total);
    s->emit_total = ne_total;
    s->num_term = nt_total;
    {
        long* fill = (long*)xmalloc(sizeof(long) * ((size_t)depth + 1));
        long t = 0;
        int row = 0;
        for (k = 1; k <= depth; ++k) fill[k] = s->emit_offsets[k - 1];
        for (j = 0; j < c_len; ++j) {
            int c = C[j];
            if (c == 0) { ++row; continue; }
            if (c < alpha) { s->term_sym[t] = c; s->term_row[t] = row; ++t; }
            else {
                int N = c - alpha;
                long d = fill[lvl[N]]++;
                s->emit_pos[d] = own_slot[N];
                s->emit_row[d] = row;
            }
        }
        free(fill);
    }
    /* terminal compaction */
    {
        int* remap = (int*)xmalloc(sizeof(int) * (size_t)alpha);
        int t, U = 1;
        for (t = 0; t < alpha; ++t) remap[t] = -1;
        remap[0] = 0;
        for (j = 0; j < total; ++j) {
            if (s->left[j] < 0 && remap[-s->left[j] - 1] < 0) remap[-s->left[j] - 1] = 0;
            if (s->right[j] < 0 && remap[-s->right[j] - 1] < 0) remap[-s->right[j] - 1] = 0;
        }
        for (j = 0; j < nt_total; ++j)
            if (remap[s->term_sym[j]] < 0) remap[s->term_sym[j]] = 0;
        for (t = 1; t < alpha; ++t) if (remap[t] == 0) ++U;
        s->term_orig = (int*)xmalloc(sizeof(int) * (size_t)U);
        s->term_orig[0] = 0;
        U = 1;
        for (t = 1; t < alpha; ++t)
            if (remap[t] == 0) { remap[t] = U; s->term_orig[U++] = t; }
        for (j = 0; j < total; ++j) {
            if (s->left[j] < 0) s->left[j] = -remap[-s->left[j] - 1] - 1;
            if (s->right[j] < 0) s->right[j] = -remap[-s->right[j] - 1] - 1;
        }
        for (j = 0; j < nt_total; ++j) s->term_sym[j] = remap[s->term_sym[j]];
        s->alpha = U;
        free(remap);
    }
    free(lvl); free(mref); free(width); free(orig); free(cur_slot); free(own_slot);
    free(nxt_slot); free(lstart); free(byl); free(ecount);
    *out = s;
    return 0;
}

/* accessors (for ctypes) */
int orc_sched_int(const orc_sched* s, int which, long* out) {
    switch (which) {
        case 0: *out = s->alpha; break;
        case 1: *out = s->depth; break;
        case 2: *out = s->max_width; break;
        case 3: *out = s->num_raw; break;
        case 4: *out = s->num_layered; break;
        case 5: *out = s->num_pt; break;
        case 6: *out = s->emit_total; break;
        case 7: *out = s->num_term; break;
        default: return 1;
    }
    return 0;
}
const int* orc_sched_arr(const orc_sched* s, int which) {
    switch (which) {
        case 0: return s->left;
        case 1: return s->right;
        case 2: return s->level_offsets;
        case 3: return s->level_widths;
        case 4: return s->emit_offsets;
        case 5: return s->emit_pos;
        case 6: return s->emit_row;
        case 7: return s->term_sym;
        case 8: return s->term_row;
        case 9: return s->term_orig;
        default: return 0;
    }
}
const float* orc_sched_coeff(const orc_sched* s) { return s->coeff; }

/* ---- FP64 sweep, cpu_selftest.cpp:39-102 ---- */
static double d_zero(int sr) { return sr == ORC_TROP ? 1e9 : 0.0; }
static double d_oplus(int sr, double a, double b) {
    if (sr == ORC_PLUS) return a + b;
    if (sr == ORC_BOOL) return (a != 0.0 || b != 0.0) ? 1.0 : 0.0;
    return a < b ? a : b;
}
static double d_leaf(int sr, double V, double x) {
    if (sr == ORC_PLUS) return V * x;
    if (sr == ORC_BOOL) return (V != 0.0 && x != 0.0) ? 1.0 : 0.0;
    {
        long iv = (long)V, ix = (long)x;
        if (iv >= 1000000000L || ix >= 1000000000L) return 1e9;
        return (double)(iv + ix);
    }
}
static double d_apply(int sr, double v, double c) { return sr == ORC_PLUS ? c * v : v; }

int orc_sweep_f64(const orc_sched* s, int sr, const double* V, const float* x, int rows, int cols, double* y) {
    int U = s->alpha, k, r;
    double* T = (double*)xmalloc(sizeof(double) * (size_t)U);
    double *prev = (double*)xmalloc(sizeof(double) * ((size_t)s->max_width + 1));
    double *cur = (double*)xmalloc(sizeof(double) * ((size_t)s->max_width + 1));
    long e, j;
    T[0] = d_zero(sr);
    for (j = 1; j < U; ++j) {
        int t = s->term_orig[j];
        T[j] = d_leaf(sr, V[(t - 1) / cols], x[(t - 1) % cols]);
    }
    for (r = 0; r < rows; ++r) y[r] = d_zero(sr);
    for (e = 0; e < s->num_term; ++e) y[s->term_row[e]] = d_oplus(sr, y[s->term_row[e]], T[s->term_sym[e]]);
    for (k = 1; k <= s->depth; ++k) {
        long a = s->level_offsets[k - 1], b = s->level_offsets[k];
        for (j = a; j < b; ++j) {
            int L = s->left[j], R = s->right[j];
            double lv = L >= 0 ? prev[L] : T[-L - 1];
            double rv = R >= 0 ? prev[R] : T[-R - 1];
            cur[j - a] = d_oplus(sr, d_apply(sr, lv, (double)s->coeff[j]), rv);
        }
        for (e = s->emit_offsets[k - 1]; e < s->emit_offsets[k]; ++e)
            y[s->emit_row[e]] = d_oplus(sr, y[s->emit_row[e]], cur[s->emit_pos[e]]);
        { double* t = prev; prev = cur; cur = t; }
    }
    free(T); free(prev); free(cur);
    return 0;
}

/* ---- float / int sweep, gpu_engine_test.cu:49-104 with gpu_engine.h:46-97 ---- */
static int i_leaf(int sr, float Vv, float xv) {
    if (sr == ORC_BOOL) return (Vv != 0.0f && xv != 0.0f) ? 1 : 0;
    {
        /* float -> int conversion; inputs beyond the int range count as +inf */
        int iv = Vv >= 2147483647.0f ? INT_MAX : (Vv <= -2147483648.0f ? INT_MIN : (int)Vv);
        int ix = xv >= 2147483647.0f ? INT_MAX : (xv <= -2147483648.0f ? INT_MIN : (int)xv);
        if (iv >= ORC_TROP_INF || ix >= ORC_TROP_INF) return ORC_TROP_INF;
        return iv + ix;
    }
}

int orc_cpu_reference(const orc_sched* s, int sr, const float* V, const float* x, int rows, int cols,
                      void* yout, int n_threads) {
    int U = s->alpha;
    long j, e;
    int k;
    (void)cols;
#ifdef _OPENMP
    int saved = omp_get_max_threads();
    omp_set_num_threads(n_threads > 0 ? n_threads : saved);
#else
    (void)n_threads;
#endif
    if (sr == ORC_PLUS) {
        float* y = (float*)yout;
        float* T = (float*)xmalloc(sizeof(float) * (size_t)U);
        float* rd = (float*)xmalloc(sizeof(float) * ((size_t)s->max_width + 1));
        float* wr = (float*)xmalloc(sizeof(float) * ((size_t)s->max_width + 1));
        T[0] = 0.0f;
        /* val/col index tables as the reference driver builds them */
#pragma omp parallel for if (U > 1000)
        for (j = 1; j < U; ++j) {
            int t = s->term_orig[j];
            T[j] = V[(t - 1) / cols] * x[(t - 1) % cols];
        }
#pragma omp parallel for if (rows > 1000)
        for (j = 0; j < rows; ++j) y[j] = 0.0f;
#pragma omp parallel for if (s->num_term > 1000)
        for (e = 0; e < s->num_term; ++e) {
#pragma omp atomic
            y[s->term_row[e]] += T[s->term_sym[e]];
        }
        for (k = 1; k <= s->depth; ++k) {
            long a = s->level_offsets[k - 1], nr = s->level_offsets[k] - a;
            long ea = s->emit_offsets[k - 1], ne = s->emit_offsets[k] - ea;
#pragma omp parallel for if (nr > 1000)
            for (j = 0; j < nr; ++j) {
                int L = s->left[a + j], R = s->right[a + j];
                float lv = L >= 0 ? rd[L] : T[-L - 1];
                float rv = R >= 0 ? rd[R] : T[-R - 1];
                float av = s->coeff[a + j] * lv;
                wr[j] = av + rv;
            }
#pragma omp parallel for if (ne > 1000)
            for (e = 0; e < ne; ++e) {
#pragma omp atomic
                y[s->emit_row[ea + e]] += wr[s->emit_pos[ea + e]];
            }
            { float* t = rd; rd = wr; wr = t; }
        }
        free(T); free(rd); free(wr);
    } else {
        int* y = (int*)yout;
        int* T = (int*)xmalloc(sizeof(int) * (size_t)U);
        int* rd = (int*)xmalloc(sizeof(int) * ((size_t)s->max_width + 1));
        int* wr = (int*)xmalloc(sizeof(int) * ((size_t)s->max_width + 1));
        const int zero = sr == ORC_TROP ? ORC_TROP_INF : 0;
        T[0] = zero;
#pragma omp parallel for if (U > 1000)
        for (j = 1; j < U; ++j) {
            int t = s->term_orig[j];
            T[j] = i_leaf(sr, V[(t - 1) / cols], x[(t - 1) % cols]);
        }
#pragma omp parallel for if (rows > 1000)
        for (j = 0; j < rows; ++j) y[j] = zero;
        for (k = 0; k <= s->depth; ++k) {
            long a = 0, nr = 0, ea, ne;
            int* src;
            const int* pos;
            const int* row;
            if (k == 0) {
                ea = 0; ne = s->num_term; src = T; pos = s->term_sym; row = s->term_row;
            } else {
                a = s->level_offsets[k - 1];
                nr = s->level_offsets[k] - a;
#pragma omp parallel for if (nr > 1000)
                for (j = 0; j < nr; ++j) {
                    int L = s->left[a + j], R = s->right[a + j];
                    int lv = L >= 0 ? rd[L] : T[-L - 1];
                    int rv = R >= 0 ? rd[R] : T[-R - 1];
                    wr[j] = sr == ORC_BOOL ? (lv | rv) : (lv < rv ? lv : rv);
                }
                ea = s->emit_offsets[k - 1];
                ne = s->emit_offsets[k] - ea;
                src = wr; pos = s->emit_pos + ea; row = s->emit_row + ea;
            }
            if (sr == ORC_BOOL) {
#pragma omp parallel for if (ne > 1000)
                for (e = 0; e < ne; ++e) {
#pragma omp atomic
                    y[row[e]] |= src[pos[e]];
                }
            } else {
#pragma omp parallel for if (ne > 1000)
                for (e = 0; e < ne; ++e) {
                    int v = src[pos[e]];
#pragma omp critical(orc_tropical_emit)
                    {
                        if (v < y[row[e]]) y[row[e]] = v;
                    }
                }
            }
            if (k > 0) { int* t = rd; rd = wr; wr = t; }
        }
        free(T); free(rd); free(wr);
    }
#ifdef _OPENMP
    omp_set_num_threads(saved);
#endif
    return 0;
}

/* ---- CSRV re-expansion and brute force, cpu_selftest.cpp:104-156 ---- */
static long expand_len(int alpha, const int* rules, const int* kinds, const int* reps, long* memo, int sym) {
    if (sym < alpha) return 1;
    {
        int i = sym - alpha;
        if (memo[i] >= 0) return memo[i];
        if (kinds && kinds[i] == 1)
            memo[i] = (long)reps[i] * expand_len(alpha, rules, kinds, reps, memo, rules[2 * i]);
        else
            memo[i] = expand_len(alpha, rules, kinds, reps, memo, rules[2 * i]) +
                      expand_len(alpha, rules, kinds, reps, memo, rules[2 * i + 1]);
        return memo[i];
    }
}

static long expand_into(int alpha, const int* rules, const int* kinds, const int* reps, int sym, int* out, long o) {
    if (sym < alpha) { out[o] = sym; return o + 1; }
    {
        int i = sym - alpha, r;
        if (kinds && kinds[i] == 1) {
            for (r = 0; r < reps[i]; ++r) o = expand_into(alpha, rules, kinds, reps, rules[2 * i], out, o);
        } else {
            o = expand_into(alpha, rules, kinds, reps, rules[2 * i], out, o);
            o = expand_into(alpha, rules, kinds, reps, rules[2 * i + 1], out, o);
        }
        return o;
    }
}

/* Expands the grammar back into its CSRV string.  With out == NULL returns
 * the length only. */
long orc_expand(int alpha, long n, const int* rules, const int* kinds, const int* reps, long c_len,
                const int* C, int* out) {
    long* memo = (long*)xmalloc(sizeof(long) * (size_t)n);
    long j, len = 0, o = 0;
    for (j = 0; j < n; ++j) memo[j] = -1;
    for (j = 0; j < c_len; ++j) len += C[j] == 0 ? 1 : expand_len(alpha, rules, kinds, reps, memo, C[j]);
    free(memo);
    if (!out) return len;
    for (j = 0; j < c_len; ++j) {
        if (C[j] == 0) out[o++] = 0;
        else o = expand_into(alpha, rules, kinds, reps, C[j], out, o);
    }
    return o;
}

int orc_brute_force(long len, const int* vc, int sr, const double* V, const float* x, int rows, int cols,
                    double* y) {
    long j;
    int row = 0, r;
    for (r = 0; r < rows; ++r) y[r] = d_zero(sr);
    for (j = 0; j < len; ++j) {
        int code = vc[j];
        if (code == 0) { ++row; continue; }
        y[row] = d_oplus(sr, y[row], d_leaf(sr, V[(code - 1) / cols], x[(code - 1) % cols]));
    }
    return 0;
}
