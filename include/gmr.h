/*
 * gmr.h -- C-ABI of the GB300-native engine for right multiplication
 * y = M x and Y = M X over RePair grammar-compressed matrices.
 *
 * Two groups of entry points:
 *
 *  1. The drop-in legacy pair, with exactly the signatures of the
 *     reference's gpu-engine/gpu_engine.h:99-136
 *       run_gpu_right_multiply_layered   (replaces gpu_engine.cu:364-397)
 *       run_gpu_right_multiply_batched   (replaces gpu_engine.cu:563-586)
 *     They take the reference's proper-layered schedule (LayeredRule +
 *     GPUSchedule, gpu-engine/layered_types.h:45-75) in HOST memory, choose
 *     the semiring from the SEMIRING environment variable, run `iters`
 *     multiplies and print the same stdout lines as the reference
 *     ("GPU kernel: ... ms/vector.", "MEM analytic bytes: ...", ...).
 *     Like the reference they return nothing; on a CUDA error they print
 *     "CUDA Error: ..." and exit(1) (gpu_engine.cu:38-46).
 *
 *  2. A status-returning handle API (no counterpart function in the
 *     reference; it splits the reference's per-call "allocate, copy,
 *     sweep, copy back, free" into load-once / multiply-many):
 *       grammar I/O   gmr_grammar_*   (.vc.R / .vc.C / .val, the format read
 *                                      at gpu_engine_test.cu:291-345)
 *       generators    gmr_gen_*, gmr_repair_compress (synthetic inputs)
 *       schedule      gmr_plan_*      (replaces build_schedule.cpp:42-227 and
 *                                      host_scheduler.cpp:31-102)
 *       engine        gmr_engine_*    (device-resident multiply)
 *     Every call returns GMR_OK (0) or an error code; gmr_last_error()
 *     gives the message of the calling thread's last failure.
 *
 * No CUDA or torch types appear in the signatures: streams are passed as
 * `void*` (a cudaStream_t), device buffers as plain pointers.
 */
#ifndef GMR_H
#define GMR_H

#include <stddef.h>
#include <stdint.h>

/* The reference's schedule structs, byte-identical to
 * gpu-engine/layered_types.h:45-75 and guarded by the same macro, so a
 * caller that already included the reference header keeps its definitions. */
#ifndef LAYERED_TYPES_H
#define LAYERED_TYPES_H
struct LayeredRule {
    int left;    /* >= 0: slot in the previous frontier; < 0: terminal T[-left-1] */
    int right;   /* same encoding; -1 is the zero terminal T[0] */
    float coeff; /* 1 for binary / pass-through rules, t for run-length rules */
};
struct GPUSchedule {
    int max_depth;
    int max_width;
    int* level_offsets;  /* max_depth + 1 */
    int* level_widths;   /* max_depth + 1 */
    int* emit_offsets;   /* max_depth + 1 */
    int* emit_pos;       /* emit_total */
    int* emit_row;       /* emit_total */
    int  emit_total;
    int* term_emit_sym;  /* num_term_emit, index into T */
    int* term_emit_row;  /* num_term_emit */
    int  num_term_emit;
};
#endif
#ifndef __cplusplus
typedef struct LayeredRule LayeredRule;
typedef struct GPUSchedule GPUSchedule;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status codes and semirings                                          */
/* ------------------------------------------------------------------ */
enum {
    GMR_OK = 0,
    GMR_ERR_ARG = 1,      /* bad argument (null pointer, negative size, ...) */
    GMR_ERR_FORMAT = 2,   /* malformed grammar / schedule (out-of-range child, ...) */
    GMR_ERR_IO = 3,       /* file could not be opened / read / written */
    GMR_ERR_CUDA = 4,     /* a CUDA runtime call failed */
    GMR_ERR_OOM = 5,      /* host or device allocation failed */
    GMR_ERR_RANGE = 6,    /* size beyond a documented limit */
    GMR_ERR_TIMEOUT = 7,  /* a bounded device-side wait gave up */
    GMR_ERR_STATE = 8     /* object used in a state that does not allow it */
};

/* Semirings (gpu_engine.h:46-97).  Element types of X / Y:
 *   GMR_PLUS_TIMES  float   X[cols][B], Y[rows][B]            (+, x)
 *   GMR_BOOLEAN     uint32  X[cols][W], Y[rows][W], W=ceil(B/32):
 *                           bit b%32 of word b/32 is right-hand side b  (OR, AND)
 *   GMR_TROPICAL    int32   X[cols][B], Y[rows][B]            (min, +)
 *                           inputs >= 1000000000 (INT_MAX included) are +inf;
 *                           outputs use 1000000000 for +inf, as the reference.
 * Right-hand sides are innermost ("column-contiguous"): X[j*B + b]. */
enum { GMR_PLUS_TIMES = 0, GMR_BOOLEAN = 1, GMR_TROPICAL = 2 };

#define GMR_TROPICAL_INF 1000000000

const char* gmr_last_error(void);
const char* gmr_version(void);

/* ------------------------------------------------------------------ */
/* Grammar (the mm-repair on-disk format)                              */
/* ------------------------------------------------------------------ */
typedef struct gmr_grammar gmr_grammar;
typedef struct {
    int alpha;          /* terminal / non-terminal boundary */
    int64_t n_rules;
    int64_t c_len;      /* length of the top sequence C (0 = row end) */
    int n_vals;         /* distinct values (.val) */
    int has_runlen;     /* 1 if any rule is run-length */
} gmr_grammar_info;

/* Reads <base>.vc.R (int32 alpha, then int32 (left,right) pairs),
 * <base>.vc.C (int32 top sequence) and <base>.val (float64 values). */
int gmr_grammar_load(const char* base, gmr_grammar** out);
int gmr_grammar_save(const gmr_grammar* g, const char* base);
/* rules: 2*n_rules ints (left, right).  kinds/reps may be NULL (all binary);
 * kind 1 = run-length N -> left^rep (grammar.h:43-48). */
int gmr_grammar_create(int alpha, int64_t n_rules, const int32_t* rules,
                       const int32_t* kinds, const int32_t* reps,
                       int64_t c_len, const int32_t* C,
                       int n_vals, const double* V, gmr_grammar** out);
int gmr_grammar_get_info(const gmr_grammar* g, gmr_grammar_info* info);
const int32_t* gmr_grammar_rules(const gmr_grammar* g);  /* 2*n_rules */
const int32_t* gmr_grammar_kinds(const gmr_grammar* g);  /* n_rules */
const int32_t* gmr_grammar_reps(const gmr_grammar* g);   /* n_rules */
const int32_t* gmr_grammar_C(const gmr_grammar* g);      /* c_len */
const double*  gmr_grammar_V(const gmr_grammar* g);      /* n_vals */
void gmr_grammar_free(gmr_grammar* g);

/* ------------------------------------------------------------------ */
/* Uncompressed CSRV matrices, seeded generators, RePair                */
/* ------------------------------------------------------------------ */
/* A CSRV string: per row the terminal codes val_idx*cols + col + 1 in
 * increasing column order, then 0.  (The format mm-repair compresses.) */
typedef struct gmr_csrv gmr_csrv;
typedef struct {
    int rows, cols;
    int64_t len;   /* codes including the row delimiters */
    int64_t nnz;
    int n_vals;
} gmr_csrv_info;

int gmr_csrv_create(int rows, int cols, int64_t len, const int32_t* codes,
                    int n_vals, const double* V, gmr_csrv** out);
/* Dense row-major matrix -> CSRV; distinct non-zero values sorted ascending. */
int gmr_csrv_from_dense(int rows, int cols, const double* M, gmr_csrv** out);
int gmr_csrv_get_info(const gmr_csrv* m, gmr_csrv_info* info);
const int32_t* gmr_csrv_codes(const gmr_csrv* m);
const double*  gmr_csrv_V(const gmr_csrv* m);
void gmr_csrv_free(gmr_csrv* m);

/* Genotype-like mosaic: rows = sites, cols = haplotypes, value 1. */
int gmr_gen_mosaic(int rows, int cols, int founders, double switch_rate,
                   double mutation, uint64_t seed, int n_threads, gmr_csrv** out);
/* Copy-model directed graph, row = node.  weighted = 0: value 1;
 * weighted = 1: integer weights 1..100 (copied entries keep their weight). */
int gmr_gen_copy_graph(int nodes, int degree, double copy_prob, int weighted,
                       uint64_t seed, int n_threads, gmr_csrv** out);
/* Grammar compression of a CSRV string by rounds of RePair pair
 * replacement (most frequent pairs first; rules never span a row end). */
int gmr_repair_compress(const gmr_csrv* m, int n_threads, gmr_grammar** out);
/* The same grammar as gmr_repair_compress (identical rules and C), computed on
 * GPU `device`: per round one radix sort of the pair occurrences, one of the
 * candidates, and scans for the counts and the greedy replacement choices.
 * Needs about 48 bytes of device memory per input symbol. */
int gmr_repair_compress_device(const gmr_csrv* m, int device, gmr_grammar** out);

/* ------------------------------------------------------------------ */
/* Schedule ("plan"): level-major, child-sorted layout                 */
/* ------------------------------------------------------------------ */
typedef struct gmr_plan gmr_plan;
typedef struct {
    int rows, cols, depth, n_vals, has_coeff;
    int64_t n_ops;        /* evaluated rules (identity pass-throughs elided) */
    int64_t n_emit;       /* non-terminal emissions */
    int64_t n_term_emit;  /* terminal emissions */
    int64_t n_terms;      /* compacted terminals U, zero terminal included */
    int64_t max_level_ops;
    /* The reference's proper-layered figures for the same grammar
     * (build_schedule.cpp:42-227): L = depth, w*, |R|, +pt, emissions, U. */
    int64_t ref_layered, ref_raw, ref_passthrough;
    int64_t ref_max_width, ref_emit, ref_term_emit, ref_alpha;
} gmr_plan_stats;

int gmr_plan_build(const gmr_grammar* g, int rows, int cols, gmr_plan** out);
/* The same plan as gmr_plan_build (identical arrays and figures, same errors),
 * built on GPU `device`: replaces the host build_schedule()
 * (build_schedule.cpp:42-227).  validate != 0 also runs the host-side plan
 * check.  Allocates device memory for the build and frees it on return. */
int gmr_plan_build_device(const gmr_grammar* g, int rows, int cols, int device, int validate,
                          gmr_plan** out);
int gmr_plan_from_layered(int rows, int cols, int alpha, int total_layered_rules,
                          const LayeredRule* rules, const int* val_indices,
                          const int* col_indices, const float* V, int n_vals,
                          const GPUSchedule* sched, gmr_plan** out);
int gmr_plan_get_stats(const gmr_plan* p, gmr_plan_stats* s);
/* ops[k] for k = 0..depth (ops[0] = 0) */
int gmr_plan_level_ops(const gmr_plan* p, int64_t* out, int n);
/* emissions of level k (k = 0: terminal emissions) for k = 0..depth */
int gmr_plan_level_emits(const gmr_plan* p, int64_t* out, int n);
/* Algorithmic bytes of one multiply of B right-hand sides, the reference's
 * analytic accounting (gpu_engine.cu:174-184) without the scratch frontiers:
 * 12*N_L + 8*E + 8*E_T + 8*(U-1) + 4*n_V + 4*cols*B' + 4*rows*B',
 * B' = B, or ceil(B/32) for the bit-packed Boolean semiring. */
double gmr_plan_alg_bytes(const gmr_plan* p, int semiring, int B);
/* Read-only view of a plan array, for inspection and tests:
 * which = 0 op_l, 1 op_r (int32 references: >= 0 arena slot, < 0 terminal
 * -ref-1), 2 op_c (float, absent unless run-length rules exist), 3 lvl_off
 * (int64, depth+1), 4 em_off (int64, depth+2), 5 em_src (int32),
 * 6 em_row (int32), 7 term_val (int32), 8 term_col (int32), 9 V (float),
 * 10 seg_off (int64, depth+2), 11 seg_row (int32), 12 seg_start (int64,
 * n_seg+1): the emissions of one (level, row) pair form one row segment;
 * after gmr_plan_prepare_left: 13 par_off (int64), 14 par_src (int32),
 * 15 erow_off (int64), 16 erow_row (int32), 17 tcol_off (int64),
 * 18 tcol_q (int32), 19 le_off (int64, depth+2), 20 le_src (int32),
 * 21 le_tgt (int32), 22 le_split (int32) (see gmr_plan_prepare_left).
 * *ptr stays valid until gmr_plan_free. */
int gmr_plan_array(const gmr_plan* p, int which, const void** ptr, int64_t* n);
/* Human-readable per-level report (the host_scheduler inspector), with the
 * left-child window statistics below at 128 rules per CTA and 32 words. */
int gmr_plan_describe(const gmr_plan* p, char* buf, size_t cap);
/* Left-child windows for shared-memory staging.  Within a level the rules
 * are sorted by left child, so the arena slots referenced by the left
 * children of rules_per_cta consecutive rules form one window [first, last].
 * For each level k = 1..depth, out[(k-1) * GMR_WINDOW_STATS + j]: j = 0, 1, 2
 * the share of the level's runs of rules_per_cta rules whose window holds at
 * most 64 / 128 / 200 KB of values of `words` 4-byte words; j = 3 the mean
 * density of the windows (distinct referenced slots / window slots); j = 4
 * the share of left children that are slots (the others are terminals).
 * *n = depth. */
#define GMR_WINDOW_STATS 5
int gmr_plan_window_stats(const gmr_plan* p, int rules_per_cta, int words, double* out, int cap, int* n);
void gmr_plan_free(gmr_plan* p);

/* ------------------------------------------------------------------ */
/* Engine: device-resident schedule + multiply                          */
/* ------------------------------------------------------------------ */
typedef struct gmr_engine gmr_engine;

/* Kernel-variant knobs; 0 = let the engine choose. */
typedef struct {
    int variant;      /* GMR_VARIANT_* */
    int vec_tile;     /* words per right-hand-side tile (must divide the
                         batch's words; 0 = engine default) */
    int ops_per_cta;  /* emissions per lane group in GMR_EMIT_SEGMENTED */
    int emit_mode;    /* GMR_EMIT_* */
    int tile_levels;  /* levels 1..tile_levels run tile by tile, the rest
                         all tiles per launch (0 = by level size) */
    int spin_limit;   /* GMR_VARIANT_PERSISTENT: polls a grid-barrier wait
                         may take before it gives up (0 = 20,000,000) */
    int push;         /* GMR_PUSH_*: whether rules fold their own values into
                         the rows that emit them (see GMR_LEVEL_PUSH) */
    int lane_bytes;   /* bytes each lane moves per value access: 16, or 32
                         (256-bit loads and stores, 8 words per lane; used for
                         (+,x) and (min,+) when the tile is 8, 16, 32, 64 or
                         128 words and X and Y are 32-byte aligned, else 16);
                         0 = engine default: 32 for (+,x) tiles of 32 words
                         or more, else 16 (GMR_LANE_BYTES=16|32 at engine
                         creation overrides it) */
} gmr_config;
enum {
    GMR_PUSH_AUTO = 0,       /* the installed per-launch table, else the engine's rule */
    GMR_PUSH_NEVER = 1,      /* every level's emissions are gathered by the next launch */
    GMR_PUSH_ALWAYS = 2,     /* every level that can push does */
    GMR_PUSH_INTERLEAVE = 3  /* every level that can interleaves (GMR_LEVEL_INTERLEAVE) */
};
enum {
    GMR_VARIANT_AUTO = 0,
    GMR_VARIANT_PLAIN = 1,   /* per-level launches, one atomic per emission */
    GMR_VARIANT_FUSED = 2,   /* per-level launches, ops+emits fused */
    GMR_VARIANT_GRAPH = 3,   /* FUSED captured once into a CUDA graph */
    GMR_VARIANT_PERSISTENT = 4 /* one cooperative launch walks every level */
};
enum {
    GMR_EMIT_AUTO = 0,
    GMR_EMIT_ATOMIC = 1,     /* one atomic per (emission, word) */
    GMR_EMIT_SEGMENTED = 2,  /* warp/chunk segmented reduction, one atomic per segment */
    GMR_EMIT_ROWS = 3        /* row-owned segments, plain read-modify-write */
};

int gmr_engine_create(const gmr_plan* p, int device, gmr_engine** out);
/* dX, dY: device pointers (layouts above). stream: cudaStream_t or NULL. */
int gmr_engine_multiply(gmr_engine* e, int semiring, const void* dX, void* dY,
                        int B, const gmr_config* cfg, void* stream);
/* Host buffers: copies X in, multiplies, copies Y out, synchronous. */
int gmr_engine_multiply_host(gmr_engine* e, int semiring, const void* hX,
                             void* hY, int B, const gmr_config* cfg);
/* n independent multiplies with host buffers (hX[i] -> hY[i]), pipelined:
 * two device staging pairs, so that copying X of multiply i+1 in and Y of
 * multiply i-1 out overlap multiply i.  The copies overlap only when the host
 * buffers are page-locked (cudaHostAlloc / cudaHostRegister).  Synchronous:
 * returns when every hY[i] is written. */
int gmr_engine_multiply_host_many(gmr_engine* e, int semiring, const void* const* hX,
                                  void* const* hY, int n, int B, const gmr_config* cfg);
/* Runs one multiply launch by launch (no graph) with a CUDA event pair
 * around every launch and writes the device time of each launch (ms) to
 * ms[0..*n): launch 0 is the prologue (Y = zero, terminal values), launch k
 * evaluates level k and folds the emissions of level k-1, the last launch
 * folds the emissions of the top level.  The engine's timing recorder. */
int gmr_engine_time_launches(gmr_engine* e, int semiring, const void* dX, void* dY,
                             int B, const gmr_config* cfg, void* stream,
                             float* ms, int cap, int* n);
/* Per-launch kernel variants (the autotuner's and the learned model's
 * decision table).  Launch slot 0 is the prologue (ignored), slot k the launch
 * of level k (rules of level k + emissions of level k-1), slot depth+1 the
 * final fold.  Variant v = e + 5 * g + 10 * c: e = 0 segmented chunk 16,
 * 1 chunk 8, 2 chunk 32 (for one lane per emission all three are the
 * warp-shuffle reduction), 3 row-owned, 4 one atomic per emission; g = 0 up
 * to 32 CTAs per SM evaluate the rules, g = 1 up to 4 (more rules per CTA);
 * c = 1 folds the emissions one source chunk (2^19 slots of the level) at a
 * time, one launch per chunk, so the chunk's values stay in L2.  An installed
 * table is used by GMR_VARIANT_AUTO multiplies of that (semiring, B).
 * Adding GMR_LEVEL_PUSH to slot k's entry (1 <= k <= depth) makes the rules of
 * level k push their values into the rows that emit them as soon as they are
 * computed (vector reductions into Y, which stays in L2), so launch k+1
 * gathers nothing of level k; a launch that pushes folds level k-1 with
 * atomics (a row-owned fold there becomes the segmented one).  Adding
 * GMR_LEVEL_INTERLEAVE instead evaluates level k in source chunks (2^19
 * slots, the chunks of c = 1 above), one launch per chunk, each launch also
 * folding the emissions of the chunk before it while that chunk's values are
 * still in L2; launch k+1 folds the last chunk.  Levels of one chunk, and
 * levels that run tile by tile, ignore the flag.
 * n = depth + 2; v = NULL clears. */
#define GMR_N_LEVEL_VARIANTS 20
#define GMR_LEVEL_PUSH 32
#define GMR_LEVEL_INTERLEAVE 64
/* Adding GMR_LEVEL_STAGE to slot k's entry (1 <= k <= depth) stages the
 * left-child window of the rules of level k in shared memory: a block takes
 * runs of 2 x (256 / lanes per rule) consecutive rules, whose left children
 * (the level is sorted by left child) lie in one window of the arena; one
 * bulk copy (cp.async.bulk on an mbarrier) brings that window into 47 KB of
 * shared memory while the right children are gathered, and the left children
 * are read from there (runs whose window is larger read from global memory).
 * That launch folds its emissions with the segmented fold.  Needs 16- or
 * 32-byte lanes in power-of-two groups, no direct terminals, and a level
 * that does not push; otherwise ignored.  Its waits are bounded: one that
 * gives up is reported by gmr_engine_status (phase = -k). */
#define GMR_LEVEL_STAGE 128
int gmr_engine_set_level_variants(gmr_engine* e, int semiring, int B, const uint8_t* v, int n);
int gmr_engine_get_level_variants(const gmr_engine* e, int semiring, int B, uint8_t* v, int cap, int* n);
/* Exhaustive autotuner: times every variant on every launch (median of
 * `reps` eager runs with the timing recorder), installs the per-launch
 * fastest, and writes the times to ms[slot * GMR_N_LEVEL_VARIANTS + v]. */
int gmr_engine_autotune(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                        void* stream, int reps, float* ms, int cap);
/* The same, trading a little time for fewer DRAM bytes: a launch whose
 * fastest variant is not source-chunked takes its chunked twin when that is at
 * most (1 + tolerance) times slower (the chunked fold reads the gathered values
 * from L2; measured on the 200k x 10k grammar at B = 32 with tolerance 0.10:
 * 1.3 % fewer vectors/s, 10 % less energy per vector).  tolerance = 0 is
 * gmr_engine_autotune. */
int gmr_engine_autotune_energy(gmr_engine* e, int semiring, const void* dX, void* dY, int B,
                               void* stream, int reps, float tolerance, float* ms, int cap);
/* ------------------------------------------------------------------ */
/* Learned cost model for the per-launch variant choice                */
/* ------------------------------------------------------------------ */
/* Features of each launch slot (depth + 2 slots, slot 0 all zero):
 *  0 log1p rules of level k          1 log1p emissions of level k-1
 *  2 log1p row segments of level k-1 3 log1p emissions per segment
 *  4 log1p emissions per distinct source (fan-out)
 *  5..8 fraction of the level's child references from level k-1, k-2,
 *       <= k-3, terminals (child-distance histogram)
 *  9 log1p MB of level k-1 values at this B   10 log2 words per slot
 * 11 semiring is (OR,AND)   12 semiring is (min,+)   13 log1p rows
 * 14 log1p rules in total   15 k / (depth + 1)
 * 16 terminals evaluated in place (the engine's default for plans with more
 *    than 4 terminals per column, such as weighted graphs: no terminal table)
 * out: [slots][GMR_N_BASE_FEATURES]. */
#define GMR_N_BASE_FEATURES 17
int gmr_plan_launch_features(const gmr_plan* p, int semiring, int B, float* out, int cap, int* n_slots);

/* Fully connected ReLU network in -> hidden^layers -> 1 (fp32), trained and
 * evaluated by this library's CUDA kernels.  Input rows are the base
 * features followed by a one-hot of the variant (in = GMR_N_BASE_FEATURES +
 * GMR_N_LEVEL_VARIANTS); the target is log(launch time in microseconds). */
typedef struct gmr_mlp gmr_mlp;
int gmr_mlp_create(int in_dim, int hidden, int layers, uint64_t seed, gmr_mlp** out);
int gmr_mlp_info(const gmr_mlp* m, int* in_dim, int* hidden, int* layers, int64_t* n_params);
/* get / set the flat parameter vector [W1 b1 W2 b2 ... Wout bout] (either may be NULL) */
int gmr_mlp_params(gmr_mlp* m, float* get, const float* set, int64_t n);
/* input normalisation: x' = (x - mean) / std */
int gmr_mlp_set_norm(gmr_mlp* m, const float* mean, const float* std);
int gmr_mlp_predict(const gmr_mlp* m, const float* X, int N, float* Y);
/* gradient of the mean squared error over the N rows (one forward + backward) */
int gmr_mlp_gradients(gmr_mlp* m, const float* X, const float* T, int N, float* grad, int64_t n, float* loss);
/* Adam, mini-batches of `batch` rows, `epochs` passes; final full-data MSE to *loss */
int gmr_mlp_train(gmr_mlp* m, const float* X, const float* T, int N, int epochs, int batch, float lr,
                  uint64_t seed, float* loss);
/* versioned ("GMRMLP01") file with a CRC-32 of its contents */
int gmr_mlp_save(const gmr_mlp* m, const char* path);
int gmr_mlp_load(const char* path, gmr_mlp** out);
void gmr_mlp_free(gmr_mlp* m);
/* Predicts every variant's time on every launch of (semiring, B), installs
 * the per-launch argmin as the engine's table, writes the predictions (log us)
 * to pred[slot * GMR_N_LEVEL_VARIANTS + v] when pred != NULL. */
int gmr_engine_choose_learned(gmr_engine* e, const gmr_plan* p, const gmr_mlp* m, int semiring, int B,
                              float* pred, int cap);

/* Random 128-byte line gather bandwidth (GB/s) of the device over a buffer
 * of buffer_bytes: the access pattern of the sweep's value gathers.  A
 * buffer that fits in L2 gives the L2 ceiling, a large one the HBM ceiling.
 * sequential != 0 reads the lines in order instead (plain read bandwidth).
 * Allocates the buffer for the measurement. */
int gmr_measure_gather_bandwidth(int device, int64_t buffer_bytes, int sequential, float* gbs);
/* The same calibration along the load paths a kernel can take (GB/s of units
 * gathered; the buffer is allocated for the measurement):
 *  GMR_GATHER_LOAD16 / GMR_GATHER_LOAD32: random units of unit_bytes read with
 *    16- / 32-byte lane loads, `depth` (1, 2, 4, 8, 16) loads in flight per
 *    thread before any is used;
 *  GMR_GATHER_SEQ16: the same 16-byte loads over the units in order;
 *  GMR_GATHER_BULK: one bulk copy (cp.async.bulk) per random unit into shared
 *    memory, `depth` (even, 2..64) copies in flight per warp in two stages of
 *    depth/2 copies that complete on one mbarrier phase each, 4 warps per
 *    block; 4 * depth * unit_bytes <= 200 KB.
 * unit_bytes: a power of two in [16, 16384] (at least one lane access).
 * gmr_measure_gather_bandwidth is GMR_GATHER_LOAD16 (or SEQ16), depth 4,
 * 128-byte units.  GMR_ERR_TIMEOUT if a bulk-copy wait gave up. */
enum { GMR_GATHER_LOAD16 = 0, GMR_GATHER_SEQ16 = 1, GMR_GATHER_LOAD32 = 2, GMR_GATHER_BULK = 3 };
int gmr_measure_gather(int device, int64_t buffer_bytes, int mode, int depth, int unit_bytes, float* gbs);

/* Status of the engine's last GMR_VARIANT_PERSISTENT multiply, valid once the
 * stream it ran on has been synchronized: *failed != 0 when a grid-barrier
 * wait gave up (Y of that multiply is not valid), *phase = where (0 =
 * prologue, k = level k).  gmr_engine_multiply_host checks it itself and
 * returns GMR_ERR_TIMEOUT. */
int gmr_engine_status(const gmr_engine* e, int* failed, int* phase);
/* Left product y = x^T M (y[c] = (+)_r x[r] (x) M[r][c]) over the same
 * grammar: a top-down sweep (each symbol's value is the (+) of its parents'
 * values and of x over the rows that emit it), then every column folds
 * leaf(V, value) over its terminals.  x is [rows][words], y [cols][words]
 * (words = B, or ceil(B/32) for GMR_BOOLEAN).  gmr_plan_prepare_left builds
 * the reverse adjacency (parents per symbol, emitting rows per symbol,
 * terminals per column) on the host; gmr_engine_enable_left uploads it.
 * The reference has no counterpart in its engine; mm-repair's CPU mat-vec
 * reports both Ax and xA. */
int gmr_plan_prepare_left(gmr_plan* p);
int gmr_engine_enable_left(gmr_engine* e, gmr_plan* p);
int gmr_engine_multiply_left(gmr_engine* e, int semiring, const void* dX, void* dY, int B, void* stream);

/* Fixpoint iteration x <- x (+) (M (x) x) on a square matrix (rows == cols)
 * in an idempotent semiring: GMR_BOOLEAN grows every bit-packed frontier to
 * the set of nodes that reach it (x | Mx, repeated); GMR_TROPICAL relaxes
 * distances to the initial set (min(x, Mx), Bellman-Ford).  dX holds the start
 * and receives the fixpoint; dY is scratch of the same shape.  Each iteration
 * is one multiply and one merge kernel that flags changes; stops when an
 * iteration changes nothing (it is counted) or after max_iters.  The whole
 * loop is one CUDA graph launch (a conditional while node decides on the
 * device whether to run the next iteration), cached per (X, Y, B).
 * *iters = iterations run.  Synchronous on `stream`.  No counterpart function
 * in the reference, whose semiring sweeps are the single steps of these
 * iterations. */
int gmr_engine_fixpoint(gmr_engine* e, int semiring, void* dX, void* dY, int B, int max_iters,
                        void* stream, int* iters);

/* Several engines in one launch: grammars of uneven size, each with its own
 * semiring, X, Y and B.  By default (GMR_PACK_GRAPH) one CUDA-graph launch
 * runs one branch per engine concurrently (each branch = that engine's AUTO
 * chain, its own autotuned per-level variants); gmr_pack_set_mode selects the
 * two single-kernel packings instead.
 * The graph is captured on the first call with a given set of arguments and
 * replayed afterwards.  All engines must live on the same device; an engine
 * may belong to one pack call at a time. */
typedef struct gmr_pack gmr_pack;
int gmr_pack_create(gmr_engine* const* engines, int n, gmr_pack** out);
int gmr_pack_multiply(gmr_pack* p, const int* semirings, const void* const* dX, void* const* dY,
                      const int* B, void* stream);
int64_t gmr_pack_last_launches(const gmr_pack* p);
/* How gmr_pack_multiply runs the pack.
 *  GMR_PACK_GRAPH (the default): the graph of per-engine branches above.
 *  GMR_PACK_LEVELS: one launch per level covers every grammar (level k of
 *    each, on its own range of blocks sized by its work: rules of level k and
 *    emissions of level k-1; launch 0 the prologues), depth of the deepest
 *    grammar + 2 launches, captured once into a graph and replayed.  Up to 32
 *    grammars.  Every grammar folds its emissions with the segmented fold.
 *  GMR_PACK_PERSISTENT: ONE cooperative kernel launch walks every grammar:
 *    phase k runs level k of every grammar that still has one, one grammar
 *    after another over the whole grid, with one grid barrier between phases.
 *    Each barrier wait gives up after spin_limit polls (0 = 20,000,000);
 *    gmr_pack_status then reports it.
 * LEVELS and PERSISTENT need one semiring for the whole pack and no engine
 * with direct terminals; otherwise the graph of branches runs. */
enum { GMR_PACK_GRAPH = 0, GMR_PACK_PERSISTENT = 1, GMR_PACK_LEVELS = 2 };
int gmr_pack_set_mode(gmr_pack* p, int mode, int spin_limit);
/* After the stream of the last gmr_pack_multiply has been synchronized:
 * *persistent = 1 if it ran as one persistent launch (GMR_PACK_PERSISTENT), *failed != 0 if a
 * grid-barrier wait gave up (the Y of that call are not valid), *phase = where. */
int gmr_pack_status(const gmr_pack* p, int* persistent, int* failed, int* phase);
void gmr_pack_free(gmr_pack* p);

/* The last gmr_engine_autotune of (semiring, B): each launch slot's time
 * (ms) under each pair of emission modes, out[k * 9 + 3 * mp + m] for slot k
 * with level k-1 in mode mp and level k in mode m (0 pulled, 1 pushed,
 * 2 interleaved; the variants are the autotuner's per-slot choice), -1 where
 * that pair was not measured.  *n_slots = depth + 2, or 0 when no autotune
 * of (semiring, B) has measured the modes. */
int gmr_engine_mode_costs(gmr_engine* e, int semiring, int B, float* out, int cap, int* n_slots);

/* Bytes each lane moves per value access in a default multiply of (semiring,
 * B) with aligned X and Y (32, 16, 8 or 4), or -1 for a bad argument. */
int gmr_engine_lane_bytes(gmr_engine* e, int semiring, int B);

/* Kernel launches issued by the calling thread's last multiply. */
int64_t gmr_engine_last_launches(const gmr_engine* e);
/* Device bytes held by the engine (schedule + scratch). */
int64_t gmr_engine_device_bytes(const gmr_engine* e);
void gmr_engine_free(gmr_engine* e);

/* ------------------------------------------------------------------ */
/* Drop-in legacy entry points (gpu_engine.h:99-136)                   */
/* ------------------------------------------------------------------ */
#ifdef __cplusplus
void run_gpu_right_multiply_layered(
    int rows, int cols, int alpha, int total_layered_rules,
    const LayeredRule* h_rules, const int* h_val_indices, const int* h_col_indices,
    const float* h_V, int num_distinct_vals, const float* h_x,
    const GPUSchedule& h_sched, float* h_y, int iters);
void run_gpu_right_multiply_batched(
    int rows, int cols, int alpha, int total_layered_rules,
    const LayeredRule* h_rules, const int* h_val_indices, const int* h_col_indices,
    const float* h_V, int num_distinct_vals, const float* h_X,
    const GPUSchedule& h_sched, float* h_Y, int B, int iters);
#else
/* C view: the C++ reference parameter is passed as a pointer. */
void run_gpu_right_multiply_layered(
    int rows, int cols, int alpha, int total_layered_rules,
    const LayeredRule* h_rules, const int* h_val_indices, const int* h_col_indices,
    const float* h_V, int num_distinct_vals, const float* h_x,
    const GPUSchedule* h_sched, float* h_y, int iters);
void run_gpu_right_multiply_batched(
    int rows, int cols, int alpha, int total_layered_rules,
    const LayeredRule* h_rules, const int* h_val_indices, const int* h_col_indices,
    const float* h_V, int num_distinct_vals, const float* h_X,
    const GPUSchedule* h_sched, float* h_Y, int B, int iters);
#endif

/* ------------------------------------------------------------------ */
/* Multiply without any allocation                                      */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference.  For callers that are not allowed to
 * allocate device memory while they run -- code that executes while another
 * component owns the device allocator (a serving loop with a fixed memory
 * budget, a memory pool that must not grow, work issued between allocator
 * checkpoints) -- this entry point multiplies without calling cudaMalloc,
 * cudaFree or any allocating routine.  The caller keeps the schedule in device
 * memory it obtained its own way (copy the arrays that gmr_plan_array returns)
 * and passes inputs and outputs.  The scratch values (one arena slot per
 * evaluated rule plus the terminal table, (n_ops + n_terms) * words * 4 bytes
 * with words = B, or ceil(B/32) for GMR_BOOLEAN) live in one statically sized
 * device array of GMR_NOALLOC_SCRATCH_BYTES (64 MiB) that every GPU loading
 * the library holds until the process exits.  Larger requests fail with
 * GMR_ERR_RANGE before anything is launched.
 *
 * The first call on a device does the set-up with that device current: it
 * looks the array up (cudaGetSymbolAddress) and loads the code of every kernel
 * this entry point can launch (all semirings and widths), so that no later
 * call loads code onto the device.  Make that first call before any stream
 * capture and before entering the region that must not allocate.  The address
 * is kept for the life of the process: resetting the device
 * (cudaDeviceReset) after the first call is not supported.
 * Every call shares the one array: calls that overlap on the GPU (different
 * streams, or host threads without ordering) race on it and give wrong
 * results; serialize them.  Nothing in the array needs to start at zero:
 * every value is written before it is read within a call.  Launches are the
 * fused per-level kernels with row-owned emission folding, on `stream`. */
#define GMR_NOALLOC_SCRATCH_BYTES (64ull << 20)
typedef struct {
    int rows, cols, depth;
    int64_t n_ops;            /* evaluated rules */
    int64_t n_terms;          /* terminals U, zero terminal included */
    const int64_t* lvl_off;   /* HOST, depth + 1 (gmr_plan_array 3) */
    const int64_t* seg_off;   /* HOST, depth + 2 (gmr_plan_array 10) */
    const int32_t* ops;       /* device, 2 * n_ops: (op_l[i], op_r[i]) pairs, 8-byte aligned */
    const float* op_c;        /* device, n_ops, or NULL when all coefficients are 1 */
    const int32_t* em_src;    /* device (gmr_plan_array 5) */
    const int32_t* seg_row;   /* device (gmr_plan_array 11) */
    const int64_t* seg_start; /* device (gmr_plan_array 12) */
    const int32_t* term_val;  /* device, n_terms - 1 */
    const int32_t* term_col;  /* device, n_terms - 1 */
    const float* V;           /* device */
} gmr_device_plan;
int gmr_multiply_noalloc(const gmr_device_plan* p, int semiring, const void* dX, void* dY,
                         int B, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GMR_H */
