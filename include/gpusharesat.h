/*
 * gpusharesat.h - C ABI of the GB300 clause-checking engine.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes (0 = ok,
 * negative = error; gss_last_error() gives the message of the calling
 * thread's last failure). No C++ or torch types cross this boundary, and no
 * C++ exception escapes it.
 *
 * Two layers:
 *
 *  1. The engine ("gss_engine_*", "gss_db_*", "gss_state_*", "gss_check_*"):
 *     a device-resident clause database checked against device-resident
 *     assignment bit planes by the sm_103a kernels. This layer replaces the
 *     reference's device runtime: GpuRunner::wholeRun / launchGpu and the
 *     kernel dFindClauses (gpuShareLib/GpuRunner.cu:133-177, 211-345), the
 *     clause SoA (gpuShareLib/Clauses.cu:47-145) and the report queue
 *     DReporter/Reporter (gpuShareLib/Reporter.cuh:33-127).
 *
 *  2. The clause sharer ("gss_sharer_*"): the C form of the reference's
 *     public C++ API, class GpuShare::GpuClauseSharer
 *     (gpuShareLib/GpuClauseSharer.h:74-163). Each function cites the method
 *     it replaces. The C++ class itself (same vtable order, same factory
 *     GpuShare::makeGpuClauseSharerPtr) is provided over these functions by
 *     include/gpuShareLib/GpuClauseSharer.h.
 *
 * Literals follow the reference: lit = 2*var + sign, sign 1 = negative
 * (gpuShareLib/SolverTypes.h:56-60).
 *
 * Host-facing assignment layout (engine layer): uint32 state[n_vars][n_words][2]
 * = {isDef, isTrue}; bit j of word w is assignment slot 32*w + j. A variable
 * is true in a slot where isDef and isTrue are set, false where isDef is set
 * and isTrue is not, undefined where isDef is clear (isTrue is then ignored),
 * as MultiLBool in gpuShareLib/BaseTypes.cuh:65-78.
 */
#ifndef GPUSHARESAT_H
#define GPUSHARESAT_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define GSS_OK 0
#define GSS_ERR_INVALID -1     /* bad argument (null handle, negative size, bad literal...) */
#define GSS_ERR_CUDA -2        /* a CUDA call failed; see gss_last_error() */
#define GSS_ERR_NOMEM -3       /* device or host allocation failed */
#define GSS_ERR_OVERFLOW -4    /* a report queue overflowed; grow it and run again */
#define GSS_ERR_STATE -5       /* call not valid in the current state */
#define GSS_ERR_NOT_FOUND -6

/* One report: clause `clause` (its index in the engine's database) reports
 * for the slots set in `mask` of 32-slot word `word`. The same 16 bytes as
 * the reference's ReportedClause {mask, solverId, GpuCref}
 * (gpuShareLib/BaseTypes.cuh:146-151), keyed by database index instead of
 * (size, index in size). `solver` is the solver that owns the word. */
typedef struct gss_report {
    uint32_t clause;
    uint32_t word;
    uint32_t mask;
    uint32_t solver;
} gss_report;

typedef struct gss_engine gss_engine;

/* Message for the calling thread's last failed call (never NULL). */
const char *gss_last_error(void);
/* Version string of the library, e.g. "gpusharesat-gb300 0.1 sm_103a". */
const char *gss_version(void);
/* Testing hook, no counterpart in the reference: the next `count` device
 * allocations of at least min_bytes made by the library fail as if the GPU
 * were out of memory (the failure is made on the host; nothing reaches the
 * device). It exercises the out-of-memory recovery of gss_sharer_gpu_run,
 * which follows GpuRunner::wholeRun's notEnoughGpuMemory path
 * (gpuShareLib/GpuRunner.cu:243-260). count = 0 turns it off. Process-wide. */
int gss_debug_fail_device_alloc(int64_t min_bytes, int count);

/* ---- engine lifetime ---- */
/* Creates an engine on CUDA device `device`. Allocates nothing large yet. */
int gss_engine_create(int device, gss_engine **out);
int gss_engine_destroy(gss_engine *eng);
/* Launch subsequent work on `stream` (a cudaStream_t; NULL = the engine's
 * own stream). The caller keeps ownership of the stream. */
int gss_engine_set_stream(gss_engine *eng, void *stream);
/* Number of check-kernel launches so far (for launch accounting). */
int64_t gss_engine_launch_count(const gss_engine *eng);
/* With a GSS_VARIANT_PERSISTENT variant: run each pass as one CUDA graph
 * (counter resets, the kernel, the count readback), captured at the first
 * pass and replayed while the buffers it names stay the same. */
int gss_engine_set_graph(gss_engine *eng, int on);
/* How many times a pass graph was captured (for tests and tuning). */
int64_t gss_engine_graph_captures(const gss_engine *eng);
/* When on, each check kernel is bracketed by CUDA events on its stream. */
int gss_engine_set_timing(gss_engine *eng, int on);
/* Sum of the bracketed kernel durations since the last call (waits for
 * them), and how many launches they cover. */
int gss_engine_kernel_time(gss_engine *eng, double *total_ms, int64_t *n_launches);

/* Check-kernel kinds. */
#define GSS_KERNEL_AUTO -1   /* default: picked from the word count at gss_state_set (8 words or more: the
                                wide kernel in its persistent form, 4 words per lane) */
#define GSS_KERNEL_DIRECT 0  /* a lane group per clause, one 32-slot word per lane */
#define GSS_KERNEL_TILED 1   /* clause tiles staged in shared memory by bulk copy, K clause slots */
#define GSS_KERNEL_WIDE4 2   /* a lane group per clause, four words per lane (256-bit loads) */
#define GSS_KERNEL_WIDE2 3   /* a lane group per clause, two words per lane (128-bit loads) */
/* Variant flags. */
#define GSS_VARIANT_L2_HINT 1    /* L2 evict-last policy on state loads (direct, tiled) */
#define GSS_VARIANT_OCCUPANCY 2  /* compile-time register cap: 8 blocks per SM (wide), 4 (pipelined wide) */
#define GSS_VARIANT_PIPELINED 4  /* wide kinds: next clause's offsets and literals loaded ahead */
#define GSS_VARIANT_PERSISTENT 8 /* wide kinds: one CTA set for the whole pass, tasks from a work counter;
                                    arguments by value, or from device memory when gss_engine_set_graph
                                    replays the pass */
/* Lane layouts of the bucketed kernel (gss_engine_set_length_plan): words
 * per lane x lanes per clause (always one 32-word state row per slot block),
 * and loads in flight per lane. GSS_LAYOUT_SKIP leaves a length class out of
 * the pass (for timing the others). */
#define GSS_LAYOUT_SKIP -1
#define GSS_LAYOUT_4x8_G1 0
#define GSS_LAYOUT_4x8_G2 1
#define GSS_LAYOUT_2x16_G1 2
#define GSS_LAYOUT_2x16_G2 3
#define GSS_LAYOUT_1x32_G1 4
#define GSS_LAYOUT_1x32_G2 5
/* Length plan: the pass checks clauses of length in (max_len[k-1],
 * max_len[k]] (class k; the last class takes everything longer too) with
 * lane layout layout[k], all classes in one persistent launch (the bucketed
 * kernel, arguments and plan in device memory, replayed as a CUDA graph when
 * gss_engine_set_graph is on). Needs a state laid out in 32-word blocks (the
 * wide kinds with 8 or 16 lanes, or the direct kind with 32). n_classes = 0
 * turns the plan off. gpusharesat_gb300.autotune picks the layouts. */
int gss_engine_set_length_plan(gss_engine *eng, int n_classes, const int32_t *max_len, const int32_t *layout);
/* Selects the check-kernel variant. A group of lanes_per_clause lanes checks
 * one clause against a slot block of lanes_per_clause x (words per lane)
 * 32-slot words (0 = automatic: one word per lane up to a full warp, or 32
 * words per block for the wide kinds); `depth` = state loads in flight per
 * lane (direct, wide) or clause slots per group (tiled); `flags` =
 * GSS_VARIANT_*. Takes effect for the next gss_state_set (the state is laid
 * out per slot block). */
int gss_engine_set_variant(gss_engine *eng, int kind, int lanes_per_clause, int depth, int flags);

/* ---- clause database (replaces HostClauses + DClauses,
 *      gpuShareLib/Clauses.cu:297-356 and :47-145) ---- */
/* Replaces the database with n_clauses clauses given in CSR form on the
 * host: clause c is lits[offsets[c] .. offsets[c+1]). Every clause needs at
 * least one literal and at most gss_max_clause_len() literals; literals must
 * be non-negative. Synchronous. */
int gss_db_set(gss_engine *eng, const int32_t *lits, const int64_t *offsets, int64_t n_clauses);
/* Appends n_clauses clauses (CSR on the host) with the given ids (NULL: the
 * ids following the largest one used so far, automatic or given). A report's `clause` is
 * the clause's id; gss_db_set numbers its clauses 0..n-1. Synchronous. */
int gss_db_append(gss_engine *eng, const int32_t *lits, const int64_t *offsets, int64_t n_clauses,
                  const uint32_t *ids);
/* Removes clauses by id: they stop taking part in passes at once (a bit per
 * clause); their space is reclaimed by gss_db_compact. Unknown ids are
 * skipped and reported as GSS_ERR_NOT_FOUND after the known ones are removed. */
int gss_db_delete(gss_engine *eng, const uint32_t *ids, int64_t n);
/* Rewrites the database without the removed clauses (in database order again). */
int gss_db_compact(gss_engine *eng);
/* Database order. The reference keeps clauses in per-size buckets
 * (gpuShareLib/Clauses.cu:47-51); here the variables are also cut into ranges
 * of 2^range_log2: each clause's literals are reordered so that those in its
 * most frequent range come first, then those of its second range, and so on,
 * and the clauses are ordered by (first range, second range, length). Warps
 * that run side by side then gather the state rows of one or two ranges, a
 * working set that stays in L2. Reports do not change (the rule does not
 * depend on literal order). range_log2: -1 automatic (2^17 variables per
 * range), 0 length order only, 11..31. Applies from the next gss_db_set,
 * gss_db_append or gss_db_compact. */
int gss_db_set_locality(gss_engine *eng, int range_log2);
/* log2 of the variables per range of the current database order (0: length
 * order only). */
int gss_db_locality_shift(const gss_engine *eng);
/* Clauses in the database, removed ones included until a compaction. */
int64_t gss_db_clause_count(const gss_engine *eng);
/* Clauses that take part in passes. */
int64_t gss_db_live_count(const gss_engine *eng);
int64_t gss_db_literal_count(const gss_engine *eng);
/* Largest variable index used by the database, -1 if empty. */
int64_t gss_db_max_var(const gss_engine *eng);
/* Position of each clause id in the plain scan order (-1: not in the
 * database); positions change at gss_db_set and gss_db_compact. */
int gss_db_positions(const gss_engine *eng, const uint32_t *ids, int64_t n, int64_t *positions);
int gss_max_clause_len(void);

/* ---- assignment state (replaces HostAssigs::fillAssigsAsync + dUpdateAssigs,
 *      gpuShareLib/Assigs.cu:100-116, 326-372) ---- */
/* Sets the assignment bit planes: state[n_vars][n_words][2] and
 * start[n_words] (slots to check in each word), and solver_of_word[n_words]
 * (may be NULL: word w belongs to solver w). `on_device` = 1 when the three
 * pointers are device pointers (copied device-to-device), 0 for host
 * pointers (copied host-to-device; pinned memory makes this asynchronous).
 * The copy is ordered on the engine's stream. */
int gss_state_set(gss_engine *eng, const uint32_t *state, int64_t n_vars, int n_words,
                  const uint32_t *start, const int32_t *solver_of_word, int on_device);

/* Replaces only the started-slot masks of the current state (n_words must be
 * the state's word count): a new set of assignment batches over the same
 * bit planes, without copying the planes again. */
int gss_state_set_start(gss_engine *eng, const uint32_t *start, int n_words);

/* ---- the check pass (replaces dFindClauses + DReporter::report,
 *      gpuShareLib/GpuRunner.cu:133-177, gpuShareLib/Reporter.cuh:41-58) ---- */
/* Sets the report capacity (records); 0 = automatic. */
int gss_check_set_capacity(gss_engine *eng, int64_t records);
/* Launches one pass over the whole database against the current state,
 * asynchronously on the engine's stream. */
int gss_check_launch(gss_engine *eng);
/* Waits for the last pass and returns its report count in *n_reports (0 when
 * no pass was launched yet). Returns GSS_ERR_OVERFLOW if the queues
 * overflowed (nothing was lost for good: raise the capacity and launch
 * again). */
int gss_check_wait(gss_engine *eng, int64_t *n_reports);
/* Copies the reports of the last pass to host memory `out` (capacity `cap`
 * records), in no particular order. */
int gss_check_copy_reports(gss_engine *eng, gss_report *out, int64_t cap, int64_t *n_reports);
/* One whole pass through host buffers: copies the state from host memory,
 * checks, and copies the reports back (what a caller with host data does
 * per pass). Synchronous. */
int gss_check_pass_host(gss_engine *eng, const uint32_t *state, int64_t n_vars, int n_words,
                        const uint32_t *start, const int32_t *solver_of_word,
                        gss_report *out, int64_t cap, int64_t *n_reports);
/* n_passes whole passes through host buffers, pipelined: while pass i is
 * checked, the state of pass i+1 is copied in and the reports of pass i-1
 * copied out (pinned host buffers make the copies overlap). states[i] (host)
 * holds pass i's bit planes, all with the same n_vars, n_words, start and
 * solver_of_word; outs[i] (host, caps[i] records) receives its reports and
 * n_reports[i] their count. Synchronous: returns when every output is filled. */
int gss_check_passes_host(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars,
                          int n_words, const uint32_t *start, const int32_t *solver_of_word,
                          gss_report *const *outs, const int64_t *caps, int64_t *n_reports);
/* The same passes with the reports packed on the device into 12-byte
 * records {clause, word, mask} (the solver of a word is the caller's
 * solver_of_word[word]): a quarter less to copy back over the host link,
 * which bounds a pass through host buffers. No counterpart in the reference. */
typedef struct gss_report_packed {
    uint32_t clause;
    uint32_t word;
    uint32_t mask;
} gss_report_packed;
int gss_check_passes_host_packed(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars,
                                 int n_words, const uint32_t *start, const int32_t *solver_of_word,
                                 gss_report_packed *const *outs, const int64_t *caps, int64_t *n_reports);
/* The same passes with 8-byte records {cell, mask}, where cell = clause *
 * n_words + word (so clause = cell / n_words, word = cell % n_words): a third
 * less than the 12-byte records over the host link. Needs (largest clause id
 * + 1) x n_words <= 2^32, else GSS_ERR_INVALID. No counterpart in the
 * reference. */
typedef struct gss_report_cell {
    uint32_t cell;
    uint32_t mask;
} gss_report_cell;
int gss_check_passes_host_cells(gss_engine *eng, int n_passes, const uint32_t *const *states, int64_t n_vars,
                                int n_words, const uint32_t *start, const int32_t *solver_of_word,
                                gss_report_cell *const *outs, const int64_t *caps, int64_t *n_reports);

/* ---- measurement probe ----
 * No counterpart in the reference. Random 256-byte row gathers, the access
 * pattern of the check kernels (one state row per literal visit), without the
 * rule: groups of 8 lanes load one random row each (32 bytes a lane), `depth`
 * rows in flight per group (1, 2 or 4), blocks_per_sm blocks of 256 threads
 * per SM, over a fresh device buffer of buffer_bytes. Returns the rows
 * delivered per second and the time of one launch. Allocates and frees the
 * buffer itself; synchronous. */
int gss_probe_gather(int device, uint64_t buffer_bytes, int depth, int blocks_per_sm, double *rows_per_s,
                     double *ms_per_launch);

/* ---- allocation-free check pass ----
 * No counterpart in the reference. For callers that cannot allocate device
 * memory: a solver process that hands its whole GPU budget to its own pool at
 * start-up (a cudaMalloc would then fail or break that budget), or a
 * latency-bound loop that must not stall in the allocator, which can
 * synchronize the device. The caller passes every input and output as device
 * pointers; the call allocates nothing and only queues work on `stream`
 * (NULL = the default stream): it returns before the pass ends.
 *
 * Inputs: the CSR clause database (lits, offsets[n_clauses + 1]); the
 * assignment words in the wide layout, state[n_blocks][n_vars][32][2] =
 * {isDef, isTrue} for words 32*b .. 32*b + 31 (pad past the last word with
 * zeros), start[n_blocks * 32] and solver_of_word[n_blocks * 32].
 * Preconditions. The inputs are in device memory, so the call cannot check
 * them; the engine (gss_db_set, gss_check_launch) checks the same ones and
 * refuses what breaks them. Here breaking one gives wrong reports or reads
 * outside the buffers:
 *   - every literal is 2*var + sign with 0 <= var < n_vars;
 *   - every clause has 1 .. gss_max_clause_len() literals
 *     (offsets[c] < offsets[c + 1]; an empty clause reports every started
 *     slot);
 *   - offsets[0] == 0 and offsets[n_clauses] < 2^31 (offsets are read as
 *     32-bit positions);
 *   - start[] and solver_of_word[] hold n_blocks * 32 entries, start zero
 *     past the last real word (a padding word with start bits set reports).
 * The call itself refuses n_parts outside 1..64, n_clauses > 0 with
 * n_vars == 0, NULL pointers and an output capacity above 2^32 records.
 * Outputs: out[n_parts * cap_per_part] report records, partition p holding
 * min(counts_out[p], cap_per_part) records from out + p * cap_per_part, with
 * `clause` the CSR index; counts_out[n_parts]. A count above cap_per_part
 * means that partition overflowed: run again with more room.
 * Limit: n_parts <= 64. The kernel's reservation counters live in one fixed
 * 256-byte device array, which every GPU that loads this library keeps until
 * the process exits, and which all calls share: overlapping calls on the GPU
 * race and give wrong counts. Each call clears the counters first (they keep
 * the previous call's values). Each call looks up the array's device address
 * on the current device (a host-side lookup that allocates nothing, so the
 * address stays right after a cudaDeviceReset); the first call on a device
 * also loads the library's device code there, so make that first call
 * before any stream capture.
 * The results are the same as gss_check_launch's with the GSS_KERNEL_WIDE4
 * variant (8 lanes per clause, depth 2). */
int gss_check_noalloc(const int32_t *lits, const int64_t *offsets, uint32_t n_clauses, const uint32_t *state,
                      uint32_t n_vars, uint32_t n_blocks, const uint32_t *start, const int32_t *solver_of_word,
                      gss_report *out, uint32_t n_parts, uint32_t cap_per_part, uint32_t *counts_out, void *stream);

/* ---- learned scan order (no counterpart in the reference) ----
 * A 12-64-64-1 MLP scores every clause before each pass from 12 features:
 * length, LBD, age, and the clause's report history (slot reports in each of
 * the last 8 passes, total reports, passes since the last report). The pass
 * then runs as two launches: the head, the first head_fraction of the scan
 * in decreasing score (grouped by length within a score bucket), whose
 * reports gss_check_wait_head returns while the tail still runs; and the
 * tail, the other clauses in the plain order. Every clause is still checked: the report set of a pass is the
 * plain scan's. Weights are FP32; inference runs the two matrix layers on
 * tensor cores with BF16 operands and FP32 accumulation. The order of the
 * next pass is computed on a stream of its own while the tail of the current
 * pass runs, so it sees reports up to two passes back. Training uses a log
 * of (features, reported) rows sampled from past passes: every
 * retrain_interval passes, train_epochs epochs of Adam on minibatches.
 * The learned order runs the direct and wide kernels through
 * gss_check_launch (not the tiled or persistent kernels, nor
 * gss_check_passes_host). */
typedef struct gss_order_params {
    double head_fraction;      /* share of the scan in the head launch (default 0.1) */
    int retrain_interval;      /* passes between trainings (default 1000; 0 = never automatically) */
    int train_epochs;          /* epochs over the log per training (default 2) */
    int batch;                 /* minibatch rows (default 4096) */
    float learning_rate;       /* Adam step size (default 1e-3) */
    int64_t log_capacity;      /* logged rows kept, newest first (default 2^20) */
    double log_rate;           /* share of clauses logged per pass (0 = about 2000 rows a pass) */
    uint64_t seed;             /* weight initialisation and minibatch sampling */
    int overlap;               /* 1: the next pass is scored while this pass's tail runs (default);
                                  0: once this pass has ended */
    int rescore_interval;      /* passes per scoring and sort (default 1: every pass). Between two, each
                                  pass only folds its reports into the history (and logs training rows)
                                  and scans in the last permutation; clauses appended since it was built
                                  are scanned in place after it. */
} gss_order_params;

void gss_order_params_default(gss_order_params *p);
/* Enables the learned order for the next passes (p NULL = defaults); the
 * history starts empty. */
int gss_order_enable(gss_engine *eng, const gss_order_params *p);
int gss_order_disable(gss_engine *eng);
/* 0 = the next passes scan in the plain order and leave the history alone
 * (for comparisons), 1 = learned order again. */
int gss_order_set_active(gss_engine *eng, int on);
/* LBD of clauses by id (0 = unknown, read as the length). */
int gss_db_set_lbd(gss_engine *eng, const uint32_t *ids, const uint16_t *lbd, int64_t n);
/* Waits for the head launch of the pass in flight and copies its reports
 * (they are also among the pass's reports from gss_check_copy_reports). */
int gss_check_wait_head(gss_engine *eng, gss_report *out, int64_t cap, int64_t *n_reports);
/* After gss_check_wait_head: waits for the pass and copies only the reports
 * that were not in its head (head + tail = the pass's reports). */
int gss_check_copy_tail(gss_engine *eng, gss_report *out, int64_t cap, int64_t *n_reports);
typedef struct gss_order_stats {
    int64_t passes;            /* ordered passes so far */
    int64_t trainings;
    double last_loss;          /* mean logistic loss of the last minibatch of the last training */
    int64_t head_positions;    /* scan positions in the head of the last pass */
    int64_t logged;            /* rows in the training log */
    double score_ms;           /* device time of the last pass's history roll, scoring and sort */
    double head_ms, tail_ms;   /* device time of its head and tail launches */
} gss_order_stats;
int gss_order_get_stats(gss_engine *eng, gss_order_stats *out);
/* Trains now on the log, as the automatic retraining does. */
int gss_order_train(gss_engine *eng);
/* Features the next pass will score the given clauses with, x[n][12]. */
int gss_order_clause_features(gss_engine *eng, const uint32_t *ids, int64_t n, float *x);
/* Rank of each clause id in the last ordered pass's scan (0 = scanned
 * first; -1 = not in the database). A diagnostic: it copies and inverts the
 * permutation on the host. */
int gss_order_scan_ranks(gss_engine *eng, const uint32_t *ids, int64_t n, int64_t *ranks);
/* The order's MLP weights (GSS_SCORER_PARAMS floats, layout as below). */
int gss_order_get_weights(gss_engine *eng, float *w);
int gss_order_set_weights(gss_engine *eng, const float *w);

/* The MLP on its own. Flat FP32 weights: W1[64][12], b1[64], W2[64][64],
 * b2[64], w3[64], b3 (5057 floats). */
#define GSS_SCORER_FEATURES 12
#define GSS_SCORER_HIDDEN 64
#define GSS_SCORER_PARAMS 5057
typedef struct gss_scorer gss_scorer;
int gss_scorer_create(int device, uint64_t seed, gss_scorer **out);
int gss_scorer_destroy(gss_scorer *s);
int gss_scorer_get_weights(gss_scorer *s, float *w);
int gss_scorer_set_weights(gss_scorer *s, const float *w);
/* Logits of n rows of features x[n][12] (host memory): BF16 inference. */
int gss_scorer_infer(gss_scorer *s, const float *x, int64_t n, float *logits);
/* Mean logistic loss of rows x with labels y[n] in {0,1}, and its FP32
 * gradient (GSS_SCORER_PARAMS floats); the weights do not change. */
int gss_scorer_gradient(gss_scorer *s, const float *x, const float *y, int64_t n, float *grad, float *loss);
/* One Adam step on rows x, labels y; *loss = the loss before the step. */
int gss_scorer_train_step(gss_scorer *s, const float *x, const float *y, int64_t n, float lr, float *loss);

/* ---- workload helper for the learned-order measurement ----
 * Plants reports into an assignment state kept in device memory in the
 * host-facing layout (uint32 state[n_vars][n_words][2]). Clause c of the
 * device CSR (lits, offsets) is planted in this pass when a hash of
 * (seed, pass, c) falls below rate[c]: in one slot picked by another hash,
 * every literal but the last is made false and the last unassigned.
 * restore = 1 puts back, from `base`, every state word the same call with
 * restore = 0 touched. All pointers are device pointers; `stream` is a
 * cudaStream_t (NULL = the default stream). */
int gss_bench_plant(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, const float *rate,
                    uint32_t *state, const uint32_t *base, int64_t n_vars, int n_words, uint64_t seed, int64_t pass,
                    int restore, void *stream);

/* ---- the clause sharer: C form of GpuShare::GpuClauseSharer
 *      (gpuShareLib/GpuClauseSharer.h:74-163) ---- */

/* Options, field for field GpuClauseSharerOptions (gpuShareLib/GpuClauseSharer.h:25-58);
 * -1 selects the default as there. */
typedef struct gss_sharer_options {
    int gpu_block_count_guideline;        /* sizes the report queues; kernels size their own grids */
    int gpu_threads_per_block_guideline;
    int min_gpu_latency_micros;           /* each gpu_run lasts at least this long (default 50) */
    int verbosity;
    double clause_activity_decay;         /* default 0.99999 */
    int quick_prof;                       /* time the phases of a pass into the global stats */
    int init_report_count_per_category;   /* default 10 */
    int max_page_locked_memory;
} gss_sharer_options;

typedef struct gss_sharer gss_sharer;
typedef void (*gss_log_fn)(const char *message, void *ctx);

/* Fills *o with the defaults of GpuClauseSharerOptions() (GpuClauseSharer.h:48-57). */
void gss_sharer_options_default(gss_sharer_options *o);
/* makeGpuClauseSharerPtr (GpuClauseSharer.h:165); opts may be NULL (defaults),
 * log_fn may be NULL (no log), device < 0 = the calling thread's current
 * CUDA device. */
int gss_sharer_create(const gss_sharer_options *opts, gss_log_fn log_fn, void *log_ctx, int device,
                      gss_sharer **out);
int gss_sharer_destroy(gss_sharer *s);

/* Called from one thread (the GPU thread), or with locking. */
int gss_sharer_gpu_run(gss_sharer *s);                                        /* gpuRun, :83 */
int gss_sharer_reduce_db(gss_sharer *s);                                      /* reduceDb, :87 */
int64_t gss_sharer_added_clause_count(gss_sharer *s);                         /* getAddedClauseCount, :90 */
int64_t gss_sharer_added_clause_count_at_last_reduce_db(gss_sharer *s);       /* :92 */
int gss_sharer_has_run_out_of_gpu_memory_once(gss_sharer *s);                 /* :95 */
int gss_sharer_gpu_mem_info(gss_sharer *s, size_t *free_bytes, size_t *total_bytes);  /* :97 */
int gss_sharer_global_stat_count(void);                                       /* :99 */
int64_t gss_sharer_global_stat(gss_sharer *s, int stat);                      /* getGlobalStat, :101 */
int gss_sharer_write_clauses_in_cnf(gss_sharer *s, FILE *file);               /* :103 */
int gss_sharer_set_var_count(gss_sharer *s, int count);                       /* setVarCount, :105 */
/* addClause (:109): returns the clause's id, or -1 when it has no literal or
 * more than the maximum length (100 unless raised below). solver = -1 when
 * the clause does not come from a solver. Thread safe. */
int64_t gss_sharer_add_clause(gss_sharer *s, int solver, const int *lits, int count);
int gss_sharer_set_cpu_solver_count(gss_sharer *s, int count);                /* :112, not thread safe */
const char *gss_sharer_one_solver_stat_name(int stat);                        /* :118 */
const char *gss_sharer_global_stat_name(int stat);                            /* :120 */
int gss_sharer_one_solver_stat_count(void);                                   /* :122 */

/* Per solver id: from that solver's thread, or with locking. */
int gss_sharer_try_set_solver_values(gss_sharer *s, int solver, const int *lits, int count);  /* :129, 1 = set */
int gss_sharer_unset_solver_values(gss_sharer *s, int solver, const int *lits, int count);    /* :134 */
int64_t gss_sharer_try_send_assignment(gss_sharer *s, int solver);            /* :139, -1 = ring full */
/* popReportedClause (:148): 1 and the clause when one is available, else 0.
 * *lits belongs to the sharer and stays valid until the next pop for the same
 * solver; the caller may reorder the literals in place (solvers do). */
int gss_sharer_pop_reported_clause(gss_sharer *s, int solver, int **lits, int *count, int64_t *gpu_clause_id);
int64_t gss_sharer_last_assig_all_reported(gss_sharer *s, int solver);        /* :151 */
/* getCurrentAssignment (:155): assig[var] = 0 true, 1 false, 2 undefined. */
int gss_sharer_current_assignment(gss_sharer *s, int solver, uint8_t *assig);
int64_t gss_sharer_one_solver_stat(gss_sharer *s, int solver, int stat);     /* :159 */

/* Extensions without a counterpart in GpuClauseSharer: raise the longest
 * accepted clause (up to gss_max_clause_len()), pick the check kernel. */
int gss_sharer_set_max_clause_len(gss_sharer *s, int n);
/* HBM budget for the serving loop: when a pass would check more than
 * max_clauses live clauses, the oldest clauses not reported in the last 8
 * passes are evicted first (then the oldest of the rest); 0 = no budget. */
int gss_sharer_set_clause_budget(gss_sharer *s, int64_t max_clauses);
int64_t gss_sharer_evicted_count(gss_sharer *s);
/* Order-preserving compactions of the device database that dropped evicted
 * clauses on the GPU. */
int64_t gss_sharer_device_compactions(gss_sharer *s);
int gss_sharer_set_variant(gss_sharer *s, int kind, int lanes_per_clause, int depth, int flags);
/* Device order of the sharer's database, as gss_db_set_locality (-1
 * automatic variable ranges, 0 length order, 11..31); applies to batches
 * appended from then on and to reduceDb. No counterpart in the reference. */
int gss_sharer_set_locality(gss_sharer *s, int range_log2);

/* ---- serving load generator (no counterpart in the reference) ----
 * Simulated solver threads drive one sharer on the calling thread's current
 * device the way GpuHelpedSolver does (glucose-syrup/gpu/GpuHelpedSolver.cc:
 * 109-157): trail-like assignments arriving in Poisson batches, a GPU thread
 * running gpu_run in a loop, and a stream of new clauses against an HBM
 * clause budget. Latency of an assignment = from its arrival until
 * last_assig_all_reported passes it. */
typedef struct gss_serving_params {
    double seconds;            /* measured time */
    double warmup_seconds;
    double assign_rate;        /* aggregate assignments per second */
    int n_solvers;
    int n_vars;
    int64_t budget;            /* HBM budget in clauses (0: none) */
    int64_t initial_clauses;   /* database at the start */
    double clause_rate;        /* stream of new clauses per second */
    double plant_rate;         /* fraction of stream clauses planted to report */
    int batch_max;             /* batches of 1..batch_max assignments */
    double trail_fraction;     /* initial trail length / n_vars */
    int trail_change;          /* an assignment unsets and sets 1..trail_change literals */
    uint64_t seed;
    int plain_scan;            /* 1: the plain single-launch scan (grid-stride wide kernel, length order)
                                  instead of the automatic persistent kernel over the range order */
} gss_serving_params;

typedef struct gss_serving_result {
    double p50_ms, p99_ms, p999_ms, mean_ms, max_ms;
    int64_t assignments;       /* completed in the measured window */
    int64_t reports_popped;
    int64_t passes;
    double checks_per_s;       /* clause x assignment checks per second, measured window */
    double assignments_per_s;
    double elapsed_s;
    int64_t evicted;
    int64_t retries;           /* submissions that found the solver's slots full */
    int64_t clauses_streamed;
    int64_t live_clauses_end;
    int64_t device_compactions;
    double run_ms_p50, run_ms_p99, run_ms_max;  /* gpuRun call durations in the measured window */
    int64_t long_runs;         /* gpuRun calls in the measured window that took more than 20 ms */
    /* where those long calls spent their time (ms, summed): waiting for the
     * pass on the GPU, cutting and launching the next, delivering reports,
     * the rest (appending clauses, eviction, compaction) */
    double long_wait_ms, long_launch_ms, long_deliver_ms, long_other_ms;
} gss_serving_result;

int gss_serving_run(const gss_serving_params *p, gss_serving_result *res);

/* ---- the reduceDb policy on its own (host only, no GPU needed) ----
 * Clause activity with decay, bump and rescale, and the thresholds a reduceDb
 * uses (gpuShareLib/Clauses.cu:231-291, 377-417, 488-525). The sharer's
 * reduceDb runs the same code; this handle exposes it for callers and tests. */
typedef struct gss_activity gss_activity;
gss_activity *gss_activity_create(float decay);
void gss_activity_destroy(gss_activity *a);
/* Decays the increment, then adds an entry with that activity; returns its index. */
int64_t gss_activity_add(gss_activity *a, int lbd);
int gss_activity_bump(gss_activity *a, int64_t i);
int gss_activity_decay(gss_activity *a);
float gss_activity_get(const gss_activity *a, int64_t i);
/* Upper bound of the log bucket holding the n-th lowest activity among
 * entries with min_lbd <= lbd < max_lbd (approxNthAct). */
float gss_activity_approx_nth(const gss_activity *a, int min_lbd, int max_lbd, int64_t n);
/* getRemovingLbdAndAct for `total` clauses: keep lbd < *min_lim, or
 * lbd < *max_lim with activity >= *act. */
int gss_activity_removing_thresholds(const gss_activity *a, int act_only, int64_t total, int *min_lim, int *max_lim,
                                     float *act);

#ifdef __cplusplus
}
#endif

#endif /* GPUSHARESAT_H */
