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

/* ---- engine lifetime ---- */
/* Creates an engine on CUDA device `device`. Allocates nothing large yet. */
int gss_engine_create(int device, gss_engine **out);
int gss_engine_destroy(gss_engine *eng);
/* Launch subsequent work on `stream` (a cudaStream_t; NULL = the engine's
 * own stream). The caller keeps ownership of the stream. */
int gss_engine_set_stream(gss_engine *eng, void *stream);
/* Number of check-kernel launches so far (for launch accounting). */
int64_t gss_engine_launch_count(const gss_engine *eng);
/* When on, each check kernel is bracketed by CUDA events on its stream. */
int gss_engine_set_timing(gss_engine *eng, int on);
/* Sum of the bracketed kernel durations since the last call (waits for
 * them), and how many launches they cover. */
int gss_engine_kernel_time(gss_engine *eng, double *total_ms, int64_t *n_launches);

/* Check-kernel kinds. */
#define GSS_KERNEL_AUTO -1   /* default: picked from the word count at gss_state_set */
#define GSS_KERNEL_DIRECT 0  /* a lane group per clause, one 32-slot word per lane */
#define GSS_KERNEL_TILED 1   /* clause tiles staged in shared memory by bulk copy, K clause slots */
#define GSS_KERNEL_WIDE4 2   /* a lane group per clause, four words per lane (256-bit loads) */
#define GSS_KERNEL_WIDE2 3   /* a lane group per clause, two words per lane (128-bit loads) */
/* Variant flags. */
#define GSS_VARIANT_L2_HINT 1    /* L2 evict-last policy on state loads (direct, tiled) */
#define GSS_VARIANT_OCCUPANCY 2  /* compile-time register cap for 8 blocks per SM (wide) */
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
int64_t gss_db_clause_count(const gss_engine *eng);
int64_t gss_db_literal_count(const gss_engine *eng);
/* Largest variable index used by the database, -1 if empty. */
int64_t gss_db_max_var(const gss_engine *eng);
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

/* ---- the check pass (replaces dFindClauses + DReporter::report,
 *      gpuShareLib/GpuRunner.cu:133-177, gpuShareLib/Reporter.cuh:41-58) ---- */
/* Sets the report capacity (records); 0 = automatic. */
int gss_check_set_capacity(gss_engine *eng, int64_t records);
/* Launches one pass over the whole database against the current state,
 * asynchronously on the engine's stream. */
int gss_check_launch(gss_engine *eng);
/* Waits for the last pass and returns its report count in *n_reports.
 * Returns GSS_ERR_OVERFLOW if the queues overflowed (nothing was lost for
 * good: raise the capacity and launch again). */
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

#ifdef __cplusplus
}
#endif

#endif /* GPUSHARESAT_H */
