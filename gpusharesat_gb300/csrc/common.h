// Internal helpers shared by the engine, the kernels and the clause sharer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "gpusharesat.h"

namespace gss {

// Longest clause the engine accepts. The reference stops at 100
// (MAX_CL_SIZE, gpuShareLib/BaseTypes.cuh:28); the sharer keeps that limit
// by default, the engine itself takes clauses up to this length.
constexpr int kMaxClauseLen = 4096;

// Tiles of the tiled check kernel: consecutive length-sorted clauses with at
// most kTileLits literals (a longer clause gets a tile of its own and is read
// from global memory). kBufLits leaves room for rounding a tile's literal
// range out to 16-byte boundaries for the bulk copy.
constexpr int kTileLits = 512;
constexpr int kBufLits = kTileLits + 8;

// Zero literals after the last clause: kernels that read a few literals ahead
// stay inside the buffer.
constexpr int kClausePad = 8;

// Database order by variable ranges of 2^shift variables: the key of a
// clause is (its most frequent range, its second range, its length);
// `reordered` (optional, len entries) receives its literals with those of
// the most frequent range first, then the second range's, and so on.
uint64_t range_order_key(const int32_t *lits, int64_t len, int shift, int32_t *reordered);
// The range shift for a database whose largest variable is max_var
// (range_log2: -1 automatic = 17, 0 = no ranges); 0 when one range would do.
int range_shift_for(int64_t max_var, int range_log2);

// Sets the calling thread's error message and returns `code`.
int set_error(int code, const char *fmt, ...);

// Checks a CUDA call; on failure records the message and returns GSS_ERR_CUDA.
#define GSS_CUDA_TRY(call)                                                        \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) {                                                  \
            return ::gss::set_error(GSS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, \
                                    cudaGetErrorString(_e), __FILE__, __LINE__);  \
        }                                                                         \
    } while (0)

#define GSS_TRY(expr)          \
    do {                       \
        int _rc = (expr);      \
        if (_rc != GSS_OK) {   \
            return _rc;        \
        }                      \
    } while (0)

// A device buffer that grows by doubling and never shrinks.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need);  // keeps nothing of the old contents
    int grow_keep(size_t need, cudaStream_t stream, size_t keep_bytes);
    void release();
    ~DevBuf() { release(); }
};

struct PinnedBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need);
    void release();
    ~PinnedBuf() { release(); }
};

// Arguments of one check pass over the length-sorted CSR clause database.
struct CheckArgs {
    const int32_t *lits;        // device, CSR literals, clauses sorted by length
    const int64_t *offsets;     // device, n_clauses + 1
    const uint32_t *orig;       // device, original index of each sorted clause
    uint32_t n_clauses;
    const uint2 *state;         // device, [n_blocks][n_vars][lpc] {isDef, isTrue}
    uint32_t n_vars;
    uint32_t n_blocks;          // slot blocks of lpc words
    const uint32_t *start;      // device, [n_blocks * lpc], zero past the last word
    const int32_t *solver_of_word;  // device, [n_blocks * lpc]
    gss_report *out;            // device, n_parts * cap_per_part records
    uint32_t *counts;           // device, n_parts counters (zeroed by the caller)
    uint32_t n_parts;
    uint32_t cap_per_part;
    int lpc;                    // lanes (32-slot words) per clause
    int g;                      // state loads in flight per lane (direct) / clause slots (tiled)
    int cache_hints;            // L1/L2 eviction hints on the loads
    // tiled kernel only
    const uint32_t *tile_clause;  // device, n_tiles + 1: first sorted clause of each tile
    const uint32_t *tile_lit;     // device, n_tiles + 1: first literal of each tile
    uint32_t n_tiles;
    uint32_t *err;                // device flag, set to nonzero when a bounded wait gives up
    const uint32_t *alive;        // device, 1 bit per clause (NULL: every clause is live)
    uint32_t alive_by_id;         // alive is indexed by orig[c] rather than by c
    // Scan order: this launch checks the clauses at scan positions
    // [scan_begin, scan_end); position i is clause perm[i] when perm is set
    // and i < perm_end, clause i otherwise.
    const uint32_t *perm;
    uint32_t scan_begin, scan_end;
    uint32_t perm_end;
};

__host__ __device__ __forceinline__ uint32_t scan_count(const CheckArgs &a) {
    return a.scan_end > a.scan_begin ? a.scan_end - a.scan_begin : 0u;
}
// Clause at offset i of this launch's scan range (i < scan_count).
__device__ __forceinline__ uint32_t scan_clause(const CheckArgs &a, uint32_t i) {
    const uint32_t p = a.scan_begin + i;
    return (a.perm && p < a.perm_end) ? __ldg(a.perm + p) : p;
}

// Whether clause c of the database takes part in the pass.
__device__ __forceinline__ bool clause_live(const CheckArgs &a, uint32_t c) {
    if (a.alive == nullptr) return true;
    const uint32_t i = a.alive_by_id ? __ldg(a.orig + c) : c;
    return (__ldg(a.alive + (i >> 5)) >> (i & 31)) & 1u;
}

// A per-range lane-layout plan for the bucketed kernel (device memory):
// range k covers scan positions [range_begin[k], range_end[k]) and is checked
// with lane layout layout[k] (GSS_LAYOUT_*); group_base[k] is the index of
// its first clause group over all ranges, group_base[n_ranges] their total.
constexpr uint32_t kMaxRanges = 8192;
struct BucketPlan {
    uint32_t n_ranges;
    uint32_t range_begin[kMaxRanges];
    uint32_t range_end[kMaxRanges];
    int32_t layout[kMaxRanges];
    uint32_t group_base[kMaxRanges + 1];
};
int layout_lanes(int layout);  // lanes per clause of a layout, 0 if unknown
int launch_check_bucketed(const CheckArgs *d_args, const BucketPlan *d_plan, uint32_t *work, cudaStream_t stream,
                          int sm_count);

// Order-preserving device compaction of a CSR clause database: keeps the
// clauses whose id (ids[c]) has its bit set in `alive`.
struct CompactArgs {
    const int32_t *lits;
    const int64_t *offsets;  // n_clauses + 1
    const uint32_t *ids;
    uint32_t n_clauses;
    const uint32_t *alive;   // bit per id
    int32_t *new_lits;       // room for the live literals + kClausePad
    int64_t *new_offsets;    // room for n_clauses + 1
    uint32_t *new_ids;       // room for n_clauses
    void *scratch;           // compact_scratch_bytes(n_clauses), 256-byte aligned
};
size_t compact_scratch_bytes(uint32_t n_clauses);
// Rebuilds a CSR clause database in a new order on the device: new clause c
// is old clause src[c], placed at new_offsets[c] (device arrays, n_new + 1
// offsets); new_ids[c] = c; kClausePad zero literals after the last one.
struct GatherArgs {
    const int32_t *lits;
    const int64_t *offsets;
    const uint32_t *src;
    const int64_t *new_offsets;
    uint32_t n_new;
    int64_t n_new_lits;
    int32_t *new_lits;     // room for n_new_lits + kClausePad
    uint32_t *new_ids;     // room for n_new
};
int gather_clauses(const GatherArgs &a, cudaStream_t stream, int sm_count);
// Packs report partitions (n_parts x cap records, counts[p] valid in
// partition p, device) into contiguous 12-byte {clause, word, mask} records,
// or, with cell_words > 0, 8-byte {clause * cell_words + word, mask} records.
int launch_pack_reports(const gss_report *parts, const uint32_t *counts, uint32_t n_parts, uint32_t cap,
                        uint32_t cell_words, uint32_t *packed, cudaStream_t stream, int sm_count);
// Synchronizes `stream`; returns the live clause and literal counts.
int compact_by_id(const CompactArgs &a, cudaStream_t stream, int sm_count, uint32_t *n_out, int64_t *lits_out);

// Launches the check kernel on `stream` (the counters must already be zero).
// Returns a GSS status.
int launch_check(const CheckArgs &a, cudaStream_t stream, int sm_count);
bool valid_variant(int lpc, int g);
int launch_check_tiled(const CheckArgs &a, cudaStream_t stream, int sm_count);
int launch_check_wide(const CheckArgs &a, int wpl, int occ, cudaStream_t stream, int sm_count);
// Pipelined wide kernel (occ: 4 blocks per SM register cap).
int launch_check_wide_pf(const CheckArgs &a, int wpl, int occ, cudaStream_t stream, int sm_count);
bool valid_wide_pf_variant(int wpl, int lpc, int g);
// Persistent wide kernel: arguments read from device memory (d_args, so that
// a captured graph serves every pass) or, when d_args is NULL, passed by
// value (h_args); tasks from the device counter `work` (zero it before each
// launch).
int launch_check_wide_persist(const CheckArgs *d_args, const CheckArgs &h_args, int wpl, int lpc, int g, uint32_t *work,
                              cudaStream_t stream, int sm_count);
bool valid_wide_persist_variant(int wpl, int lpc, int g);
bool valid_wide_variant(int wpl, int lpc, int g, int occ);
bool valid_tiled_variant(int lpc, int k);

// [n_vars][n_words] -> [n_blocks][n_vars][lpc], zero-padded words.
int launch_relayout(const uint2 *src, uint2 *dst, uint32_t n_vars, uint32_t n_words, uint32_t lpc,
                    uint32_t n_blocks, cudaStream_t stream, int sm_count);

}  // namespace gss
