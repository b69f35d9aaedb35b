// The engine's state (internal: shared by the engine's C ABI and the
// learned scan order; not part of the public headers).
#pragma once

#include <stdint.h>

#include <utility>
#include <vector>

#include "common.h"

namespace gss {
struct OrderState;
}
using gss::DevBuf;
using gss::PinnedBuf;

struct gss_engine {
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int64_t launches = 0;

    // clause database: CSR, clauses sorted by length (stable), with the
    // original index of each sorted clause
    DevBuf lits, offsets, orig;
    int64_t n_clauses = 0, n_lits = 0, max_var = -1;
    // tiles of the tiled kernel (first clause / first literal of each tile)
    DevBuf tile_clause, tile_lit;
    uint32_t n_tiles = 0;
    bool tiles_stale = true;
    // host mirror of the database, in device order, for appends, deletes and
    // compaction; alive bits (1 per device clause) mark deleted clauses
    std::vector<int32_t> h_lits;
    std::vector<int64_t> h_off;
    std::vector<uint32_t> h_ids;
    std::vector<uint32_t> index_of;  // clause id -> device index (0xFFFFFFFF: none)
    std::vector<uint32_t> h_alive;
    DevBuf alive;
    bool alive_dirty = false;
    int64_t n_dead = 0;
    uint32_t next_id = 0;
    // variable ranges of the database order (gss_db_set_locality): log2 of
    // the variables per range, -1 automatic, 0 length order only
    int range_log2 = -1;

    // kernel variant: kind (GSS_KERNEL_*), lanes (words) per clause (0 = pick
    // from the word count), loads in flight / clause slots, cache hints
    int kind = GSS_KERNEL_AUTO, lpc = 0, g = 2, flags = 0;
    DevBuf err;

    // assignment state, block-major [n_blocks][n_vars][state_bw words]
    DevBuf state, state_raw, start, solver_of_word;
    int64_t n_vars = 0;
    int n_words = 0;
    int n_blocks = 0;
    // effective variant the state was laid out for (resolved from the
    // requested one and the word count by gss_state_set)
    int state_kind = GSS_KERNEL_DIRECT;
    int state_lpc = 0;  // lanes per clause
    int state_g = 2;
    int state_bw = 0;   // words per slot block

    // report queues: n_parts partitions of cap_per_part records
    DevBuf reports, counts;
    uint32_t n_parts = 16;
    uint32_t cap_per_part = 0;
    int64_t requested_cap = 0;
    PinnedBuf h_counts;
    bool pass_pending = false;

    // pipelined passes through host buffers (gss_check_passes_host): second
    // state and report buffers, copy streams and events
    // slots 1 and 2 of the three-slot pipeline (slot 0 is the engine's own)
    DevBuf state2, state_raw2, reports2, counts2;
    DevBuf state3, state_raw3, reports3, counts3;
    DevBuf packed[3];  // 12-byte records of gss_check_passes_host_packed
    PinnedBuf h_counts2, h_counts3;
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t ev_h2d[3] = {}, ev_kernel[3] = {}, ev_d2h[3] = {};

    // persistent kernel: arguments in device memory, task counter; optional
    // CUDA graph of a pass (memsets, kernel, count readback), recaptured when
    // a buffer it names changes
    DevBuf d_args, work;
    // length plan of the bucketed kernel (gss_engine_set_length_plan): class
    // bounds and lane layouts; the position ranges are rebuilt on the device
    // when plan_built differs from db_version
    std::vector<int32_t> plan_max_len, plan_layout;
    DevBuf d_plan;
    uint64_t db_version = 0;  // counts every change of the database's positions
    uint64_t plan_built = ~0ull;
    uint32_t plan_ranges = 0;
    bool use_graph = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<uintptr_t> graph_key;
    int64_t graph_captures = 0;

    // optional CUDA-event timing of each check kernel (on the launch stream)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending;

    // learned scan order (NULL: plain length-sorted scan); db_epoch counts
    // gss_db_set calls, so the order knows when clause ids start over;
    gss::OrderState *order = nullptr;
    uint64_t db_epoch = 0;
    uint64_t layout_epoch = 0;  // counts gss_db_set and gss_db_compact (positions change)
};


namespace gss {
// Learned scan order hooks, called by the engine's pass (order.cu).
// Before the scan: the scan permutation of this pass (computed while the
// previous pass ran, or now on the engine's stream). It covers positions
// [0, *covered); *head = scan positions in the head. Clauses appended after
// it was computed (positions from *covered on) are scanned after it.
int order_prepare(gss_engine *eng, const uint32_t **perm, uint32_t *head, uint32_t *covered);
// Waits until no scoring for a coming pass reads the engine's buffers; every
// call that frees, moves or rewrites them calls this first.
void order_quiesce(gss_engine *eng);
// After the head launch: records the head's report counts for early delivery.
int order_after_head(gss_engine *eng, const DevBuf &counts);
// After the tail launch: folds the pass's reports into the report history.
int order_after_pass(gss_engine *eng, const DevBuf &reports, const DevBuf &counts);
bool order_active(const gss_engine *eng);
void order_destroy(gss_engine *eng);
}  // namespace gss
