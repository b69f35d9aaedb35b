// The clause sharer: host side of the GpuClauseSharer API over the check
// engine. Internal header (the C ABI is in include/gpusharesat.h).
#pragma once

#include <atomic>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_set>
#include <vector>

#include "activity.h"
#include "common.h"

namespace gss {

// Values as the reference's lbool: 0 true, 1 false, 2 undefined
// (gpuShareLib/SolverTypes.h:81-83).
constexpr uint8_t kTrue = 0, kFalse = 1, kUndef = 2;
constexpr int kSlots = 32;  // assignments per solver per pass (Assigs.cuh:37-39)

// Statistics, in the reference's order and with its names
// (gpuShareLib/GlobalStats.h:23-37, gpuShareLib/OneSolverStats.h:24-29).
enum GlobalStat {
    kGpuClauses, kGpuClauseLengthSum, kGpuClausesAdded, kGpuRuns, kClauseTestsOnGroups, kClauseTestsOnAssigs,
    kTotalAssigClauseTested, kGpuReduceDbs, kGpuReports, kTimeSpentTestingClauses, kTimeSpentFillingAssigs,
    kTimeSpentFillingReported, kTimeSpentReduceGpuDb, kGlobalStatCount
};
enum SolverStat {
    kVarUpdatesSentToGpu, kAssigsSentToGpu, kFailuresToFindAssig, kReportedClauses, kReportedClausesUnit,
    kReportedClausesBinary, kSolverStatCount
};
extern const char *const kGlobalStatNames[kGlobalStatCount];
extern const char *const kSolverStatNames[kSolverStatCount];

// A change of one variable for one solver in the current pass window: its
// value in each of the 32 slots (MultiLBool, gpuShareLib/BaseTypes.cuh:65-68).
struct VarUpdate {
    uint32_t var;
    uint32_t is_def;
    uint32_t is_true;
};

// Ids of the assignments one solver sent in one pass (AssigIdsPerSolver,
// gpuShareLib/BaseTypes.cuh:42-54).
struct AssigIds {
    int64_t start = 0;
    int count = 0;
};

// The 32-slot ring of one solver (OneSolverAssigs, gpuShareLib/Assigs.cu:143-300).
struct SolverAssigs {
    std::mutex lock;
    uint32_t not_completed = ~0u;
    int64_t current_id = 0;
    int64_t first_id_used = 0;
    std::vector<uint8_t> last_val;
    std::vector<VarUpdate> updates;
    std::vector<int32_t> update_pos;
    std::vector<int32_t> to_unset;  // literals unset while the ring was full
    void set_var_locked(uint32_t var, uint8_t val);
    bool available_locked() const { return current_id != first_id_used + kSlots; }
    int64_t done_locked();
};

// Clauses reported to one solver by one pass (ClauseBatch, gpuShareLib/Reported.cu:35-69).
struct ClauseBatch {
    std::vector<int32_t> lits;
    std::vector<std::pair<int64_t, int32_t>> clauses;  // (gpu clause id, first literal)
    size_t next = 0;
    AssigIds assig;
    uint32_t had_some = 0;
    int64_t assig_which_knows = 0;
    void clear() {
        lits.clear();
        clauses.clear();
        next = 0;
        had_some = 0;
    }
    bool pop(int32_t *&l, int &count, int64_t &id) {
        if (next >= clauses.size()) return false;
        const int32_t b = clauses[next].second;
        const int32_t e = next + 1 < clauses.size() ? clauses[next + 1].second : (int32_t) lits.size();
        l = lits.data() + b;
        count = e - b;
        id = clauses[next].first;
        next++;
        return true;
    }
};

// Per-solver queue of batches: [min, inter) consumed but kept until the
// solver's later assignments know about their clauses, [inter, visible)
// ready for the solver (ConcurrentQueue, gpuShareLib/ConcurrentQueue.h:115-196).
struct BatchQueue {
    std::mutex lock;
    std::deque<std::unique_ptr<ClauseBatch>> items;  // items[0] has index `min`
    std::vector<std::unique_ptr<ClauseBatch>> spare;
    int64_t min = 0, inter = 0, visible = 0;
    ClauseBatch *take_next();     // getIncrInter
    ClauseBatch *oldest();        // getMin
    void release_oldest();        // removeMin
    ClauseBatch *new_batch();     // getNew (not visible yet)
    void publish();               // addNew
};

struct SolverReported {
    std::unordered_set<int64_t> not_again;                 // clausesToNotImportAgain
    std::deque<std::pair<int64_t, int64_t>> dont_import;   // (gpu clause id, assignment id)
    ClauseBatch *current = nullptr;
    int64_t last_sent = 0;
    std::atomic<int64_t> last_all_reported{0};
    BatchQueue queue;
};

// A clause on the device; its activity is the entry of the same index in
// Sharer::act_ (both are kept in device order).
struct ClauseMeta {
    int64_t gpu_id;
    uint32_t lit_off;      // into the host literal arena
    uint32_t len;
    int32_t last_report;   // pass of its last report, -1 if never reported
};

struct Options {
    int block_count = -1, threads_per_block = -1, min_latency_us = -1, verbosity = 1;
    double activity_decay = -1;
    bool quick_prof = true;
    int init_report_count = -1, max_page_locked = -1;
};

class Sharer {
public:
    Sharer(const Options &o, std::function<void(const std::string &)> log);
    ~Sharer();
    int init(int device);

    int gpu_run();
    int reduce_db();
    int64_t added_clause_count() const { return stats_[kGpuClausesAdded]; }
    int64_t added_at_last_reduce() const { return added_at_last_reduce_; }
    bool ran_out_of_memory() const { return out_of_memory_; }
    int mem_info(size_t *free_b, size_t *total_b);
    int64_t global_stat(int s) const;
    int write_cnf(FILE *f);
    int set_var_count(int n);
    int64_t add_clause(int solver, const int *lits, int count);
    int set_solver_count(int n);
    bool try_set_values(int solver, const int *lits, int count);
    void unset_values(int solver, const int *lits, int count);
    int64_t try_send(int solver);
    bool pop_reported(int solver, int *&lits, int &count, int64_t &id);
    int64_t last_all_reported(int solver) const;
    void current_assignment(int solver, uint8_t *out);
    int64_t solver_stat(int solver, int s) const;
    int solver_count() const { return (int) solvers_.size(); }
    int max_clause_len() const { return max_len_; }
    void set_max_clause_len(int n) { max_len_ = n; }
    int set_variant(int kind, int lpc, int depth, int flags);
    void set_clause_budget(int64_t n) { budget_ = n; }
    // device order of appended batches and reduceDb survivors: variable
    // ranges of 2^r (-1: automatic, 0: length order), as gss_db_set_locality
    void set_locality(int r) { range_log2_ = r; }
    int64_t evicted() const { return evicted_; }
    int64_t device_compactions() const { return device_compactions_; }
    int64_t live_clauses() const { return (int64_t) meta_.size() - n_dead_; }

private:
    // One pass in flight or waiting for delivery. Two of them alternate, so
    // the host delivers pass N's reports while the GPU checks pass N+1.
    struct Pass {
        bool pending = false;    // launched, not collected
        bool collected = false;  // counts read and reports copying to the host, not delivered
        bool noted = false;      // its reports already marked on the clauses (last report, activity)
        std::vector<AssigIds> assig;
        uint32_t n_clauses = 0;
        int64_t n_updates = 0;
        int64_t assig_total = 0;
        int active_words = 0;
        int64_t n_reports = 0;
        int32_t number = 0;      // pass_no_ at its launch
        // device report queues and their counters, pinned host copies of the
        // counters (+ error flag), the start and last-slot masks and the reports
        DevBuf d_reports, d_counts;
        uint32_t cap_per_part = 0;
        PinnedBuf h_counts, h_start, h_last, h_reports;
        cudaEvent_t counted = nullptr;  // counts copied to h_counts
        cudaEvent_t copied = nullptr;   // reports copied to h_reports
    };

    int collect(Pass &p);
    int note_reports(Pass &p);
    int deliver(Pass &p);
    int finish_pending();
    int reduce_now(bool on_device);
    int rebuild_on_device(const std::vector<uint32_t> &src);
    int recover_from_oom();
    int launch_pass();
    int run_check(Pass &p);
    int ensure_state();
    int append_clauses(std::vector<int64_t> &ids, std::vector<int32_t> &lits, std::vector<uint32_t> &lens);
    void reserve_for_budget(size_t n_new, size_t n_new_lits);
    int upload_db();
    void evict(int64_t n);
    int compact(bool upload = true, std::vector<uint32_t> *old_index = nullptr);
    int compact_device();
    int sync_alive();
    void mark_alive(size_t lo_word, size_t hi_word);
    void unset_pending_locked(int solver);
    void log(int level, const std::string &msg) const;

    Options opt_;
    std::function<void(const std::string &)> log_fn_;
    int device_ = 0, sm_count_ = 0;
    cudaStream_t stream_ = nullptr;
    int max_len_ = 100;  // MAX_CL_SIZE, gpuShareLib/BaseTypes.cuh:28
    int range_log2_ = -1;

    // statistics
    std::vector<std::atomic<int64_t>> stats_;
    std::vector<std::vector<std::atomic<int64_t>>> solver_stats_;

    // clause staging (addClause, any thread)
    std::mutex stage_lock_;
    int64_t next_clause_id_ = 0;
    std::vector<int64_t> st_ids_;
    std::vector<int32_t> st_lits_;
    std::vector<uint32_t> st_lens_;

    // clauses on the device, in device order
    std::vector<int32_t> h_lits_;
    std::vector<ClauseMeta> meta_;
    std::unique_ptr<ClauseActivity> act_;
    int64_t added_at_last_reduce_ = 0;
    bool out_of_memory_ = false;
    // Device database: CSR of the clauses in device order, and d_orig_, the
    // index in meta_ of each (the id reports carry). Device order is meta_
    // order with evicted clauses compacted away.
    DevBuf d_lits_, d_offsets_, d_orig_;
    DevBuf d_lits2_, d_offsets2_, d_orig2_, d_compact_;  // compaction targets, swapped in
    std::vector<uint32_t> h_dev_meta_;  // host copy of d_orig_: meta_ index of each device position
    int64_t dev_lits_ = 0;
    uint32_t dev_clauses_ = 0;
    int64_t max_var_ = -1;
    // HBM budget: the oldest clauses not reported in the last kRecentPasses
    // passes are evicted. An evicted clause keeps its meta_ entry (a
    // tombstone: its bit in h_alive_ is clear) until a reduceDb or until
    // tombstones are half of meta_; on the device it is skipped through the
    // bitmap and dropped by compact_device() once evicted clauses are a fifth
    // of the device database.
    int64_t budget_ = 0;
    int64_t reserved_for_ = 0;  // the budget whose room reserve_for_budget set aside
    int64_t evicted_ = 0;
    int64_t n_dead_ = 0;     // tombstones in meta_
    int64_t dev_dead_ = 0;   // evicted clauses still in the device arrays
    size_t evict_cursor_ = 0;
    int32_t pass_no_ = 0;    // passes launched so far (the number of the next one)
    std::vector<uint32_t> h_alive_;  // bit per meta_ index
    DevBuf d_alive_;
    PinnedBuf h_alive_stage_;        // staging of alive-bit uploads
    cudaEvent_t alive_staged_ = nullptr;
    bool alive_synced_ = false;      // d_alive_ holds h_alive_ except [alive_lo_, alive_hi_)
    size_t alive_lo_ = SIZE_MAX, alive_hi_ = 0;
    int64_t device_compactions_ = 0;

    // assignments
    int n_vars_ = 0;
    std::vector<std::unique_ptr<SolverAssigs>> solvers_;
    std::vector<std::unique_ptr<SolverReported>> reported_;
    DevBuf d_state_, d_start_, d_sow_, d_updates_, d_last_mask_;
    PinnedBuf h_updates_;
    PinnedBuf h_append_;             // staging of appended clauses (literals, offsets, ids)
    cudaEvent_t append_staged_ = nullptr;
    int dev_vars_ = 0, dev_words_ = 0;
    int kind_ = GSS_KERNEL_AUTO, lpc_req_ = 0, depth_req_ = 2, flags_ = 0;
    int eff_kind_ = GSS_KERNEL_DIRECT, eff_lpc_ = 1, eff_depth_ = 2, bw_ = 1, n_blocks_ = 0;

    // reports: two passes, alternating (the one launched last is pass_[cur_])
    DevBuf d_err_, d_work_;  // kernel error flag, persistent kernel's task counter
    uint32_t n_parts_ = 16;
    uint32_t report_cap_ = 0;  // records per partition that earlier passes needed
    Pass pass_[2];
    int cur_ = 0;
};

}  // namespace gss
