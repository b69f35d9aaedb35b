// The clause sharer: the GpuClauseSharer API (gpuShareLib/GpuClauseSharer.h:74-163)
// implemented over the check engine.
//
// Host side, restating the reference's semantics:
//  * per-solver 32-slot assignment ring with snapshot-at-send semantics
//    (OneSolverAssigs::setVarLocked / copyUpdatesLocked, gpuShareLib/Assigs.cu:163-300;
//    deferred unsets, gpuShareLib/GpuClauseSharerImpl.cu:130-191);
//  * clause staging and activity (HostClauses::addClause, getUpdatesForDevice,
//    bump/decay/rescale and reduceDb, gpuShareLib/Clauses.cu:199-525);
//  * report delivery with dedup and self-export filtering (Reported::fill /
//    popReportedClause, gpuShareLib/Reported.cu:97-204).
// Device side, the GB300 design: the clause database and every solver's 32
// slots stay resident in HBM ([block][var][words] bit planes, one 32-slot word
// per solver); each pass uploads only the changed variables, scatters them,
// runs the check kernel, and broadcasts the last slot into all 32 after it
// (dUpdateAssigs / dSetAllAssigsToLast, gpuShareLib/Assigs.cu:100-141, without
// the reference's cross-solver aggregate, which the exact kernel does not need).
//
// Pipeline: gpuRun() first collects the pass launched by the previous call,
// then cuts and launches a new one, so the results of pass N are delivered at
// call N+1, as in GpuRunner::wholeRun (gpuShareLib/GpuRunner.cu:211-261).
// Unlike the reference's reporter (Reporter.cuh:41-49), no report is ever
// dropped: if the queues overflow, the collected pass is checked again with
// larger queues before its variables are broadcast to their last slot.
#include <math.h>
#include <stdarg.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <limits>
#include <sstream>
#include <thread>

#include "sharer.h"

namespace gss {

const char *const kGlobalStatNames[kGlobalStatCount] = {
    "gpuClauses", "gpuClauseLengthSum", "gpuClausesAdded", "gpuRuns", "clauseTestsOnGroups", "clauseTestsOnAssigs",
    "totalAssigClauseTested", "gpuReduceDbs", "gpuReports", "timeSpentTestingClauses", "timeSpentFillingAssigs",
    "timeSpentFillingReported", "timeSpentReduceGpuDb"};
const char *const kSolverStatNames[kSolverStatCount] = {"varUpdatesSentToGpu", "assigsSentToGpu",
                                                        "failuresToFindAssig", "reportedClauses",
                                                        "reportedClausesUnit", "reportedClausesBinary"};

namespace {

int64_t now_us() {
    return std::chrono::duration_cast<std::chrono::microseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct DevUpdate {
    uint32_t var;
    uint32_t word;
    uint32_t is_def;
    uint32_t is_true;
};

// state[(word / bw) * n_vars + var][word % bw] = update
__global__ void scatter_updates_kernel(const DevUpdate *__restrict__ u, uint32_t n, uint2 *__restrict__ state,
                                       uint32_t n_vars, uint32_t bw) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DevUpdate x = u[i];
        const size_t idx = ((size_t) (x.word / bw) * n_vars + x.var) * bw + x.word % bw;
        state[idx] = make_uint2(x.is_def, x.is_true);
    }
}

// After the check: every slot of an updated variable takes the value of the
// solver's last slot (dSetAllAssigsToLast, gpuShareLib/Assigs.cu:118-141).
__global__ void set_to_last_kernel(const DevUpdate *__restrict__ u, uint32_t n, const uint32_t *__restrict__ last,
                                   uint2 *__restrict__ state, uint32_t n_vars, uint32_t bw) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DevUpdate x = u[i];
        const uint32_t m = last[x.word];
        const size_t idx = ((size_t) (x.word / bw) * n_vars + x.var) * bw + x.word % bw;
        state[idx] = make_uint2((x.is_def & m) ? ~0u : 0u, (x.is_true & m) ? ~0u : 0u);
    }
}

// Copies words [0, n_words) of every variable < n_vars from one block-major
// layout to another (solver or variable count changes).
__global__ void copy_layout_kernel(const uint2 *__restrict__ src, uint32_t src_vars, uint32_t src_bw,
                                   uint2 *__restrict__ dst, uint32_t dst_vars, uint32_t dst_bw, uint32_t n_vars,
                                   uint32_t n_words) {
    const uint64_t total = (uint64_t) n_vars * n_words;
    for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t) gridDim.x * blockDim.x) {
        const uint32_t v = (uint32_t) (i / n_words), w = (uint32_t) (i % n_words);
        dst[((size_t) (w / dst_bw) * dst_vars + v) * dst_bw + w % dst_bw] =
            src[((size_t) (w / src_bw) * src_vars + v) * src_bw + w % src_bw];
    }
}

unsigned grid_for(uint64_t n, int sm_count) {
    uint64_t b = (n + 255) / 256;
    if (b > (uint64_t) sm_count * 8) b = (uint64_t) sm_count * 8;
    return (unsigned) std::max<uint64_t>(b, 1);
}

}  // namespace

// ---- one solver's ring ----

void SolverAssigs::set_var_locked(uint32_t var, uint8_t val) {
    // gpuShareLib/Assigs.cu:163-185: slots not completed yet take the new
    // value; completed slots keep the value the variable had when they were
    // sent, which is last_val while the variable has no update in this window.
    const uint32_t set_m = val != kUndef ? ~0u : 0u;
    const uint32_t true_m = val == kTrue ? ~0u : 0u;
    const int32_t p = update_pos[var];
    if (p < 0 || (size_t) p >= updates.size() || updates[p].var != var) {
        VarUpdate u;
        u.var = var;
        const uint32_t old_set = last_val[var] != kUndef ? ~0u : 0u;
        const uint32_t old_true = last_val[var] == kTrue ? ~0u : 0u;
        u.is_def = (not_completed & set_m) | (~not_completed & old_set);
        u.is_true = (not_completed & true_m) | (~not_completed & old_true);
        update_pos[var] = (int32_t) updates.size();
        updates.push_back(u);
    } else {
        VarUpdate &u = updates[p];
        u.is_def = (u.is_def & ~not_completed) | (not_completed & set_m);
        u.is_true = (u.is_true & ~not_completed) | (not_completed & true_m);
    }
    last_val[var] = val;
}

int64_t SolverAssigs::done_locked() {
    // gpuShareLib/Assigs.cu:194-201
    const int pos = (int) (current_id % kSlots);
    not_completed &= ~(1u << pos);
    return current_id++;
}

// ---- batch queues ----

ClauseBatch *BatchQueue::take_next() {
    std::lock_guard<std::mutex> g(lock);
    if (inter == visible) return nullptr;
    ClauseBatch *b = items[(size_t) (inter - min)].get();
    inter++;
    return b;
}

ClauseBatch *BatchQueue::oldest() {
    std::lock_guard<std::mutex> g(lock);
    if (inter == min) return nullptr;
    return items.front().get();
}

void BatchQueue::release_oldest() {
    std::lock_guard<std::mutex> g(lock);
    spare.push_back(std::move(items.front()));
    items.pop_front();
    min++;
}

ClauseBatch *BatchQueue::new_batch() {
    std::lock_guard<std::mutex> g(lock);
    std::unique_ptr<ClauseBatch> b;
    if (!spare.empty()) {
        b = std::move(spare.back());
        spare.pop_back();
    } else {
        b.reset(new ClauseBatch());
    }
    b->clear();
    items.push_back(std::move(b));
    return items.back().get();
}

void BatchQueue::publish() {
    std::lock_guard<std::mutex> g(lock);
    visible++;
}

// ---- sharer ----

Sharer::Sharer(const Options &o, std::function<void(const std::string &)> log)
    : opt_(o), log_fn_(std::move(log)), stats_(kGlobalStatCount) {
    for (auto &s : stats_) s = 0;
}

Sharer::~Sharer() {
    if (stream_) {
        cudaSetDevice(device_);
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
    for (Pass &p : pass_) {
        if (p.counted) cudaEventDestroy(p.counted);
        if (p.copied) cudaEventDestroy(p.copied);
    }
    if (alive_staged_) cudaEventDestroy(alive_staged_);
    if (append_staged_) cudaEventDestroy(append_staged_);
}

void Sharer::log(int level, const std::string &msg) const {
    if (opt_.verbosity >= level && log_fn_) log_fn_(msg);
}

int Sharer::init(int device) {
    // Option defaults and checks of GpuClauseSharerImpl's constructor
    // (gpuShareLib/GpuClauseSharerImpl.cu:40-65).
    if (opt_.min_latency_us < 0) opt_.min_latency_us = 50;
    if (opt_.activity_decay < 0) opt_.activity_decay = 0.99999;
    if (opt_.activity_decay >= 1) return set_error(GSS_ERR_INVALID, "Clause activity decay must be strictly smaller than 1");
    if (opt_.init_report_count < 0) opt_.init_report_count = 10;
    if (opt_.init_report_count == 0) return set_error(GSS_ERR_INVALID, "initReportCountPerCategory must not be 0");
    if (opt_.threads_per_block == 0) return set_error(GSS_ERR_INVALID, "gpuThreadsPerBlockGuideline must not be 0");
    if (opt_.block_count == 0) return set_error(GSS_ERR_INVALID, "gpuBlockCountGuideline must not be 0");
    act_.reset(new ClauseActivity((float) opt_.activity_decay));
    if (device < 0) GSS_CUDA_TRY(cudaGetDevice(&device));
    device_ = device;
    GSS_CUDA_TRY(cudaSetDevice(device_));
    GSS_CUDA_TRY(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_));
    if (opt_.block_count < 0) {
        opt_.block_count = 2 * sm_count_;
        std::ostringstream os;
        os << "c Setting block count guideline to " << opt_.block_count << " (twice the number of multiprocessors)\n";
        log(1, os.str());
    }
    if (opt_.threads_per_block < 0) opt_.threads_per_block = 512;
    GSS_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    for (Pass &p : pass_) {
        GSS_CUDA_TRY(cudaEventCreateWithFlags(&p.counted, cudaEventDisableTiming));
        GSS_CUDA_TRY(cudaEventCreateWithFlags(&p.copied, cudaEventDisableTiming));
        GSS_TRY(p.d_counts.reserve(sizeof(uint32_t) * n_parts_));
        GSS_TRY(p.h_counts.reserve(sizeof(uint32_t) * (n_parts_ + 1)));
    }
    GSS_CUDA_TRY(cudaEventCreateWithFlags(&alive_staged_, cudaEventDisableTiming));
    GSS_CUDA_TRY(cudaEventCreateWithFlags(&append_staged_, cudaEventDisableTiming));
    GSS_TRY(d_err_.reserve(sizeof(uint32_t)));
    // one solver until told otherwise (HostAssigs constructor, Assigs.cu:311)
    return set_solver_count(1);
}

int Sharer::mem_info(size_t *free_b, size_t *total_b) {
    GSS_CUDA_TRY(cudaSetDevice(device_));
    GSS_CUDA_TRY(cudaMemGetInfo(free_b, total_b));
    return GSS_OK;
}

int64_t Sharer::global_stat(int s) const {
    if (s < 0 || s >= kGlobalStatCount) return 0;
    return stats_[s];
}

int64_t Sharer::solver_stat(int solver, int s) const {
    if (solver < 0 || solver >= (int) solver_stats_.size() || s < 0 || s >= kSolverStatCount) return 0;
    return solver_stats_[solver][s];
}

int Sharer::set_var_count(int n) {
    if (n < 0) return set_error(GSS_ERR_INVALID, "negative variable count");
    for (auto &sa : solvers_) {
        std::lock_guard<std::mutex> g(sa->lock);
        if ((int) sa->last_val.size() < n) {
            sa->last_val.resize(n, kUndef);
            sa->update_pos.resize(n, -1);
        }
    }
    if (n > n_vars_) n_vars_ = n;
    return GSS_OK;
}

int Sharer::set_solver_count(int n) {
    if (n < 1) return set_error(GSS_ERR_INVALID, "solver count must be at least 1");
    const int old = (int) solvers_.size();
    for (int s = old; s < n; s++) {
        solvers_.emplace_back(new SolverAssigs());
        solvers_.back()->last_val.assign(n_vars_, kUndef);
        solvers_.back()->update_pos.assign(n_vars_, -1);
        reported_.emplace_back(new SolverReported());
        solver_stats_.emplace_back(kSolverStatCount);
        for (auto &x : solver_stats_.back()) x = 0;
    }
    return GSS_OK;
}

int Sharer::set_variant(int kind, int lpc, int depth, int flags) {
    if (kind != GSS_KERNEL_AUTO && kind != GSS_KERNEL_DIRECT && kind != GSS_KERNEL_WIDE4 && kind != GSS_KERNEL_WIDE2)
        return set_error(GSS_ERR_INVALID, "the sharer runs the direct or wide kernels");
    if (kind == GSS_KERNEL_DIRECT && lpc != 0 && !valid_variant(lpc, depth))
        return set_error(GSS_ERR_INVALID, "no direct kernel variant for %d lanes per clause, depth %d", lpc, depth);
    if ((kind == GSS_KERNEL_WIDE4 || kind == GSS_KERNEL_WIDE2) &&
        !valid_wide_variant(kind == GSS_KERNEL_WIDE4 ? 4 : 2, lpc ? lpc : (kind == GSS_KERNEL_WIDE4 ? 8 : 16), depth,
                            (flags & GSS_VARIANT_OCCUPANCY) ? 1 : 0))
        return set_error(GSS_ERR_INVALID, "no wide kernel variant for %d lanes per clause, depth %d", lpc, depth);
    if ((kind == GSS_KERNEL_WIDE4 || kind == GSS_KERNEL_WIDE2) && (flags & GSS_VARIANT_PERSISTENT) &&
        !valid_wide_persist_variant(kind == GSS_KERNEL_WIDE4 ? 4 : 2, lpc ? lpc : (kind == GSS_KERNEL_WIDE4 ? 8 : 16),
                                    depth))
        return set_error(GSS_ERR_INVALID, "no persistent wide kernel variant for %d lanes per clause, depth %d", lpc,
                         depth);
    kind_ = kind;
    lpc_req_ = lpc;
    depth_req_ = depth;
    flags_ = flags;
    dev_words_ = -1;  // force a re-layout at the next pass
    return GSS_OK;
}

// ---- clause export ----

int64_t Sharer::add_clause(int solver, const int *lits, int count) {
    // HostClauses::addClause (gpuShareLib/Clauses.cu:349-356): too long -> -1.
    // An empty clause is refused too (the reference asserts on it later).
    if (count > max_len_ || count < 1 || (count > 0 && !lits)) return -1;
    if (solver >= (int) solvers_.size()) return -1;
    for (int i = 0; i < count; i++)
        if (lits[i] < 0) return -1;
    int64_t id;
    {
        std::lock_guard<std::mutex> g(stage_lock_);
        id = next_clause_id_++;
        st_ids_.push_back(id);
        st_lits_.insert(st_lits_.end(), lits, lits + count);
        st_lens_.push_back((uint32_t) count);
    }
    if (solver >= 0) {
        // Reported::clauseWasAdded (gpuShareLib/Reported.cu:97-103)
        SolverReported &r = *reported_[solver];
        r.not_again.insert(id);
        r.dont_import.emplace_back(id, r.last_sent + 1);
    }
    return id;
}

// ---- assignments ----

void Sharer::unset_pending_locked(int solver) {
    SolverAssigs &sa = *solvers_[solver];
    for (int32_t l : sa.to_unset) sa.set_var_locked((uint32_t) l >> 1, kUndef);
    solver_stats_[solver][kVarUpdatesSentToGpu] += (int64_t) sa.to_unset.size();
    sa.to_unset.clear();
}

bool Sharer::try_set_values(int solver, const int *lits, int count) {
    // GpuClauseSharerImpl::trySetSolverValues (GpuClauseSharerImpl.cu:130-147)
    if (solver < 0 || solver >= (int) solvers_.size()) return false;
    SolverAssigs &sa = *solvers_[solver];
    std::lock_guard<std::mutex> g(sa.lock);
    if (!sa.available_locked()) {
        solver_stats_[solver][kFailuresToFindAssig]++;
        return false;
    }
    unset_pending_locked(solver);
    for (int i = 0; i < count; i++) {
        const uint32_t v = (uint32_t) lits[i] >> 1;
        if (v >= sa.last_val.size()) continue;  // beyond setVarCount: ignored
        sa.set_var_locked(v, (lits[i] & 1) ? kFalse : kTrue);
    }
    solver_stats_[solver][kVarUpdatesSentToGpu] += count;
    return true;
}

void Sharer::unset_values(int solver, const int *lits, int count) {
    // GpuClauseSharerImpl::unsetSolverValues (GpuClauseSharerImpl.cu:159-176)
    if (solver < 0 || solver >= (int) solvers_.size()) return;
    SolverAssigs &sa = *solvers_[solver];
    std::lock_guard<std::mutex> g(sa.lock);
    if (sa.available_locked()) {
        unset_pending_locked(solver);
        for (int i = 0; i < count; i++) {
            const uint32_t v = (uint32_t) lits[i] >> 1;
            if (v < sa.last_val.size()) sa.set_var_locked(v, kUndef);
        }
        solver_stats_[solver][kVarUpdatesSentToGpu] += count;
    } else {
        sa.to_unset.insert(sa.to_unset.end(), lits, lits + count);
    }
}

int64_t Sharer::try_send(int solver) {
    // GpuClauseSharerImpl::trySendAssignment (GpuClauseSharerImpl.cu:178-191)
    if (solver < 0 || solver >= (int) solvers_.size()) return -1;
    SolverAssigs &sa = *solvers_[solver];
    std::lock_guard<std::mutex> g(sa.lock);
    if (!sa.available_locked()) {
        solver_stats_[solver][kFailuresToFindAssig]++;
        return -1;
    }
    const int64_t id = sa.done_locked();
    solver_stats_[solver][kAssigsSentToGpu]++;
    reported_[solver]->last_sent = id;
    return id;
}

void Sharer::current_assignment(int solver, uint8_t *out) {
    // GpuClauseSharerImpl::getCurrentAssignment (GpuClauseSharerImpl.cu:238-244)
    if (solver < 0 || solver >= (int) solvers_.size() || !out) return;
    SolverAssigs &sa = *solvers_[solver];
    std::lock_guard<std::mutex> g(sa.lock);
    memcpy(out, sa.last_val.data(), sa.last_val.size());
    for (int32_t l : sa.to_unset) {
        const uint32_t v = (uint32_t) l >> 1;
        if (v < sa.last_val.size()) out[v] = kUndef;
    }
}

int64_t Sharer::last_all_reported(int solver) const {
    if (solver < 0 || solver >= (int) reported_.size()) return 0;
    return reported_[solver]->last_all_reported;
}

// ---- import ----

bool Sharer::pop_reported(int solver, int *&lits, int &count, int64_t &id) {
    // Reported::popReportedClause (gpuShareLib/Reported.cu:105-158)
    if (solver < 0 || solver >= (int) reported_.size()) return false;
    SolverReported &r = *reported_[solver];
    while (true) {
        if (!r.current) r.current = r.queue.take_next();
        if (!r.current) return false;
        int32_t *l;
        int c;
        int64_t cid;
        while (r.current->pop(l, c, cid)) {
            // A clause may trigger for several assignments that did not know
            // about it yet: import it once.
            if (r.not_again.insert(cid).second) {
                solver_stats_[solver][kReportedClauses]++;
                if (c == 1) solver_stats_[solver][kReportedClausesUnit]++;
                if (c == 2) solver_stats_[solver][kReportedClausesBinary]++;
                lits = l;
                count = c;
                id = cid;
                return true;
            }
        }
        r.current->assig_which_knows = r.last_sent + 1;
        const int64_t seen_until = r.current->assig.start + r.current->assig.count;
        // Batches whose clauses every later assignment knows about: those
        // clauses will not trigger again (unless deleted by the solver).
        while (true) {
            ClauseBatch *old = r.queue.oldest();
            if (!old || old->assig_which_knows > seen_until) break;
            for (auto &cl : old->clauses) r.not_again.erase(cl.first);
            r.queue.release_oldest();
        }
        while (!r.dont_import.empty() && r.dont_import.front().second < seen_until) {
            r.not_again.erase(r.dont_import.front().first);
            r.dont_import.pop_front();
        }
        r.last_all_reported = seen_until;
        r.current = nullptr;
    }
}

// ---- device ----

int Sharer::ensure_state() {
    const int n_words = (int) solvers_.size();
    // Variables used by clauses but never declared are undefined for every
    // solver: the device state covers them too.
    const int need_vars = (int) std::max<int64_t>(n_vars_, max_var_ + 1);
    // resolve the kernel variant for this word count (as gss_state_set)
    int kind = kind_, lpc = lpc_req_, depth = depth_req_;
    if (kind == GSS_KERNEL_AUTO) {
        depth = 2;
        if (n_words >= 8) {
            kind = GSS_KERNEL_WIDE4;
            lpc = n_words >= 32 ? 8 : n_words >= 16 ? 4 : 2;
        } else {
            kind = GSS_KERNEL_DIRECT;
            lpc = 1;
            while (lpc < n_words) lpc *= 2;
            if (lpc == 1) depth = 1;
        }
    }
    const int wpl = kind == GSS_KERNEL_WIDE4 ? 4 : kind == GSS_KERNEL_WIDE2 ? 2 : 1;
    if (lpc == 0) {
        lpc = 1;
        if (wpl == 1)
            while (lpc < n_words && lpc < 32) lpc *= 2;
        else
            lpc = 32 / wpl;
    }
    const int bw = lpc * wpl;
    const int n_blocks = (n_words + bw - 1) / bw;
    if (dev_vars_ == need_vars && dev_words_ == n_words && bw == bw_ && d_state_.ptr) {
        eff_kind_ = kind;
        eff_lpc_ = lpc;
        eff_depth_ = depth;
        return GSS_OK;
    }
    const size_t bytes = std::max<size_t>((size_t) n_blocks * std::max(need_vars, 1) * bw * sizeof(uint2), 8);
    DevBuf fresh;
    GSS_TRY(fresh.reserve(bytes));
    GSS_CUDA_TRY(cudaMemsetAsync(fresh.ptr, 0, bytes, stream_));
    if (d_state_.ptr && dev_vars_ > 0 && dev_words_ > 0) {
        const uint32_t nv = (uint32_t) std::min(dev_vars_, need_vars);
        const uint32_t nw = (uint32_t) std::min(dev_words_, n_words);
        copy_layout_kernel<<<grid_for((uint64_t) nv * nw, sm_count_), 256, 0, stream_>>>(
            (const uint2 *) d_state_.ptr, (uint32_t) dev_vars_, (uint32_t) bw_, (uint2 *) fresh.ptr,
            (uint32_t) need_vars, (uint32_t) bw, nv, nw);
        GSS_CUDA_TRY(cudaGetLastError());
    }
    GSS_CUDA_TRY(cudaStreamSynchronize(stream_));
    std::swap(d_state_.ptr, fresh.ptr);
    std::swap(d_state_.bytes, fresh.bytes);
    dev_vars_ = need_vars;
    dev_words_ = n_words;
    bw_ = bw;
    n_blocks_ = n_blocks;
    eff_kind_ = kind;
    eff_lpc_ = lpc;
    eff_depth_ = depth;
    GSS_TRY(d_start_.reserve(sizeof(uint32_t) * n_blocks * bw));
    GSS_TRY(d_sow_.reserve(sizeof(int32_t) * n_blocks * bw));
    GSS_TRY(d_last_mask_.reserve(sizeof(uint32_t) * n_blocks * bw));
    std::vector<int32_t> sow(n_blocks * bw);
    for (int w = 0; w < n_blocks * bw; w++) sow[w] = w < n_words ? w : 0;
    GSS_CUDA_TRY(cudaMemcpy(d_sow_.ptr, sow.data(), sow.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return GSS_OK;
}

int Sharer::upload_db() {
    // whole database (after reduceDb or a host compaction): meta_ order
    const uint32_t n = (uint32_t) meta_.size();
    std::vector<int64_t> offsets(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + meta_[i].len;
    std::vector<int32_t> lits(offsets[n] + kClausePad, 0);
    for (uint32_t i = 0; i < n; i++)
        memcpy(&lits[offsets[i]], &h_lits_[meta_[i].lit_off], meta_[i].len * sizeof(int32_t));
    // compact the host arena to the device order
    h_lits_.assign(lits.begin(), lits.begin() + offsets[n]);
    for (uint32_t i = 0; i < n; i++) meta_[i].lit_off = (uint32_t) offsets[i];
    std::vector<uint32_t> orig(std::max<uint32_t>(n, 1));
    for (uint32_t i = 0; i < n; i++) orig[i] = i;
    GSS_TRY(d_lits_.reserve(lits.size() * sizeof(int32_t)));
    GSS_TRY(d_offsets_.reserve((n + 1) * sizeof(int64_t)));
    GSS_TRY(d_orig_.reserve(orig.size() * sizeof(uint32_t)));
    GSS_CUDA_TRY(cudaMemcpyAsync(d_lits_.ptr, lits.data(), lits.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                 stream_));
    GSS_CUDA_TRY(cudaMemcpyAsync(d_offsets_.ptr, offsets.data(), (n + 1) * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, stream_));
    GSS_CUDA_TRY(cudaMemcpyAsync(d_orig_.ptr, orig.data(), orig.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 stream_));
    GSS_CUDA_TRY(cudaStreamSynchronize(stream_));
    dev_clauses_ = n;
    dev_lits_ = offsets[n];
    h_dev_meta_.resize(n);
    for (uint32_t i = 0; i < n; i++) h_dev_meta_[i] = i;
    h_alive_.assign((n + 31) / 32, ~0u);
    n_dead_ = 0;
    dev_dead_ = 0;
    evict_cursor_ = 0;
    alive_synced_ = false;
    alive_lo_ = SIZE_MAX;
    alive_hi_ = 0;
    return GSS_OK;
}

void Sharer::mark_alive(size_t lo_word, size_t hi_word) {
    alive_lo_ = std::min(alive_lo_, lo_word);
    alive_hi_ = std::max(alive_hi_, hi_word);
}

int Sharer::sync_alive() {
    // Brings d_alive_ up to h_alive_: all of it the first time, then the
    // words changed since (evictions take the oldest clauses, appends add at
    // the end, so the range stays short).
    const size_t words = std::max<size_t>(h_alive_.size(), 1);
    if (!alive_synced_) {
        alive_lo_ = 0;
        alive_hi_ = h_alive_.size();
    }
    if (d_alive_.bytes < words * sizeof(uint32_t)) {
        GSS_TRY(d_alive_.grow_keep(words * sizeof(uint32_t), stream_,
                                   alive_synced_ ? std::min(d_alive_.bytes, words * sizeof(uint32_t)) : 0));
    }
    alive_hi_ = std::min(alive_hi_, h_alive_.size());
    if (alive_lo_ < alive_hi_) {
        // through pinned staging: a copy from pageable memory would wait for
        // the whole stream (the pass in flight) first
        const size_t bytes = (alive_hi_ - alive_lo_) * sizeof(uint32_t);
        GSS_CUDA_TRY(cudaEventSynchronize(alive_staged_));  // the previous upload has left the stage
        GSS_TRY(h_alive_stage_.reserve(bytes));
        memcpy(h_alive_stage_.ptr, h_alive_.data() + alive_lo_, bytes);
        GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) d_alive_.ptr + alive_lo_, h_alive_stage_.ptr, bytes,
                                     cudaMemcpyHostToDevice, stream_));
        GSS_CUDA_TRY(cudaEventRecord(alive_staged_, stream_));
    }
    alive_synced_ = true;
    alive_lo_ = SIZE_MAX;
    alive_hi_ = 0;
    return GSS_OK;
}

int Sharer::compact_device() {
    // drops evicted clauses from the device arrays (order kept, on the GPU)
    GSS_TRY(sync_alive());
    const uint32_t n = dev_clauses_;
    const int64_t live_lits = dev_lits_;  // an upper bound on what stays
    GSS_TRY(d_lits2_.reserve((size_t) (live_lits + kClausePad) * sizeof(int32_t)));
    GSS_TRY(d_offsets2_.reserve(((size_t) n + 1) * sizeof(int64_t)));
    GSS_TRY(d_orig2_.reserve(std::max<size_t>(n, 1) * sizeof(uint32_t)));
    GSS_TRY(d_compact_.reserve(compact_scratch_bytes(n)));
    CompactArgs c;
    c.lits = (const int32_t *) d_lits_.ptr;
    c.offsets = (const int64_t *) d_offsets_.ptr;
    c.ids = (const uint32_t *) d_orig_.ptr;
    c.n_clauses = n;
    c.alive = (const uint32_t *) d_alive_.ptr;
    c.new_lits = (int32_t *) d_lits2_.ptr;
    c.new_offsets = (int64_t *) d_offsets2_.ptr;
    c.new_ids = (uint32_t *) d_orig2_.ptr;
    c.scratch = d_compact_.ptr;
    uint32_t kept;
    int64_t kept_lits;
    GSS_TRY(compact_by_id(c, stream_, sm_count_, &kept, &kept_lits));
    for (auto bufs : {std::make_pair(&d_lits_, &d_lits2_), std::make_pair(&d_offsets_, &d_offsets2_),
                      std::make_pair(&d_orig_, &d_orig2_)}) {
        std::swap(bufs.first->ptr, bufs.second->ptr);
        std::swap(bufs.first->bytes, bufs.second->bytes);
    }
    // the same order-preserving filter on the host's copy of the id map
    size_t w = 0;
    for (size_t p = 0; p < h_dev_meta_.size(); p++) {
        const uint32_t i = h_dev_meta_[p];
        if ((h_alive_[i >> 5] >> (i & 31)) & 1u) h_dev_meta_[w++] = i;
    }
    h_dev_meta_.resize(w);
    if (w != kept) return set_error(GSS_ERR_STATE, "device compaction kept %u clauses, the host expects %zu", kept, w);
    dev_clauses_ = kept;
    dev_lits_ = kept_lits;
    dev_dead_ = 0;
    device_compactions_++;
    return GSS_OK;
}

void Sharer::evict(int64_t n) {
    // Oldest first among the clauses not reported in the last kRecentPasses
    // passes (the first sweep); then, if that is not enough, the oldest of
    // the rest (the second). Age is the order of meta_ (the device order
    // keeps it): arrival order, except that a reduceDb sorts its survivors by
    // length. evict_cursor_ is the oldest live clause the first sweep may
    // still take (the oldest one it skipped as recently reported, or the one
    // after the last it took).
    constexpr int32_t kRecentPasses = 8;
    auto live = [&](size_t i) { return (h_alive_[i >> 5] >> (i & 31)) & 1u; };
    auto take = [&](size_t i) {
        h_alive_[i >> 5] &= ~(1u << (i & 31));
        mark_alive(i >> 5, (i >> 5) + 1);
        n_dead_++;
        dev_dead_++;
        evicted_++;
        stats_[kGpuClauses]--;
        stats_[kGpuClauseLengthSum] -= meta_[i].len;
    };
    size_t first_skipped = SIZE_MAX;
    size_t i = evict_cursor_;
    for (; i < meta_.size() && n > 0; i++) {
        if (h_alive_[i >> 5] == 0) {  // a whole word of tombstones
            i |= 31;
            continue;
        }
        if (!live(i)) continue;
        const ClauseMeta &m = meta_[i];
        if (m.last_report >= 0 && pass_no_ - m.last_report <= kRecentPasses) {
            first_skipped = std::min(first_skipped, i);
            continue;
        }
        take(i);
        n--;
    }
    evict_cursor_ = std::min(first_skipped, i);
    for (size_t j = 0; j < meta_.size() && n > 0; j++) {
        if (!live(j)) continue;
        take(j);
        n--;
    }
}

int Sharer::compact(bool upload, std::vector<uint32_t> *old_index) {
    // drops evicted clauses from meta_ and the activities, keeping the order
    // (and so the age order); upload = rebuild the device database too;
    // old_index receives the former index of each kept clause
    std::vector<uint8_t> keep(meta_.size(), 0);
    std::vector<ClauseMeta> kept;
    kept.reserve(meta_.size() - n_dead_);
    if (old_index) old_index->clear();
    for (size_t i = 0; i < meta_.size(); i++) {
        if (h_alive_[i >> 5] & (1u << (i & 31))) {
            keep[i] = 1;
            kept.push_back(meta_[i]);
            if (old_index) old_index->push_back((uint32_t) i);
        }
    }
    act_->compact(keep);
    meta_.swap(kept);
    if (upload) return upload_db();
    h_alive_.assign((meta_.size() + 31) / 32, ~0u);
    n_dead_ = 0;
    evict_cursor_ = 0;
    return GSS_OK;
}

void Sharer::reserve_for_budget(size_t n_new, size_t n_new_lits) {
    // Under an HBM budget the database streams: clauses come in, the oldest
    // leave as tombstones. Host arrays hold up to twice the budget before a
    // host compaction, device arrays about 1.25 times before a device one.
    // Growing those arrays by doubling in the middle of serving stalls one
    // pass for tens of milliseconds (a 400 MB host copy at 2^24 clauses), so
    // their room is set aside once, the first time the budget is in force.
    if (budget_ <= 0 || reserved_for_ >= budget_) return;
    const size_t host_clauses = (size_t) (2 * budget_) + n_new + 4096;
    meta_.reserve(host_clauses);
    act_->reserve(host_clauses);
    h_alive_.reserve((host_clauses + 31) / 32);
    const size_t dev_clauses = (size_t) (budget_ + budget_ / 4) + n_new + 4096;
    const double mean_len = (double) (stats_[kGpuClauseLengthSum] + (int64_t) n_new_lits) /
                            (double) std::max<int64_t>(stats_[kGpuClauses] + (int64_t) n_new, 1);
    const size_t dev_lits = (size_t) (mean_len * (double) dev_clauses * 1.1) + kClausePad;
    h_lits_.reserve(h_lits_.size() + (size_t) (mean_len * (double) budget_) + n_new_lits);
    // best effort: without the device room, the arrays grow when needed (and
    // a failure there takes the out-of-memory path)
    if (d_lits_.grow_keep(dev_lits * sizeof(int32_t), stream_, (size_t) dev_lits_ * sizeof(int32_t)) == GSS_OK &&
        d_offsets_.grow_keep((dev_clauses + 1) * sizeof(int64_t), stream_,
                             (size_t) (dev_clauses_ ? dev_clauses_ + 1 : 0) * sizeof(int64_t)) == GSS_OK &&
        d_orig_.grow_keep(dev_clauses * sizeof(uint32_t), stream_, (size_t) dev_clauses_ * sizeof(uint32_t)) ==
            GSS_OK) {
        d_alive_.grow_keep((host_clauses + 31) / 32 * sizeof(uint32_t), stream_,
                           alive_synced_ ? std::min(d_alive_.bytes, (host_clauses + 31) / 32 * sizeof(uint32_t)) : 0);
    }
    reserved_for_ = budget_;
}

int Sharer::append_clauses(std::vector<int64_t> &ids, std::vector<int32_t> &lits, std::vector<uint32_t> &lens) {
    // HostClauses::getUpdatesForDevice (gpuShareLib/Clauses.cu:318-346): per
    // new clause, decay the activity increment, then give the clause that
    // increment as its activity (PerSizeKeeper::addClause, :200-217).
    const size_t first = meta_.size();
    std::vector<size_t> order(ids.size());
    std::vector<uint32_t> starts(ids.size());
    uint32_t off = 0;
    for (size_t i = 0; i < ids.size(); i++) {
        order[i] = i;
        starts[i] = off;
        off += lens[i];
    }
    for (int32_t l : lits) max_var_ = std::max<int64_t>(max_var_, (int64_t) (l >> 1));
    reserve_for_budget(ids.size(), lits.size());
    for (size_t i = 0; i < ids.size(); i++) {
        // the API carries no LBD: LBD := length (GpuClauseSharerImpl.cu:125)
        act_->add((int) lens[i]);
        ClauseMeta m;
        m.gpu_id = ids[i];
        m.len = lens[i];
        m.lit_off = 0;
        m.last_report = -1;
        meta_.push_back(m);
        stats_[kGpuClausesAdded]++;
        stats_[kGpuClauses]++;
        stats_[kGpuClauseLengthSum] += lens[i];
    }
    // Device order of this batch: by length (warps then check equal
    // lengths), and with a large variable count by (variable range, second
    // range, length) with each clause's device literals grouped by range, as
    // the engine's database order (range_order_key). The host arena keeps
    // the literals as the solver gave them, for delivery.
    const int shift = range_shift_for(max_var_, range_log2_);
    std::vector<uint64_t> key(ids.size());
    std::vector<int32_t> relits(shift ? lits.size() : 0);
    for (size_t i = 0; i < ids.size(); i++)
        key[i] = shift ? range_order_key(&lits[starts[i]], lens[i], shift, &relits[starts[i]]) : lens[i];
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return key[a] < key[b]; });
    const std::vector<int32_t> &dev_src = shift ? relits : lits;
    std::vector<ClauseMeta> sorted(ids.size());
    // the new clauses go after the device's last clause
    const int64_t base_off = dev_lits_;
    const uint32_t dpos = dev_clauses_;
    std::vector<int32_t> new_lits;
    new_lits.reserve(off + kClausePad);
    std::vector<int64_t> new_offsets;
    new_offsets.reserve(ids.size());
    int64_t end_off = base_off;
    for (size_t k = 0; k < order.size(); k++) {
        const size_t i = order[k];
        ClauseMeta m = meta_[first + i];
        m.lit_off = (uint32_t) (h_lits_.size());
        h_lits_.insert(h_lits_.end(), lits.begin() + starts[i], lits.begin() + starts[i] + lens[i]);
        new_lits.insert(new_lits.end(), dev_src.begin() + starts[i], dev_src.begin() + starts[i] + lens[i]);
        sorted[k] = m;
        end_off += lens[i];
        new_offsets.push_back(end_off);
    }
    std::copy(sorted.begin(), sorted.end(), meta_.begin() + first);
    std::vector<uint32_t> order32(order.begin(), order.end());
    act_->permute_tail(first, order32);
    new_lits.resize(off + kClausePad, 0);
    const uint32_t n = (uint32_t) meta_.size();
    const uint32_t n_dev = dpos + (uint32_t) ids.size();
    // The host side is complete here: if the device side below runs out of
    // memory, the caller rebuilds the device database from the host's.
    h_alive_.resize((n + 31) / 32, 0u);
    for (size_t i = first; i < n; i++) h_alive_[i >> 5] |= 1u << (i & 31);
    mark_alive(first >> 5, h_alive_.size());
    if (end_off > 0x7FFFFF00LL) return set_error(GSS_ERR_NOMEM, "clause database exceeds 2^31 literals");
    // grow the device arrays, keeping their contents
    GSS_TRY(d_lits_.grow_keep((end_off + kClausePad) * sizeof(int32_t), stream_, base_off * sizeof(int32_t)));
    GSS_TRY(d_offsets_.grow_keep((n_dev + 1) * sizeof(int64_t), stream_, (dpos + 1) * sizeof(int64_t)));
    GSS_TRY(d_orig_.grow_keep(n_dev * sizeof(uint32_t), stream_, dpos * sizeof(uint32_t)));
    // The batch goes up through one pinned stage (a copy from pageable
    // memory would first wait for the whole stream, the pass in flight
    // included): literals (+ zero padding), the offsets of the clause ends
    // (after a leading zero when the database was empty), the ids.
    const size_t nb = ids.size();
    const size_t lit_bytes = new_lits.size() * sizeof(int32_t);
    const size_t off_bytes = (nb + 1) * sizeof(int64_t);
    const size_t lit_pad = (lit_bytes + 15) & ~(size_t) 15;
    const size_t stage_bytes = lit_pad + off_bytes + nb * sizeof(uint32_t);
    // A bulk load (the initial database, a large burst) goes up from pageable
    // memory instead of growing the pinned stage past kMaxAppendStage; that
    // copy waits for the stream, which a bulk load can afford.
    constexpr size_t kMaxAppendStage = 64u << 20;
    std::vector<char> bulk;
    char *stage;
    if (stage_bytes > kMaxAppendStage) {
        bulk.resize(stage_bytes);
        stage = bulk.data();
    } else {
        GSS_CUDA_TRY(cudaEventSynchronize(append_staged_));  // the previous batch has left the stage
        GSS_TRY(h_append_.reserve(stage_bytes));
        stage = (char *) h_append_.ptr;
    }
    memcpy(stage, new_lits.data(), lit_bytes);
    int64_t *st_off = (int64_t *) (stage + lit_pad);
    st_off[0] = 0;
    memcpy(st_off + 1, new_offsets.data(), nb * sizeof(int64_t));
    uint32_t *st_orig = (uint32_t *) (stage + lit_pad + off_bytes);
    for (size_t k = 0; k < nb; k++) st_orig[k] = (uint32_t) (first + k);
    GSS_CUDA_TRY(cudaMemcpyAsync((int32_t *) d_lits_.ptr + base_off, stage, lit_bytes, cudaMemcpyHostToDevice,
                                 stream_));
    // offsets: [dpos] stays (or gets the leading zero), [dpos + 1 ..] are the new ends
    if (dpos == 0)
        GSS_CUDA_TRY(cudaMemcpyAsync(d_offsets_.ptr, st_off, off_bytes, cudaMemcpyHostToDevice, stream_));
    else
        GSS_CUDA_TRY(cudaMemcpyAsync((int64_t *) d_offsets_.ptr + dpos + 1, st_off + 1, nb * sizeof(int64_t),
                                     cudaMemcpyHostToDevice, stream_));
    GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) d_orig_.ptr + dpos, st_orig, nb * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, stream_));
    if (!bulk.empty()) {
        GSS_CUDA_TRY(cudaStreamSynchronize(stream_));  // `bulk` is freed on return
    } else {
        GSS_CUDA_TRY(cudaEventRecord(append_staged_, stream_));
    }
    dev_clauses_ = n_dev;
    dev_lits_ = end_off;
    h_dev_meta_.resize(n_dev);
    for (size_t k = 0; k < nb; k++) h_dev_meta_[dpos + k] = (uint32_t) (first + k);
    return GSS_OK;
}

int Sharer::run_check(Pass &p) {
    // start masks: p.h_start (pinned) holds n_blocks_ * bw_ words
    const size_t padded = (size_t) n_blocks_ * bw_;
    GSS_CUDA_TRY(cudaMemcpyAsync(d_start_.ptr, p.h_start.ptr, padded * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 stream_));
    // capacity: from the option (records per category x categories, as the
    // reference sizes its reporter) and what earlier passes needed
    const int64_t want = std::max<int64_t>((int64_t) opt_.init_report_count * opt_.block_count,
                                           (int64_t) report_cap_ * n_parts_);
    const int64_t per = std::min<int64_t>((want + n_parts_ - 1) / n_parts_, 0x7FFFFFFF);
    if ((uint32_t) per > p.cap_per_part || !p.d_reports.ptr) {
        GSS_TRY(p.d_reports.reserve((size_t) per * n_parts_ * sizeof(gss_report)));
        p.cap_per_part = (uint32_t) per;
    }
    CheckArgs a;
    memset(&a, 0, sizeof a);
    a.lits = (const int32_t *) d_lits_.ptr;
    a.offsets = (const int64_t *) d_offsets_.ptr;
    a.orig = (const uint32_t *) d_orig_.ptr;
    a.n_clauses = p.n_clauses;
    a.scan_begin = 0;
    a.scan_end = p.n_clauses;
    a.state = (const uint2 *) d_state_.ptr;
    a.n_vars = (uint32_t) std::max(dev_vars_, 1);
    a.n_blocks = (uint32_t) n_blocks_;
    a.start = (const uint32_t *) d_start_.ptr;
    a.solver_of_word = (const int32_t *) d_sow_.ptr;
    a.out = (gss_report *) p.d_reports.ptr;
    a.counts = (uint32_t *) p.d_counts.ptr;
    a.n_parts = n_parts_;
    a.cap_per_part = p.cap_per_part;
    a.lpc = eff_lpc_;
    a.g = eff_depth_;
    a.cache_hints = (flags_ & GSS_VARIANT_L2_HINT) ? 1 : 0;
    a.err = (uint32_t *) d_err_.ptr;
    a.alive = nullptr;
    if (dev_dead_ > 0) {
        // evicted clauses still on the device: skipped through the bitmap
        GSS_TRY(sync_alive());
        a.alive = (const uint32_t *) d_alive_.ptr;
        a.alive_by_id = 1;
    }
    GSS_CUDA_TRY(cudaMemsetAsync(a.counts, 0, sizeof(uint32_t) * n_parts_, stream_));
    GSS_CUDA_TRY(cudaMemsetAsync(a.err, 0, sizeof(uint32_t), stream_));
    if (p.active_words > 0 && p.n_clauses > 0) {
        const int wpl = eff_kind_ == GSS_KERNEL_WIDE4 ? 4 : 2;
        const bool wide = eff_kind_ == GSS_KERNEL_WIDE4 || eff_kind_ == GSS_KERNEL_WIDE2;
        if (wide && ((flags_ & GSS_VARIANT_PERSISTENT) ||
                     (kind_ == GSS_KERNEL_AUTO && valid_wide_persist_variant(wpl, eff_lpc_, eff_depth_)))) {
            // the persistent form, as the engine's automatic variant
            GSS_TRY(d_work_.reserve(sizeof(uint32_t)));
            GSS_CUDA_TRY(cudaMemsetAsync(d_work_.ptr, 0, sizeof(uint32_t), stream_));
            GSS_TRY(launch_check_wide_persist(nullptr, a, wpl, eff_lpc_, eff_depth_, (uint32_t *) d_work_.ptr, stream_,
                                              sm_count_));
        } else if (wide) {
            GSS_TRY(launch_check_wide(a, wpl, (flags_ & GSS_VARIANT_OCCUPANCY) ? 1 : 0, stream_, sm_count_));
        } else {
            GSS_TRY(launch_check(a, stream_, sm_count_));
        }
    }
    GSS_CUDA_TRY(cudaMemcpyAsync(p.h_counts.ptr, p.d_counts.ptr, sizeof(uint32_t) * n_parts_, cudaMemcpyDeviceToHost,
                                 stream_));
    GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) p.h_counts.ptr + n_parts_, d_err_.ptr, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, stream_));
    GSS_CUDA_TRY(cudaEventRecord(p.counted, stream_));
    return GSS_OK;
}

int Sharer::collect(Pass &p) {
    // GpuRunner::wholeRun waits for the check of the pass in flight
    // (afterFindClauses, gpuShareLib/GpuRunner.cu:216-222), then queues the
    // copy of its reports (scheduleGpuToCpuCopyAsync, :325-328) behind the
    // set-to-last of its variables (launchGpu, :356-357).
    const int64_t t0 = now_us();
    GSS_CUDA_TRY(cudaEventSynchronize(p.counted));
    if (opt_.quick_prof) stats_[kTimeSpentTestingClauses] += now_us() - t0;
    for (int attempt = 0;; attempt++) {
        const uint32_t *hc = (const uint32_t *) p.h_counts.ptr;
        if (hc[n_parts_] != 0) return set_error(GSS_ERR_CUDA, "a bounded wait in the check kernel gave up");
        int64_t total = 0;
        bool overflow = false;
        uint32_t most = 0;
        for (uint32_t q = 0; q < n_parts_; q++) {
            total += hc[q];
            overflow |= hc[q] > p.cap_per_part;
            most = std::max(most, hc[q]);
        }
        if (!overflow) {
            p.n_reports = total;
            GSS_TRY(p.h_reports.reserve(std::max<size_t>((size_t) total, 1) * sizeof(gss_report)));
            int64_t pos = 0;
            for (uint32_t q = 0; q < n_parts_; q++) {
                if (!hc[q]) continue;
                GSS_CUDA_TRY(cudaMemcpyAsync((gss_report *) p.h_reports.ptr + pos,
                                             (gss_report *) p.d_reports.ptr + (size_t) q * p.cap_per_part,
                                             hc[q] * sizeof(gss_report), cudaMemcpyDeviceToHost, stream_));
                pos += hc[q];
            }
            break;
        }
        if (attempt >= 3) return set_error(GSS_ERR_OVERFLOW, "report queues kept overflowing");
        // The pass's slots are still on the device (not broadcast yet): check
        // again with room for all (for the later passes too).
        report_cap_ = (uint32_t) std::min<int64_t>((int64_t) most * 2 + 1024, 0x7FFFFFFF);
        GSS_TRY(run_check(p));
        GSS_CUDA_TRY(cudaEventSynchronize(p.counted));
    }
    // the pass's variables take their last slot's value in all 32 slots
    // (stream-ordered: the next pass's updates are scattered after this)
    if (p.n_updates > 0) {
        GSS_CUDA_TRY(cudaMemcpyAsync(d_last_mask_.ptr, p.h_last.ptr, (size_t) n_blocks_ * bw_ * sizeof(uint32_t),
                                     cudaMemcpyHostToDevice, stream_));
        set_to_last_kernel<<<grid_for(p.n_updates, sm_count_), 256, 0, stream_>>>(
            (const DevUpdate *) d_updates_.ptr, (uint32_t) p.n_updates, (const uint32_t *) d_last_mask_.ptr,
            (uint2 *) d_state_.ptr, (uint32_t) dev_vars_, (uint32_t) bw_);
        GSS_CUDA_TRY(cudaGetLastError());
    }
    GSS_CUDA_TRY(cudaEventRecord(p.copied, stream_));
    p.pending = false;
    p.collected = true;
    p.noted = false;
    return GSS_OK;
}

int Sharer::note_reports(Pass &p) {
    // The clause-side effects of a collected pass, cheap and needed before
    // the next eviction: statistics, activity bumps and last-report passes
    // (GpuRunner::gatherGpuRunResults, gpuShareLib/GpuRunner.cu:360-378).
    if (!p.collected || p.noted) return GSS_OK;
    GSS_CUDA_TRY(cudaEventSynchronize(p.copied));
    const gss_report *rep = (const gss_report *) p.h_reports.ptr;
    stats_[kGpuRuns]++;
    stats_[kTotalAssigClauseTested] += (int64_t) p.n_clauses * p.assig_total;
    stats_[kClauseTestsOnGroups] += p.n_clauses;
    stats_[kClauseTestsOnAssigs] += (int64_t) p.n_clauses * p.active_words;
    stats_[kGpuReports] += p.n_reports;
    for (int64_t i = 0; i < p.n_reports; i++) {
        act_->bump(rep[i].clause);
        meta_[rep[i].clause].last_report = p.number;
    }
    p.noted = true;
    return GSS_OK;
}

int Sharer::deliver(Pass &p) {
    // Reported::fill (gpuShareLib/Reported.cu:160-204): a batch for every
    // solver that had assignments in the pass, reported or not.
    if (!p.collected) return GSS_OK;
    GSS_TRY(note_reports(p));
    const int64_t t1 = now_us();
    const gss_report *rep = (const gss_report *) p.h_reports.ptr;
    std::vector<ClauseBatch *> batch(reported_.size(), nullptr);
    for (size_t s = 0; s < p.assig.size() && s < reported_.size(); s++) {
        if (p.assig[s].count > 0) {
            batch[s] = reported_[s]->queue.new_batch();
            batch[s]->assig = p.assig[s];
        }
    }
    for (int64_t i = 0; i < p.n_reports; i++) {
        const gss_report &r = rep[i];
        const int s = (int) r.solver;
        if (s < 0 || s >= (int) batch.size()) continue;
        if (!batch[s]) {
            batch[s] = reported_[s]->queue.new_batch();
            batch[s]->assig = p.assig[s];
        }
        ClauseBatch &b = *batch[s];
        const ClauseMeta &m = meta_[r.clause];
        b.clauses.emplace_back(m.gpu_id, (int32_t) b.lits.size());
        b.lits.insert(b.lits.end(), h_lits_.begin() + m.lit_off, h_lits_.begin() + m.lit_off + m.len);
        b.had_some |= r.mask;
    }
    for (size_t s = 0; s < batch.size(); s++)
        if (batch[s]) reported_[s]->queue.publish();
    if (opt_.quick_prof) stats_[kTimeSpentFillingReported] += now_us() - t1;
    p.collected = false;
    return GSS_OK;
}

int Sharer::finish_pending() {
    // collects and delivers every pass (before a reduceDb renumbers clauses)
    Pass &p = pass_[cur_];
    if (p.pending) GSS_TRY(collect(p));
    GSS_TRY(deliver(pass_[cur_ ^ 1]));
    return deliver(p);
}

int Sharer::launch_pass() {
    // GpuRunner::startGpuRunAsync (gpuShareLib/GpuRunner.cu:274-321). The
    // pass launched by the previous call (pass_[cur_]) is collected: its
    // reports are on their way to the host and its set-to-last is queued.
    Pass &prev = pass_[cur_];
    Pass &p = pass_[cur_ ^ 1];
    GSS_TRY(deliver(p));  // delivered by the previous call already; kept for safety
    std::vector<int64_t> ids;
    std::vector<int32_t> lits;
    std::vector<uint32_t> lens;
    {
        std::lock_guard<std::mutex> g(stage_lock_);
        ids.swap(st_ids_);
        lits.swap(st_lits_);
        lens.swap(st_lens_);
    }
    if (!ids.empty()) {
        int rc = append_clauses(ids, lits, lens);
        if (rc == GSS_ERR_NOMEM) rc = recover_from_oom();
        GSS_TRY(rc);
    }
    if (budget_ > 0 && live_clauses() > budget_) {
        // eviction keeps the recently reported clauses: it needs the
        // collected pass's reports on the clauses first
        GSS_TRY(note_reports(prev));
        evict(live_clauses() - budget_);
        if (n_dead_ * 2 > (int64_t) meta_.size()) {
            GSS_TRY(deliver(prev));  // a host compaction renumbers the clauses its reports name
            GSS_TRY(compact());      // host tombstones: rebuild everything
        } else if (dev_dead_ * 5 > (int64_t) dev_clauses_) {
            GSS_TRY(compact_device());
        }
    }
    if (stats_[kGpuClauses] == 0) return GSS_OK;  // nothing to check: assignments wait
    int rc = ensure_state();
    if (rc == GSS_ERR_NOMEM) {
        GSS_TRY(recover_from_oom());
        rc = ensure_state();
    }
    GSS_TRY(rc);
    const int64_t t0 = now_us();
    const int n_solvers = (int) solvers_.size();
    const size_t padded = (size_t) n_blocks_ * bw_;
    GSS_TRY(p.h_start.reserve(padded * sizeof(uint32_t)));
    GSS_TRY(p.h_last.reserve(padded * sizeof(uint32_t)));
    uint32_t *start = (uint32_t *) p.h_start.ptr;
    uint32_t *last = (uint32_t *) p.h_last.ptr;
    memset(start, 0, padded * sizeof(uint32_t));
    memset(last, 0, padded * sizeof(uint32_t));
    p.assig.assign(n_solvers, AssigIds());
    p.assig_total = 0;
    p.active_words = 0;
    std::vector<DevUpdate> ups;
    for (int s = 0; s < n_solvers; s++) {
        SolverAssigs &sa = *solvers_[s];
        // HostAssigs::fillAssigsAsync (Assigs.cu:347-357): a solver whose lock
        // is busy sends nothing this pass.
        if (!sa.lock.try_lock()) continue;
        // OneSolverAssigs::copyUpdatesLocked (Assigs.cu:243-300)
        p.assig[s].start = sa.first_id_used;
        p.assig[s].count = (int) (sa.current_id - sa.first_id_used);
        int64_t last_id;
        if (sa.current_id == 0)
            last_id = 0;
        else if (sa.current_id == sa.first_id_used + kSlots)
            last_id = sa.current_id - 1;
        else
            last_id = sa.current_id;
        start[s] = ~sa.not_completed;
        last[s] = 1u << (uint32_t) (last_id % kSlots);
        for (const VarUpdate &u : sa.updates)
            if ((int) u.var < dev_vars_) ups.push_back(DevUpdate{u.var, (uint32_t) s, u.is_def, u.is_true});
        sa.updates.clear();
        sa.first_id_used = sa.current_id;
        sa.not_completed = ~0u;
        sa.lock.unlock();
        p.assig_total += p.assig[s].count;
        if (start[s]) p.active_words++;
    }
    p.n_updates = (int64_t) ups.size();
    // The rings are cut: from here on the pass must run. If a device buffer
    // cannot grow, the database is reduced and the same updates are sent
    // again (GpuRunner::wholeRun, gpuShareLib/GpuRunner.cu:243-260).
    auto send_and_check = [&]() -> int {
        if (!ups.empty()) {
            // h_updates_ is free: the previous pass's copy from it ran before
            // that pass's check, which has finished
            const size_t bytes = ups.size() * sizeof(DevUpdate);
            GSS_TRY(d_updates_.reserve(bytes));
            GSS_TRY(h_updates_.reserve(bytes));
            memcpy(h_updates_.ptr, ups.data(), bytes);
            GSS_CUDA_TRY(cudaMemcpyAsync(d_updates_.ptr, h_updates_.ptr, bytes, cudaMemcpyHostToDevice, stream_));
            scatter_updates_kernel<<<grid_for(ups.size(), sm_count_), 256, 0, stream_>>>(
                (const DevUpdate *) d_updates_.ptr, (uint32_t) ups.size(), (uint2 *) d_state_.ptr,
                (uint32_t) dev_vars_, (uint32_t) bw_);
            GSS_CUDA_TRY(cudaGetLastError());
        }
        p.n_clauses = dev_clauses_;
        return run_check(p);
    };
    rc = send_and_check();
    if (rc == GSS_ERR_NOMEM) {
        GSS_TRY(recover_from_oom());
        rc = send_and_check();
    }
    GSS_TRY(rc);
    if (opt_.quick_prof) stats_[kTimeSpentFillingAssigs] += now_us() - t0;
    p.pending = true;
    p.number = pass_no_++;
    cur_ ^= 1;
    return GSS_OK;
}

int Sharer::recover_from_oom() {
    // GpuRunner::wholeRun on notEnoughGpuMemory (gpuShareLib/GpuRunner.cu:243-260):
    // reduce the clause database (HostClauses::reduceDb) and remember it
    // (hasRunOutOfGpuMemoryOnce, which solvers read to stop growing their
    // reduce period, glucose-syrup/gpu/GpuMultiSolver.cc:130-134). The
    // reduced database is rebuilt on the device from the host's copy, whose
    // old device buffers are freed first.
    out_of_memory_ = true;
    log(1, "c Ran out of GPU memory: reducing the GPU clause database\n");
    GSS_TRY(finish_pending());
    return reduce_now(false);  // an upload frees the old device buffers before allocating new ones
}

int Sharer::gpu_run() {
    // GpuClauseSharerImpl::gpuRun -> GpuRunner::wholeRun
    // (gpuShareLib/GpuClauseSharerImpl.cu:83-94, GpuRunner.cu:211-261): the
    // pass in flight is collected, the next one is cut and launched, and the
    // collected pass's reports are delivered to the solvers' queues while the
    // new one runs on the GPU.
    const int64_t t0 = now_us();
    GSS_CUDA_TRY(cudaSetDevice(device_));
    Pass &prev = pass_[cur_];
    if (prev.pending) GSS_TRY(collect(prev));
    GSS_TRY(launch_pass());
    GSS_TRY(deliver(prev));
    const int64_t spent = now_us() - t0;
    if (spent < opt_.min_latency_us) std::this_thread::sleep_for(std::chrono::microseconds(opt_.min_latency_us - spent));
    return GSS_OK;
}

int Sharer::reduce_db() {
    // GpuClauseSharerImpl::reduceDb -> wholeRun(false) then HostClauses::reduceDb
    // (gpuShareLib/GpuClauseSharerImpl.cu:105-110, gpuShareLib/Clauses.cu:426-465),
    // with the implementation's activity-only policy (actOnly = true,
    // GpuClauseSharerImpl.cu:72): keep clauses of length 1 and 2, and longer
    // ones with lbd < 100 whose activity reaches the median estimate.
    GSS_CUDA_TRY(cudaSetDevice(device_));
    GSS_TRY(finish_pending());
    return reduce_now(true);
}

int Sharer::reduce_now(bool on_device) {
    // Where each clause is on the device now, by meta_ index (-1: not there,
    // which happens only after a failed upload).
    std::vector<int64_t> dev_pos(meta_.size(), -1);
    if (h_dev_meta_.size() == dev_clauses_)
        for (size_t p = 0; p < h_dev_meta_.size(); p++) dev_pos[h_dev_meta_[p]] = (int64_t) p;
    std::vector<uint32_t> from_compact;  // meta_ index before the tombstones went
    if (n_dead_ > 0) {
        GSS_TRY(compact(false, &from_compact));  // the rebuild below replaces the device side
    } else {
        from_compact.resize(meta_.size());
        for (size_t i = 0; i < meta_.size(); i++) from_compact[i] = (uint32_t) i;
    }
    const int64_t t0 = now_us();
    added_at_last_reduce_ = stats_[kGpuClausesAdded];
    stats_[kGpuReduceDbs]++;
    {
        std::ostringstream os;
        os << "c Reducing gpu clause db, clause count is " << stats_[kGpuClauses];
        log(2, os.str());
    }
    int min_lim, max_lim;
    float act;
    act_->removing_thresholds(true, stats_[kGpuClauses], min_lim, max_lim, act);
    // PerSizeKeeper::tryRemoveClausesAsync (Clauses.cu:249-282) only looks at
    // clauses of length 3 and more.
    std::vector<ClauseMeta> kept;
    std::vector<uint32_t> kept_from;
    std::vector<uint8_t> keep(meta_.size(), 0);
    kept.reserve(meta_.size());
    int64_t len_sum = 0;
    for (size_t i = 0; i < meta_.size(); i++) {
        const ClauseMeta &m = meta_[i];
        if (m.len <= 2 || ClauseActivity::keep(act_->lbd((uint32_t) i), act_->activity((uint32_t) i), min_lim,
                                               max_lim, act)) {
            keep[i] = 1;
            kept.push_back(m);
            kept_from.push_back(from_compact[i]);
            len_sum += m.len;
        }
    }
    act_->compact(keep);
    // the kept clauses in the device order of appended batches (length, or
    // variable range, second range, length)
    const int shift = range_shift_for(max_var_, range_log2_);
    std::vector<uint64_t> key(kept.size());
    for (size_t k = 0; k < kept.size(); k++)
        key[k] = shift ? range_order_key(&h_lits_[kept[k].lit_off], kept[k].len, shift, nullptr) : kept[k].len;
    std::vector<uint32_t> order(kept.size());
    for (uint32_t i = 0; i < order.size(); i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    const uint32_t n = (uint32_t) kept.size();
    meta_.resize(n);
    std::vector<uint32_t> src(std::max<uint32_t>(n, 1));
    bool all_on_device = on_device;
    for (uint32_t k = 0; k < n; k++) {
        meta_[k] = kept[order[k]];
        const int64_t p = dev_pos[kept_from[order[k]]];
        all_on_device &= p >= 0;
        src[k] = (uint32_t) std::max<int64_t>(p, 0);
    }
    act_->permute(order);
    stats_[kGpuClauses] = (int64_t) meta_.size();
    stats_[kGpuClauseLengthSum] = len_sum;
    if (all_on_device) {
        GSS_TRY(rebuild_on_device(src));
    } else {
        GSS_TRY(upload_db());
    }
    stats_[kTimeSpentReduceGpuDb] += now_us() - t0;
    {
        std::ostringstream os;
        os << "c Done reducing gpu clause db, clause count is " << stats_[kGpuClauses];
        log(2, os.str());
    }
    return GSS_OK;
}

int Sharer::rebuild_on_device(const std::vector<uint32_t> &src) {
    // The device database in meta_ order, its literals moved on the device
    // (gather_clauses): only the old position and the new offset of each
    // clause go up, 12 bytes a clause, instead of all its literals.
    const uint32_t n = (uint32_t) meta_.size();
    std::vector<int64_t> offsets(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + meta_[i].len;
    const int64_t n_lits = offsets[n];
    GSS_TRY(d_lits2_.reserve((size_t) (n_lits + kClausePad) * sizeof(int32_t)));
    GSS_TRY(d_offsets2_.reserve(((size_t) n + 1) * sizeof(int64_t)));
    GSS_TRY(d_orig2_.reserve(std::max<size_t>(n, 1) * sizeof(uint32_t)));
    GSS_TRY(d_compact_.reserve(std::max<size_t>(n, 1) * sizeof(uint32_t)));
    GSS_CUDA_TRY(cudaMemcpy(d_offsets2_.ptr, offsets.data(), ((size_t) n + 1) * sizeof(int64_t),
                            cudaMemcpyHostToDevice));
    GSS_CUDA_TRY(cudaMemcpy(d_compact_.ptr, src.data(), std::max<size_t>(n, 1) * sizeof(uint32_t),
                            cudaMemcpyHostToDevice));
    GatherArgs g;
    g.lits = (const int32_t *) d_lits_.ptr;
    g.offsets = (const int64_t *) d_offsets_.ptr;
    g.src = (const uint32_t *) d_compact_.ptr;
    g.new_offsets = (const int64_t *) d_offsets2_.ptr;
    g.n_new = n;
    g.n_new_lits = n_lits;
    g.new_lits = (int32_t *) d_lits2_.ptr;
    g.new_ids = (uint32_t *) d_orig2_.ptr;
    GSS_TRY(gather_clauses(g, stream_, sm_count_));
    GSS_CUDA_TRY(cudaStreamSynchronize(stream_));
    for (auto bufs : {std::make_pair(&d_lits_, &d_lits2_), std::make_pair(&d_offsets_, &d_offsets2_),
                      std::make_pair(&d_orig_, &d_orig2_)}) {
        std::swap(bufs.first->ptr, bufs.second->ptr);
        std::swap(bufs.first->bytes, bufs.second->bytes);
    }
    // the host arena in the new order too
    std::vector<int32_t> arena((size_t) n_lits);
    for (uint32_t i = 0; i < n; i++) {
        memcpy(&arena[offsets[i]], &h_lits_[meta_[i].lit_off], meta_[i].len * sizeof(int32_t));
        meta_[i].lit_off = (uint32_t) offsets[i];
    }
    h_lits_.swap(arena);
    dev_clauses_ = n;
    dev_lits_ = n_lits;
    h_dev_meta_.resize(n);
    for (uint32_t i = 0; i < n; i++) h_dev_meta_[i] = i;
    h_alive_.assign((n + 31) / 32, ~0u);
    n_dead_ = 0;
    dev_dead_ = 0;
    evict_cursor_ = 0;
    alive_synced_ = false;
    alive_lo_ = SIZE_MAX;
    alive_hi_ = 0;
    device_compactions_++;
    return GSS_OK;
}

int Sharer::write_cnf(FILE *f) {
    // HostClauses::writeClausesInCnf (gpuShareLib/Clauses.cu:527-547); the
    // header goes to the same file as the clauses.
    if (!f) return set_error(GSS_ERR_INVALID, "file is NULL");
    fprintf(f, "p cnf %d %lld\n", n_vars_, (long long) stats_[kGpuClauses]);
    std::vector<size_t> order(meta_.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return meta_[a].len < meta_[b].len; });
    for (size_t i : order) {
        if (!(h_alive_[i >> 5] & (1u << (i & 31)))) continue;
        const ClauseMeta &m = meta_[i];
        for (uint32_t k = 0; k < m.len; k++) {
            const int32_t l = h_lits_[m.lit_off + k];
            fprintf(f, "%d ", ((l >> 1) + 1) * ((l & 1) ? -1 : 1));
        }
        fprintf(f, "0\n");
    }
    return GSS_OK;
}

}  // namespace gss

// ---------------------------------------------------------------- C ABI ----

using gss::Sharer;

struct gss_sharer {
    std::unique_ptr<Sharer> impl;
};

extern "C" {

int gss_sharer_create(const gss_sharer_options *opts, gss_log_fn log_fn, void *log_ctx, int device,
                      gss_sharer **out) {
    if (!out) return gss::set_error(GSS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    gss::Options o;
    if (opts) {
        o.block_count = opts->gpu_block_count_guideline;
        o.threads_per_block = opts->gpu_threads_per_block_guideline;
        o.min_latency_us = opts->min_gpu_latency_micros;
        o.verbosity = opts->verbosity;
        o.activity_decay = opts->clause_activity_decay;
        o.quick_prof = opts->quick_prof != 0;
        o.init_report_count = opts->init_report_count_per_category;
        o.max_page_locked = opts->max_page_locked_memory;
    }
    std::function<void(const std::string &)> lf;
    if (log_fn) lf = [log_fn, log_ctx](const std::string &s) { log_fn(s.c_str(), log_ctx); };
    std::unique_ptr<gss_sharer> h(new gss_sharer());
    h->impl.reset(new Sharer(o, lf));
    int rc = h->impl->init(device);
    if (rc != GSS_OK) return rc;
    *out = h.release();
    return GSS_OK;
}

void gss_sharer_options_default(gss_sharer_options *o) {
    if (!o) return;
    // GpuClauseSharerOptions() (gpuShareLib/GpuClauseSharer.h:48-57)
    o->gpu_block_count_guideline = -1;
    o->gpu_threads_per_block_guideline = -1;
    o->min_gpu_latency_micros = -1;
    o->verbosity = 1;
    o->clause_activity_decay = -1;
    o->quick_prof = 1;
    o->init_report_count_per_category = -1;
    o->max_page_locked_memory = -1;
}

int gss_sharer_destroy(gss_sharer *s) {
    delete s;
    return GSS_OK;
}

#define GSS_SHARER(s)                                                       \
    do {                                                                    \
        if (!(s)) return gss::set_error(GSS_ERR_INVALID, "sharer is NULL"); \
    } while (0)

int gss_sharer_gpu_run(gss_sharer *s) {
    GSS_SHARER(s);
    return s->impl->gpu_run();
}

int gss_sharer_reduce_db(gss_sharer *s) {
    GSS_SHARER(s);
    return s->impl->reduce_db();
}

int64_t gss_sharer_added_clause_count(gss_sharer *s) { return s ? s->impl->added_clause_count() : 0; }

int64_t gss_sharer_added_clause_count_at_last_reduce_db(gss_sharer *s) {
    return s ? s->impl->added_at_last_reduce() : 0;
}

int gss_sharer_has_run_out_of_gpu_memory_once(gss_sharer *s) { return s ? (int) s->impl->ran_out_of_memory() : 0; }

int gss_sharer_gpu_mem_info(gss_sharer *s, size_t *free_bytes, size_t *total_bytes) {
    GSS_SHARER(s);
    if (!free_bytes || !total_bytes) return gss::set_error(GSS_ERR_INVALID, "NULL output");
    return s->impl->mem_info(free_bytes, total_bytes);
}

int gss_sharer_global_stat_count(void) { return gss::kGlobalStatCount; }

int64_t gss_sharer_global_stat(gss_sharer *s, int stat) { return s ? s->impl->global_stat(stat) : 0; }

const char *gss_sharer_global_stat_name(int stat) {
    return (stat >= 0 && stat < gss::kGlobalStatCount) ? gss::kGlobalStatNames[stat] : NULL;
}

int gss_sharer_one_solver_stat_count(void) { return gss::kSolverStatCount; }

const char *gss_sharer_one_solver_stat_name(int stat) {
    return (stat >= 0 && stat < gss::kSolverStatCount) ? gss::kSolverStatNames[stat] : NULL;
}

int64_t gss_sharer_one_solver_stat(gss_sharer *s, int solver, int stat) {
    return s ? s->impl->solver_stat(solver, stat) : 0;
}

int gss_sharer_write_clauses_in_cnf(gss_sharer *s, FILE *file) {
    GSS_SHARER(s);
    return s->impl->write_cnf(file);
}

int gss_sharer_set_var_count(gss_sharer *s, int count) {
    GSS_SHARER(s);
    return s->impl->set_var_count(count);
}

int64_t gss_sharer_add_clause(gss_sharer *s, int solver, const int *lits, int count) {
    return s ? s->impl->add_clause(solver, lits, count) : -1;
}

int gss_sharer_set_cpu_solver_count(gss_sharer *s, int count) {
    GSS_SHARER(s);
    return s->impl->set_solver_count(count);
}

int gss_sharer_try_set_solver_values(gss_sharer *s, int solver, const int *lits, int count) {
    return s ? (int) s->impl->try_set_values(solver, lits, count) : 0;
}

int gss_sharer_unset_solver_values(gss_sharer *s, int solver, const int *lits, int count) {
    GSS_SHARER(s);
    s->impl->unset_values(solver, lits, count);
    return GSS_OK;
}

int64_t gss_sharer_try_send_assignment(gss_sharer *s, int solver) { return s ? s->impl->try_send(solver) : -1; }

int gss_sharer_pop_reported_clause(gss_sharer *s, int solver, int **lits, int *count, int64_t *gpu_clause_id) {
    if (!s || !lits || !count || !gpu_clause_id) return 0;
    int *l = nullptr;
    int c = 0;
    int64_t id = 0;
    if (!s->impl->pop_reported(solver, l, c, id)) return 0;
    *lits = l;
    *count = c;
    *gpu_clause_id = id;
    return 1;
}

int64_t gss_sharer_last_assig_all_reported(gss_sharer *s, int solver) {
    return s ? s->impl->last_all_reported(solver) : 0;
}

int gss_sharer_current_assignment(gss_sharer *s, int solver, uint8_t *assig) {
    GSS_SHARER(s);
    s->impl->current_assignment(solver, assig);
    return GSS_OK;
}

int gss_sharer_set_max_clause_len(gss_sharer *s, int n) {
    GSS_SHARER(s);
    if (n < 1 || n > gss::kMaxClauseLen) return gss::set_error(GSS_ERR_INVALID, "maximum clause length out of range");
    s->impl->set_max_clause_len(n);
    return GSS_OK;
}

int gss_sharer_set_clause_budget(gss_sharer *s, int64_t max_clauses) {
    GSS_SHARER(s);
    if (max_clauses < 0) return gss::set_error(GSS_ERR_INVALID, "negative clause budget");
    s->impl->set_clause_budget(max_clauses);
    return GSS_OK;
}

int64_t gss_sharer_evicted_count(gss_sharer *s) { return s ? s->impl->evicted() : -1; }
int64_t gss_sharer_device_compactions(gss_sharer *s) { return s ? s->impl->device_compactions() : -1; }

int gss_sharer_set_locality(gss_sharer *s, int range_log2) {
    if (!s) return gss::set_error(GSS_ERR_INVALID, "sharer is NULL");
    if (range_log2 != -1 && range_log2 != 0 && (range_log2 < 11 || range_log2 > 31))
        return gss::set_error(GSS_ERR_INVALID, "range_log2 must be -1 (automatic), 0 (off) or 11..31, not %d", range_log2);
    s->impl->set_locality(range_log2);
    return GSS_OK;
}

int gss_sharer_set_variant(gss_sharer *s, int kind, int lanes_per_clause, int depth, int flags) {
    GSS_SHARER(s);
    return s->impl->set_variant(kind, lanes_per_clause, depth, flags);
}

}  // extern "C"
