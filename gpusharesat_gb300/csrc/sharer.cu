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
    if (done_) cudaEventDestroy(done_);
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
    GSS_CUDA_TRY(cudaEventCreateWithFlags(&done_, cudaEventDisableTiming));
    GSS_TRY(d_counts_.reserve(sizeof(uint32_t) * n_parts_));
    GSS_TRY(d_err_.reserve(sizeof(uint32_t)));
    GSS_TRY(h_counts_.reserve(sizeof(uint32_t) * (n_parts_ + 1)));
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
        GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) d_alive_.ptr + alive_lo_, h_alive_.data() + alive_lo_,
                                     (alive_hi_ - alive_lo_) * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_));
        GSS_CUDA_TRY(cudaStreamSynchronize(stream_));  // pageable source
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

int Sharer::compact(bool upload) {
    // drops evicted clauses from meta_ and the activities, keeping the order
    // (and so the age order); upload = rebuild the device database too
    std::vector<uint8_t> keep(meta_.size(), 0);
    std::vector<ClauseMeta> kept;
    kept.reserve(meta_.size() - n_dead_);
    for (size_t i = 0; i < meta_.size(); i++) {
        if (h_alive_[i >> 5] & (1u << (i & 31))) {
            keep[i] = 1;
            kept.push_back(meta_[i]);
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
    // device order of this batch: by length (warps then check equal lengths)
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return lens[a] < lens[b]; });
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
        new_lits.insert(new_lits.end(), lits.begin() + starts[i], lits.begin() + starts[i] + lens[i]);
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
    if (end_off > 0x7FFFFF00LL) return set_error(GSS_ERR_NOMEM, "clause database exceeds 2^31 literals");
    // grow the device arrays, keeping their contents
    GSS_TRY(d_lits_.grow_keep((end_off + kClausePad) * sizeof(int32_t), stream_, base_off * sizeof(int32_t)));
    GSS_TRY(d_offsets_.grow_keep((n_dev + 1) * sizeof(int64_t), stream_, (dpos + 1) * sizeof(int64_t)));
    GSS_TRY(d_orig_.grow_keep(n_dev * sizeof(uint32_t), stream_, dpos * sizeof(uint32_t)));
    std::vector<uint32_t> orig(ids.size());
    for (size_t k = 0; k < ids.size(); k++) orig[k] = (uint32_t) (first + k);
    GSS_CUDA_TRY(cudaMemcpyAsync((int32_t *) d_lits_.ptr + base_off, new_lits.data(), new_lits.size() * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, stream_));
    if (dpos == 0) {
        int64_t zero = 0;
        GSS_CUDA_TRY(cudaMemcpyAsync(d_offsets_.ptr, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, stream_));
    }
    GSS_CUDA_TRY(cudaMemcpyAsync((int64_t *) d_offsets_.ptr + dpos + 1, new_offsets.data(),
                                 new_offsets.size() * sizeof(int64_t), cudaMemcpyHostToDevice, stream_));
    GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) d_orig_.ptr + dpos, orig.data(), orig.size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, stream_));
    GSS_CUDA_TRY(cudaStreamSynchronize(stream_));  // the host vectors above are pageable
    dev_clauses_ = n_dev;
    dev_lits_ = end_off;
    h_alive_.resize((n + 31) / 32, 0u);
    for (size_t i = first; i < n; i++) h_alive_[i >> 5] |= 1u << (i & 31);
    mark_alive(first >> 5, h_alive_.size());
    return GSS_OK;
}

int Sharer::run_check(Pass &p) {
    const size_t padded = (size_t) n_blocks_ * bw_;
    std::vector<uint32_t> start(padded, 0u);
    for (size_t w = 0; w < p.start.size() && w < padded; w++) start[w] = p.start[w];
    GSS_CUDA_TRY(cudaMemcpyAsync(d_start_.ptr, start.data(), padded * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 stream_));
    // capacity: from the option (records per category x categories, as the
    // reference sizes its reporter) and what earlier passes needed
    const int64_t want = std::max<int64_t>((int64_t) opt_.init_report_count * opt_.block_count,
                                           (int64_t) cap_per_part_ * n_parts_);
    const int64_t per = std::min<int64_t>((want + n_parts_ - 1) / n_parts_, 0x7FFFFFFF);
    if ((uint32_t) per > cap_per_part_ || !d_reports_.ptr) {
        GSS_TRY(d_reports_.reserve((size_t) per * n_parts_ * sizeof(gss_report)));
        cap_per_part_ = (uint32_t) per;
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
    a.out = (gss_report *) d_reports_.ptr;
    a.counts = (uint32_t *) d_counts_.ptr;
    a.n_parts = n_parts_;
    a.cap_per_part = cap_per_part_;
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
        if (eff_kind_ == GSS_KERNEL_WIDE4 || eff_kind_ == GSS_KERNEL_WIDE2) {
            GSS_TRY(launch_check_wide(a, eff_kind_ == GSS_KERNEL_WIDE4 ? 4 : 2,
                                      (flags_ & GSS_VARIANT_OCCUPANCY) ? 1 : 0, stream_, sm_count_));
        } else {
            GSS_TRY(launch_check(a, stream_, sm_count_));
        }
    }
    GSS_CUDA_TRY(cudaMemcpyAsync(h_counts_.ptr, d_counts_.ptr, sizeof(uint32_t) * n_parts_, cudaMemcpyDeviceToHost,
                                 stream_));
    GSS_CUDA_TRY(cudaMemcpyAsync((uint32_t *) h_counts_.ptr + n_parts_, d_err_.ptr, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, stream_));
    GSS_CUDA_TRY(cudaEventRecord(done_, stream_));
    return GSS_OK;
}

int Sharer::gather() {
    // GpuRunner::gatherGpuRunResults (gpuShareLib/GpuRunner.cu:360-383)
    Pass &p = pass_;
    const int64_t t0 = now_us();
    GSS_CUDA_TRY(cudaEventSynchronize(done_));
    if (opt_.quick_prof) stats_[kTimeSpentTestingClauses] += now_us() - t0;
    for (int attempt = 0;; attempt++) {
        const uint32_t *hc = (const uint32_t *) h_counts_.ptr;
        if (hc[n_parts_] != 0) return set_error(GSS_ERR_CUDA, "a bounded wait in the check kernel gave up");
        int64_t total = 0;
        bool overflow = false;
        for (uint32_t q = 0; q < n_parts_; q++) {
            total += hc[q];
            overflow |= hc[q] > cap_per_part_;
        }
        if (!overflow) {
            h_reports_.resize((size_t) total);
            int64_t pos = 0;
            for (uint32_t q = 0; q < n_parts_; q++) {
                if (!hc[q]) continue;
                GSS_CUDA_TRY(cudaMemcpyAsync(h_reports_.data() + pos,
                                             (gss_report *) d_reports_.ptr + (size_t) q * cap_per_part_,
                                             hc[q] * sizeof(gss_report), cudaMemcpyDeviceToHost, stream_));
                pos += hc[q];
            }
            GSS_CUDA_TRY(cudaStreamSynchronize(stream_));
            break;
        }
        if (attempt >= 3) return set_error(GSS_ERR_OVERFLOW, "report queues kept overflowing");
        // The pass's slots are still on the device (not broadcast yet): check again with room for all.
        cap_per_part_ = 0;
        const int64_t want = total * 2 + (int64_t) n_parts_ * 1024;
        GSS_TRY(d_reports_.reserve((size_t) want * sizeof(gss_report)));
        cap_per_part_ = (uint32_t) std::min<int64_t>(want / n_parts_, 0x7FFFFFFF);
        GSS_TRY(run_check(p));
        GSS_CUDA_TRY(cudaEventSynchronize(done_));
    }
    // the pass's variables take their last slot's value in all 32 slots
    if (p.n_updates > 0) {
        std::vector<uint32_t> last((size_t) n_blocks_ * bw_, 0u);
        for (size_t w = 0; w < p.last_mask.size() && w < last.size(); w++) last[w] = p.last_mask[w];
        GSS_CUDA_TRY(cudaMemcpyAsync(d_last_mask_.ptr, last.data(), last.size() * sizeof(uint32_t),
                                     cudaMemcpyHostToDevice, stream_));
        set_to_last_kernel<<<grid_for(p.n_updates, sm_count_), 256, 0, stream_>>>(
            (const DevUpdate *) d_updates_.ptr, (uint32_t) p.n_updates, (const uint32_t *) d_last_mask_.ptr,
            (uint2 *) d_state_.ptr, (uint32_t) dev_vars_, (uint32_t) bw_);
        GSS_CUDA_TRY(cudaGetLastError());
        GSS_CUDA_TRY(cudaStreamSynchronize(stream_));
    }
    stats_[kGpuRuns]++;
    stats_[kTotalAssigClauseTested] += (int64_t) p.n_clauses * p.assig_total;
    stats_[kClauseTestsOnGroups] += p.n_clauses;
    stats_[kClauseTestsOnAssigs] += (int64_t) p.n_clauses * p.active_words;
    stats_[kGpuReports] += (int64_t) h_reports_.size();
    for (const gss_report &r : h_reports_) {
        act_->bump(r.clause);
        meta_[r.clause].last_report = pass_no_;
    }
    pass_no_++;
    const int64_t t1 = now_us();
    // Reported::fill (gpuShareLib/Reported.cu:160-204): a batch for every
    // solver that had assignments in the pass, reported or not.
    std::vector<ClauseBatch *> batch(reported_.size(), nullptr);
    for (size_t s = 0; s < p.assig.size() && s < reported_.size(); s++) {
        if (p.assig[s].count > 0) {
            batch[s] = reported_[s]->queue.new_batch();
            batch[s]->assig = p.assig[s];
        }
    }
    for (const gss_report &r : h_reports_) {
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
    p.pending = false;
    return GSS_OK;
}

int Sharer::launch_pass() {
    // GpuRunner::startGpuRunAsync (gpuShareLib/GpuRunner.cu:274-321)
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
        if (rc == GSS_ERR_NOMEM) out_of_memory_ = true;
        GSS_TRY(rc);
    }
    if (budget_ > 0 && live_clauses() > budget_) {
        evict(live_clauses() - budget_);
        if (n_dead_ * 2 > (int64_t) meta_.size())
            GSS_TRY(compact());  // host tombstones: rebuild everything
        else if (dev_dead_ * 5 > (int64_t) dev_clauses_)
            GSS_TRY(compact_device());
    }
    if (stats_[kGpuClauses] == 0) return GSS_OK;  // nothing to check: assignments wait
    GSS_TRY(ensure_state());
    const int64_t t0 = now_us();
    Pass &p = pass_;
    const int n_solvers = (int) solvers_.size();
    p.assig.assign(n_solvers, AssigIds());
    p.start.assign(n_solvers, 0u);
    p.last_mask.assign(n_solvers, 0u);
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
        p.start[s] = ~sa.not_completed;
        p.last_mask[s] = 1u << (uint32_t) (last_id % kSlots);
        for (const VarUpdate &u : sa.updates)
            if ((int) u.var < dev_vars_) ups.push_back(DevUpdate{u.var, (uint32_t) s, u.is_def, u.is_true});
        sa.updates.clear();
        sa.first_id_used = sa.current_id;
        sa.not_completed = ~0u;
        sa.lock.unlock();
        p.assig_total += p.assig[s].count;
        if (p.start[s]) p.active_words++;
    }
    p.n_updates = (int64_t) ups.size();
    if (!ups.empty()) {
        const size_t bytes = ups.size() * sizeof(DevUpdate);
        GSS_TRY(h_updates_.reserve(bytes));
        GSS_TRY(d_updates_.reserve(bytes));
        memcpy(h_updates_.ptr, ups.data(), bytes);
        GSS_CUDA_TRY(cudaMemcpyAsync(d_updates_.ptr, h_updates_.ptr, bytes, cudaMemcpyHostToDevice, stream_));
        scatter_updates_kernel<<<grid_for(ups.size(), sm_count_), 256, 0, stream_>>>(
            (const DevUpdate *) d_updates_.ptr, (uint32_t) ups.size(), (uint2 *) d_state_.ptr, (uint32_t) dev_vars_,
            (uint32_t) bw_);
        GSS_CUDA_TRY(cudaGetLastError());
    }
    if (opt_.quick_prof) stats_[kTimeSpentFillingAssigs] += now_us() - t0;
    p.n_clauses = dev_clauses_;
    GSS_TRY(run_check(p));
    p.pending = true;
    return GSS_OK;
}

int Sharer::gpu_run() {
    // GpuClauseSharerImpl::gpuRun (gpuShareLib/GpuClauseSharerImpl.cu:83-94)
    const int64_t t0 = now_us();
    GSS_CUDA_TRY(cudaSetDevice(device_));
    if (pass_.pending) GSS_TRY(gather());
    GSS_TRY(launch_pass());
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
    if (pass_.pending) GSS_TRY(gather());
    if (n_dead_ > 0) GSS_TRY(compact(false));  // the upload below rebuilds the device side
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
    std::vector<uint8_t> keep(meta_.size(), 0);
    kept.reserve(meta_.size());
    int64_t len_sum = 0;
    for (size_t i = 0; i < meta_.size(); i++) {
        const ClauseMeta &m = meta_[i];
        if (m.len <= 2 || ClauseActivity::keep(act_->lbd((uint32_t) i), act_->activity((uint32_t) i), min_lim,
                                               max_lim, act)) {
            keep[i] = 1;
            kept.push_back(m);
            len_sum += m.len;
        }
    }
    act_->compact(keep);
    std::vector<uint32_t> order(kept.size());
    for (uint32_t i = 0; i < order.size(); i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return kept[a].len < kept[b].len; });
    meta_.resize(kept.size());
    for (size_t k = 0; k < order.size(); k++) meta_[k] = kept[order[k]];
    act_->permute(order);
    stats_[kGpuClauses] = (int64_t) meta_.size();
    stats_[kGpuClauseLengthSum] = len_sum;
    GSS_TRY(upload_db());
    stats_[kTimeSpentReduceGpuDb] += now_us() - t0;
    {
        std::ostringstream os;
        os << "c Done reducing gpu clause db, clause count is " << stats_[kGpuClauses];
        log(2, os.str());
    }
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

int gss_sharer_set_variant(gss_sharer *s, int kind, int lanes_per_clause, int depth, int flags) {
    GSS_SHARER(s);
    return s->impl->set_variant(kind, lanes_per_clause, depth, flags);
}

}  // extern "C"
