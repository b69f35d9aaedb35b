// GpuShare::makeGpuClauseSharerPtr: the C++ class of gpuShareLib/GpuClauseSharer.h
// (include/gpuShareLib/GpuClauseSharer.h) over the C ABI of gpusharesat.h.
// Host-only C++: solvers that include the header and link this library get
// the GB300 engine without other changes.
//
// Errors: the reference prints a message and exits on CUDA failures
// (exitIfError, gpuShareLib/Helper.cu:25-30) and on invalid options
// (writeMessageAndThrow, gpuShareLib/GpuClauseSharerImpl.cu:19-22); this
// class does the same, since the C++ interface has no error returns.
#include <stdio.h>
#include <stdlib.h>

#include "gpuShareLib/GpuClauseSharer.h"
#include "gpusharesat.h"

namespace {

class Gb300ClauseSharer : public GpuShare::GpuClauseSharer {
public:
    Gb300ClauseSharer(const GpuShare::GpuClauseSharerOptions &o, std::function<void(const std::string &)> log)
        : log_(std::move(log)) {
        gss_sharer_options so;
        gss_sharer_options_default(&so);
        so.gpu_block_count_guideline = o.gpuBlockCountGuideline;
        so.gpu_threads_per_block_guideline = o.gpuThreadsPerBlockGuideline;
        so.min_gpu_latency_micros = o.minGpuLatencyMicros;
        so.verbosity = o.verbosity;
        so.clause_activity_decay = o.clauseActivityDecay;
        so.quick_prof = o.quickProf ? 1 : 0;
        so.init_report_count_per_category = o.initReportCountPerCategory;
        so.max_page_locked_memory = o.maxPageLockedMemory;
        check(gss_sharer_create(&so, log_ ? &Gb300ClauseSharer::log_thunk : NULL, &log_, -1, &s_));
    }
    ~Gb300ClauseSharer() override { gss_sharer_destroy(s_); }

    void gpuRun() override { check(gss_sharer_gpu_run(s_)); }
    void reduceDb() override { check(gss_sharer_reduce_db(s_)); }
    long getAddedClauseCount() override { return (long) gss_sharer_added_clause_count(s_); }
    long getAddedClauseCountAtLastReduceDb() override {
        return (long) gss_sharer_added_clause_count_at_last_reduce_db(s_);
    }
    bool hasRunOutOfGpuMemoryOnce() override { return gss_sharer_has_run_out_of_gpu_memory_once(s_) != 0; }
    void getGpuMemInfo(size_t &free, size_t &total) override { check(gss_sharer_gpu_mem_info(s_, &free, &total)); }
    int getGlobalStatCount() override { return gss_sharer_global_stat_count(); }
    long getGlobalStat(GpuShare::GlobalStats stat) override { return (long) gss_sharer_global_stat(s_, (int) stat); }
    void writeClausesInCnf(FILE *file) override { check(gss_sharer_write_clauses_in_cnf(s_, file)); }
    void setVarCount(int n) override { check(gss_sharer_set_var_count(s_, n)); }
    long addClause(int solverId, int *lits, int count) override {
        return (long) gss_sharer_add_clause(s_, solverId, lits, count);
    }
    void setCpuSolverCount(int n) override { check(gss_sharer_set_cpu_solver_count(s_, n)); }
    const char *getOneSolverStatName(GpuShare::OneSolverStats stat) override {
        return gss_sharer_one_solver_stat_name((int) stat);
    }
    const char *getGlobalStatName(GpuShare::GlobalStats stat) override {
        return gss_sharer_global_stat_name((int) stat);
    }
    int getOneSolverStatCount() override { return gss_sharer_one_solver_stat_count(); }
    bool trySetSolverValues(int solver, int *lits, int count) override {
        return gss_sharer_try_set_solver_values(s_, solver, lits, count) != 0;
    }
    void unsetSolverValues(int solver, int *lits, int count) override {
        check(gss_sharer_unset_solver_values(s_, solver, lits, count));
    }
    long trySendAssignment(int solver) override { return (long) gss_sharer_try_send_assignment(s_, solver); }
    bool popReportedClause(int solver, int *&lits, int &count, long &gpuClauseId) override {
        int64_t id = 0;
        if (!gss_sharer_pop_reported_clause(s_, solver, &lits, &count, &id)) return false;
        gpuClauseId = (long) id;
        return true;
    }
    long getLastAssigAllReported(int solver) override { return (long) gss_sharer_last_assig_all_reported(s_, solver); }
    void getCurrentAssignment(int solver, uint8_t *assig) override {
        check(gss_sharer_current_assignment(s_, solver, assig));
    }
    long getOneSolverStat(int solver, GpuShare::OneSolverStats stat) override {
        return (long) gss_sharer_one_solver_stat(s_, solver, (int) stat);
    }

private:
    static void log_thunk(const char *msg, void *ctx) {
        (*static_cast<std::function<void(const std::string &)> *>(ctx))(std::string(msg));
    }
    static void check(int rc) {
        if (rc != GSS_OK) {
            fprintf(stderr, "gpusharesat: %s\n", gss_last_error());
            exit(1);
        }
    }

    std::function<void(const std::string &)> log_;
    gss_sharer *s_ = nullptr;
};

}  // namespace

namespace GpuShare {

GpuClauseSharer *makeGpuClauseSharerPtr(GpuClauseSharerOptions opts,
                                        std::function<void(const std::string &str)> logFunc) {
    return new Gb300ClauseSharer(opts, logFunc);
}

}  // namespace GpuShare
