// GpuShare::GpuClauseSharer - the C++ interface solvers use to share clauses
// through the GPU. Drop-in for gpuShareLib/GpuClauseSharer.h of GpuShareSat:
// the options struct, the two stat enums, the class with its virtual methods
// in the same order and with the same signatures (so the vtable layout is the
// same), its inline do-nothing defaults, and the factory have to stay as they
// are there for glucose-syrup and rel-newtech to compile and link unchanged.
// The implementation behind the factory is the GB300 engine, reached through
// the C ABI of gpusharesat.h.
#ifndef GPUSHARESAT_GB300_GPU_CLAUSE_SHARER_H
#define GPUSHARESAT_GB300_GPU_CLAUSE_SHARER_H

#include <stdint.h>
#include <stdio.h>

#include <functional>
#include <string>

namespace GpuShare {

struct GpuClauseSharerOptions {
    // Guideline for the number of GPU blocks; -1: twice the number of SMs.
    // (Here it sizes the report queues; the kernels size their own grids.)
    int gpuBlockCountGuideline;
    // Guideline for threads per block; -1 for the default (512).
    int gpuThreadsPerBlockGuideline;
    // Every gpuRun() lasts at least this many microseconds; -1: 50.
    int minGpuLatencyMicros;
    // 0: quiet, 1: some output, 2: more.
    int verbosity;
    // Decay of clause activity, strictly between 0 and 1; negative: 0.99999.
    double clauseActivityDecay;
    // Time the phases of a pass into the global statistics.
    bool quickProf;
    // Initial report capacity per category; -1: 10.
    int initReportCountPerCategory;
    // Largest pinned host allocation in bytes; -1: inferred.
    int maxPageLockedMemory;

    GpuClauseSharerOptions()
        : gpuBlockCountGuideline(-1),
          gpuThreadsPerBlockGuideline(-1),
          minGpuLatencyMicros(-1),
          verbosity(1),
          clauseActivityDecay(-1),
          quickProf(true),
          initReportCountPerCategory(-1),
          maxPageLockedMemory(-1) {}
};

enum GlobalStats {
#define X(v) v,
#include "GlobalStats.h"
#undef X
};

enum OneSolverStats {
#define X(v) v,
#include "OneSolverStats.h"
#undef X
};

class GpuClauseSharer {
public:
    // --- from one thread (the GPU thread), or with locking ---

    // One pass: delivers the reports of the previous pass and starts a new
    // one. Meant to be called in a loop by a dedicated thread.
    virtual void gpuRun() {}

    // Removes about half of the clauses on the GPU (lowest activity first).
    virtual void reduceDb() {}

    // Clauses added so far, deleted ones included.
    virtual long getAddedClauseCount() { return 0; }

    virtual long getAddedClauseCountAtLastReduceDb() { return 0; }

    virtual bool hasRunOutOfGpuMemoryOnce() { return false; }

    virtual void getGpuMemInfo(size_t &free, size_t &total) {}

    virtual int getGlobalStatCount() { return 0; }

    virtual long getGlobalStat(GlobalStats stat) { return 0; }

    virtual void writeClausesInCnf(FILE *file) {}

    virtual void setVarCount(int newCount) {}

    // Adds a clause (the caller keeps `lits`). solverId: the solver it comes
    // from, so that it is not reported back to it for assignments it already
    // sent; -1 if none. Returns the clause's id, -1 if it was refused.
    virtual long addClause(int solverId, int *lits, int count) { return -1; }

    // Not thread safe with any other method.
    virtual void setCpuSolverCount(int count) {}

    // --- thread safe ---

    virtual const char *getOneSolverStatName(OneSolverStats stat) { return NULL; }

    virtual const char *getGlobalStatName(GlobalStats stat) { return NULL; }

    virtual int getOneSolverStatCount() { return 0; }

    // --- per solver id: from that solver's thread, or with locking ---

    // Sets the literals true in this solver's current assignment, all or none.
    // False when the solver already has 32 assignments waiting for the GPU.
    virtual bool trySetSolverValues(int cpuSolverId, int *lits, int count) { return false; }

    // Unsets the literals' variables (call it when backtracking).
    virtual void unsetSolverValues(int cpuSolverId, int *lits, int count) {}

    // Sends the current assignment: every clause is checked against it.
    // Returns its id (increasing), or -1 when it could not be sent.
    virtual long trySendAssignment(int cpuSolverId) { return -1; }

    // Next clause reported for this solver; lits belong to the sharer and stay
    // valid until the next call for this solver. A clause is reported once as
    // long as the solver keeps it and it does not trigger again.
    virtual bool popReportedClause(int cpuSolverId, int *&lits, int &count, long &gpuClauseId) { return false; }

    // The latest assignment id for which all reports have been delivered.
    virtual long getLastAssigAllReported(int cpuSolverId) { return 0; }

    // The solver's current assignment: 0 true, 1 false, 2 undefined per variable.
    virtual void getCurrentAssignment(int cpuSolverId, uint8_t *assig) {}

    // --- from any thread (may lag behind the solver's own thread) ---

    virtual long getOneSolverStat(int cpuSolverId, OneSolverStats stat) { return 0; }

    virtual ~GpuClauseSharer() {}
};

GpuClauseSharer *makeGpuClauseSharerPtr(GpuClauseSharerOptions opts,
                                        std::function<void(const std::string &str)> logFunc);

}  // namespace GpuShare

#endif
