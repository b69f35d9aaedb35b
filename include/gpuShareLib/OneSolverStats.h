// Per-solver statistics of the clause sharer, as an X-macro list (no include
// guard). Names and order are the reference's
// (gpuShareLib/OneSolverStats.h:24-29), indices of GpuShare::OneSolverStats.
X(varUpdatesSentToGpu)
X(assigsSentToGpu)
X(failuresToFindAssig)
X(reportedClauses)
X(reportedClausesUnit)
X(reportedClausesBinary)
