// Global statistics of the clause sharer, as an X-macro list (no include
// guard: include it with X defined). Names and order are part of the API:
// they are the reference's (gpuShareLib/GlobalStats.h:23-37), indices of
// GpuShare::GlobalStats.
X(gpuClauses)
X(gpuClauseLengthSum)
X(gpuClausesAdded)
X(gpuRuns)
X(clauseTestsOnGroups)
X(clauseTestsOnAssigs)
X(totalAssigClauseTested)
X(gpuReduceDbs)
X(gpuReports)
X(timeSpentTestingClauses)
X(timeSpentFillingAssigs)
X(timeSpentFillingReported)
X(timeSpentReduceGpuDb)
