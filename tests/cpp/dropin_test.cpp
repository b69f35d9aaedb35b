// Uses the sharer only through the reference's C++ interface
// (gpuShareLib/GpuClauseSharer.h), as glucose-syrup and rel-newtech do:
// include the header, make the sharer with makeGpuClauseSharerPtr, call the
// virtual methods. Restates two known-answer tests of
// glucose-syrup/test/GpuSolverTest.cu (testClausesAssigsReported :343-391,
// testFindClausesMultiThread :394-454). Exit code 0 = pass.
#include <stdio.h>

#include <memory>
#include <string>
#include <vector>

#include "gpuShareLib/GpuClauseSharer.h"
#include "gpuShareLib/Profiler.h"
#include "gpuShareLib/Utils.h"
#include "gpuShareLib/my_make_unique.h"

using GpuShare::GpuClauseSharer;

static int failures = 0;
#define EXPECT(cond)                                                \
    do {                                                            \
        if (!(cond)) {                                              \
            fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
            failures++;                                             \
        }                                                           \
    } while (0)

static int lit(int v, bool neg = false) { return 2 * v + (neg ? 1 : 0); }

static int pop_count(GpuClauseSharer &s, int solver) {
    int *lits;
    int count;
    long id;
    int n = 0;
    while (s.popReportedClause(solver, lits, count, id)) n++;
    return n;
}

static void execute(GpuClauseSharer &s) {
    s.gpuRun();
    s.gpuRun();
}

static std::unique_ptr<GpuClauseSharer> make(int vars, int solvers) {
    GpuShare::GpuClauseSharerOptions o;
    o.gpuBlockCountGuideline = 3;
    o.gpuThreadsPerBlockGuideline = 32;
    o.minGpuLatencyMicros = 50;
    o.verbosity = 0;
    GpuShare::Logger logger{0, GpuShare::directPrint};
    std::unique_ptr<GpuClauseSharer> s(GpuShare::makeGpuClauseSharerPtr(o, logger.logFunc));
    s->setVarCount(vars);
    s->setCpuSolverCount(solvers);
    return s;
}

int main() {
    {
        auto s = make(3, 3);
        for (int v = 0; v < 3; v++) {
            int l = lit(v);
            s->addClause(-1, &l, 1);
        }
        std::vector<int> a = {lit(0, true), lit(1), lit(2)}, b = {lit(0), lit(1, true), lit(2, true)},
                         c = {lit(0), lit(1, true), lit(2)};
        EXPECT(s->trySetSolverValues(0, a.data(), 3));
        EXPECT(s->trySendAssignment(0) == 0);
        EXPECT(s->trySetSolverValues(0, b.data(), 3));
        EXPECT(s->trySendAssignment(0) == 1);
        EXPECT(s->trySetSolverValues(1, c.data(), 3));
        EXPECT(s->trySendAssignment(1) == 0);
        execute(*s);
        EXPECT(pop_count(*s, 0) == 3);
        EXPECT(pop_count(*s, 1) == 1);
        EXPECT(pop_count(*s, 2) == 0);
        int one = lit(1);
        EXPECT(s->trySetSolverValues(0, &one, 1));
        EXPECT(s->trySendAssignment(0) == 2);
        execute(*s);
        EXPECT(pop_count(*s, 0) == 1);
        EXPECT(pop_count(*s, 1) == 0);
        EXPECT(s->getGlobalStatCount() == 13);
        EXPECT(std::string(s->getGlobalStatName(GpuShare::gpuClauses)) == "gpuClauses");
        EXPECT(s->getGlobalStat(GpuShare::gpuClauses) == 3);
        EXPECT(s->getOneSolverStat(0, GpuShare::reportedClauses) == 4);
    }
    {
        auto s = make(3, 1);
        std::vector<int> vals = {lit(0, true), lit(1)};
        EXPECT(s->trySetSolverValues(0, vals.data(), 2));
        EXPECT(s->trySendAssignment(0) == 0);
        std::vector<std::vector<int>> cls = {{lit(0), lit(1)}, {lit(0), lit(1, true)}, {lit(1, true), lit(2)}};
        for (auto &cl : cls) s->addClause(-1, cl.data(), (int) cl.size());
        execute(*s);
        int *lits;
        int count;
        long id;
        int seen = 0;
        while (s->popReportedClause(0, lits, count, id)) {
            EXPECT(count == 2);
            EXPECT(id == 1 || id == 2);
            if (id == 1) EXPECT(lits[0] == lit(0) && lits[1] == lit(1, true));
            if (id == 2) EXPECT(lits[0] == lit(1, true) && lits[1] == lit(2));
            seen++;
        }
        EXPECT(seen == 2);
        unsigned long t = 0;
        {
            GpuShare::TimeGauge tg(t, true);
        }
        auto p = my_make_unique<int>(5);
        EXPECT(*p == 5);
        FILE *f = tmpfile();
        s->writeClausesInCnf(f);
        fclose(f);
    }
    if (failures) {
        fprintf(stderr, "%d failure(s)\n", failures);
        return 1;
    }
    printf("drop-in C++ test passed\n");
    return 0;
}
