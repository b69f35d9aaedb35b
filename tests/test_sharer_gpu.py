"""The GpuClauseSharer API on the GPU, through the C ABI.

1. The reference's API-level known-answer tests (glucose-syrup/test/GpuSolverTest.cu),
   restated on the sharer's calls: what a solver thread does through
   GpuHelpedSolver (tryCopyTrailForGpu = unset + trySetSolverValues +
   trySendAssignment; gpuImportClauses = popReportedClause until empty) is
   done here directly. `execute` is two gpuRun()s, as TestHelper.cu:55-59.
2. Differential tests against the plain-Python model of the API semantics
   (oracle/sharer_model.py) on random call sequences.
3. A many-solver pass compared with the C oracle.
"""
import numpy as np
import pytest

import oracle
from oracle.sharer_model import SharerModel

pytestmark = pytest.mark.gpu


def lit(v, neg=False):
    return 2 * v + (1 if neg else 0)


def make(lib, n_vars, n_solvers, **kw):
    """A sharer with the reference tests' small dimensions (TestHelper.cu:31-35):
    3 blocks x 32 threads, so report queues start small and overflow often."""
    import gpusharesat_gb300 as g
    opts = dict(gpuBlockCountGuideline=3, gpuThreadsPerBlockGuideline=32, minGpuLatencyMicros=50, verbosity=0)
    opts.update(kw)
    s = g.ClauseSharer(**opts)
    s.setVarCount(n_vars)
    s.setCpuSolverCount(n_solvers)
    return s


def execute(s):
    s.gpuRun()
    s.gpuRun()


class Trail:
    """The part of GpuHelpedSolver that talks to the sharer: a trail of
    literals sent up to trail_copied_until (GpuHelpedSolver.cc:109-157)."""

    def __init__(self, sharer, solver):
        self.s, self.id, self.trail, self.copied = sharer, solver, [], 0

    def enqueue(self, *lits):
        self.trail.extend(lits)

    def backtrack_to(self, n):
        if self.copied > n:
            self.s.unsetSolverValues(self.id, self.trail[n:self.copied])
            self.copied = n
        del self.trail[n:]

    def send(self):
        ok = True
        if self.copied < len(self.trail):
            ok = self.s.trySetSolverValues(self.id, self.trail[self.copied:])
            if ok:
                self.copied = len(self.trail)
        return ok and self.s.trySendAssignment(self.id) >= 0


# ------------------------------------------------------------ known answers

def test_clauses_assigs_reported(lib):
    """GpuSolverTest.cu:343-391: 3 unit clauses, 3 solvers -> 3, 1, 0 imports,
    then one more assignment of solver 0 -> 1 and 0."""
    s = make(lib, 3, 3)
    for v in range(3):
        s.addClause(-1, [lit(v)])
    assert s.trySetSolverValues(0, [lit(0, True), lit(1), lit(2)])
    assert s.trySendAssignment(0) == 0
    assert s.trySetSolverValues(0, [lit(0), lit(1, True), lit(2, True)])
    assert s.trySendAssignment(0) == 1
    assert s.trySetSolverValues(1, [lit(0), lit(1, True), lit(2)])
    assert s.trySendAssignment(1) == 0
    execute(s)
    assert [len(s.popAll(i)) for i in range(3)] == [3, 1, 0]
    assert s.trySetSolverValues(0, [lit(1)])
    assert s.trySendAssignment(0) == 2
    execute(s)
    assert len(s.popAll(0)) == 1
    assert len(s.popAll(1)) == 0


def test_find_clauses_multi_thread(lib):
    """GpuSolverTest.cu:394-454: under x0=F x1=T x2=U exactly (x0|~x1) and
    (~x1|x2) are reported, each with its literals."""
    s = make(lib, 3, 1, gpuBlockCountGuideline=1)
    assert s.trySetSolverValues(0, [lit(0, True), lit(1)])
    assert s.trySendAssignment(0) == 0
    s.addClause(-1, [lit(0), lit(1)])
    s.addClause(-1, [lit(0), lit(1, True)])
    s.addClause(-1, [lit(1, True), lit(2)])
    execute(s)
    got = sorted(tuple(l) for l, _ in s.popAll(0))
    assert got == [(lit(0), lit(1, True)), (lit(1, True), lit(2))]
    assert s.popReportedClause(0) is None


def test_import_binary_and_unary(lib):
    """SolverImportBinary (:456-484) / SolverImportUnary (:656-676): a clause
    with one undefined literal and the rest false is reported."""
    s = make(lib, 3, 1)
    t = Trail(s, 0)
    t.enqueue(lit(0), lit(2))
    s.addClause(-1, [lit(0, True), lit(1)])
    s.addClause(-1, [lit(1)])
    assert t.send()
    execute(s)
    got = sorted(tuple(l) for l, _ in s.popAll(0))
    assert got == [(lit(0, True), lit(1)), (lit(1),)]
    assert s.getOneSolverStat(0, "reportedClausesUnit") == 1
    assert s.getOneSolverStat(0, "reportedClausesBinary") == 1


def test_one_assignment_then_two(lib):
    """GpuSolverTest.cu:486-508: (~x0|~x1|x2) reports once, for the third
    assignment only."""
    s = make(lib, 4, 1)
    s.addClause(-1, [lit(0, True), lit(1, True), lit(2)])
    t = Trail(s, 0)
    t.enqueue(lit(0))
    assert t.send()
    execute(s)
    t.enqueue(lit(3))
    assert t.send()
    t.enqueue(lit(1))
    assert t.send()
    execute(s)
    assert len(s.popAll(0)) == 1


def test_doesnt_import_same_clause_twice(lib):
    """GpuSolverTest.cu:511-538: two assignments of one pass both trigger the
    clause; it is imported once."""
    s = make(lib, 3, 1)
    t = Trail(s, 0)
    t.enqueue(lit(0))
    assert t.send()
    t.backtrack_to(0)
    t.enqueue(lit(1, True))
    assert t.send()
    s.addClause(-1, [lit(0, True), lit(1)])
    execute(s)
    s.popAll(0)
    assert s.getOneSolverStat(0, "reportedClauses") == 1


def test_doesnt_import_same_clause_twice_on_successive_runs(lib):
    """GpuSolverTest.cu:540-564: the same, with the two assignments in two
    passes (two batches)."""
    s = make(lib, 3, 1)
    s.addClause(-1, [lit(0, True), lit(1)])
    t = Trail(s, 0)
    t.enqueue(lit(0))
    assert t.send()
    s.gpuRun()
    t.backtrack_to(0)
    t.enqueue(lit(1, True))
    assert t.send()
    s.gpuRun()
    s.popAll(0)
    s.gpuRun()
    s.popAll(0)
    assert s.getOneSolverStat(0, "reportedClauses") == 1


def test_two_solvers_import_binary(lib):
    """GpuSolverTest.cu:605-632: x0 true in solver 0, false in solver 1; each
    imports the one clause that implies something for it."""
    s = make(lib, 3, 2)
    t0, t1 = Trail(s, 0), Trail(s, 1)
    t0.enqueue(lit(0))
    t1.enqueue(lit(0, True))
    s.addClause(-1, [lit(0, True), lit(1)])
    s.addClause(-1, [lit(0), lit(1, True)])
    assert t0.send() and t1.send()
    execute(s)
    assert [tuple(l) for l, _ in s.popAll(0)] == [(lit(0, True), lit(1))]
    assert [tuple(l) for l, _ in s.popAll(1)] == [(lit(0), lit(1, True))]


def test_solver_unsets(lib):
    """GpuSolverTest.cu:634-654: after backtracking, a variable is undefined
    again on the GPU."""
    s = make(lib, 2, 1)
    t = Trail(s, 0)
    t.enqueue(lit(1))
    assert t.send()
    execute(s)
    assert s.popAll(0) == []
    t.backtrack_to(0)
    t.enqueue(lit(0))
    s.addClause(-1, [lit(0, True), lit(1)])
    assert t.send()
    execute(s)
    assert len(s.popAll(0)) == 1


def test_many_clauses_reported_all_at_once(lib):
    """GpuSolverTest.cu:696-724: 4000 unit clauses, one assignment with every
    third variable true -> 4000 - 1334 = 2666 imports."""
    n = 4000
    s = make(lib, n, 1, gpuBlockCountGuideline=2, initReportCountPerCategory=5000)
    t = Trail(s, 0)
    for i in range(n):
        if i % 3 == 0:
            t.enqueue(lit(i))
        s.addClause(-1, [lit(i)])
    assert t.send()
    execute(s)
    got = s.popAll(0)
    assert len(got) == 2666
    assert sorted(l[0] >> 1 for l, _ in got) == [i for i in range(n) if i % 3 != 0]
    assert s.getOneSolverStat(0, "reportedClausesUnit") == 2666


def test_solver_passes_many_assignments(lib):
    """GpuSolverTest.cu:949-981: 32 assignments in one pass, clause i
    reported for assignment i only: 32 imports, no failure to send."""
    s = make(lib, 64, 3, initReportCountPerCategory=100)
    t = Trail(s, 0)
    for i in range(32):
        s.addClause(-1, [lit(2 * i, True), lit(2 * i + 1)])
        t.backtrack_to(0)
        t.enqueue(lit(2 * i))
        assert t.send()
    execute(s)
    got = s.popAll(0)
    assert len(got) == 32
    assert s.getOneSolverStat(0, "failuresToFindAssig") == 0
    # a 33rd assignment in the same window would not fit the 32-slot ring
    for i in range(32):
        assert s.trySendAssignment(1) == i
    assert s.trySendAssignment(1) == -1
    assert s.getOneSolverStat(1, "failuresToFindAssig") == 1


def test_clause_from_solver_not_reported_back(lib):
    """testSendClauseToGpu (GpuSolverTest.cu:999-1035): a clause the solver
    exported is not reported back for assignments it sent before."""
    s = make(lib, 3, 1)
    t = Trail(s, 0)
    t.enqueue(lit(0))
    assert t.send()
    s.addClause(0, [lit(0, True), lit(1, True)])
    execute(s)
    assert s.popAll(0) == []
    assert s.getGlobalStat("gpuClauses") == 1
    assert s.getGlobalStat("gpuClauseLengthSum") == 2
    assert s.getOneSolverStat(0, "reportedClauses") == 0


def test_reduce_db(lib):
    """testReduceDb (GpuSolverTest.cu:889-935): the reported (bumped) clause
    survives reduceDb, the other is removed; later clauses still work."""
    s = make(lib, 5, 1)
    s.addClause(-1, [lit(1, True), lit(3), lit(4)])
    s.addClause(-1, [lit(0, True), lit(2), lit(4)])
    t = Trail(s, 0)
    t.enqueue(lit(0), lit(4, True))
    assert t.send()
    execute(s)
    got = s.popAll(0)
    assert [tuple(l) for l, _ in got] == [(lit(0, True), lit(2), lit(4))]
    assert s.getGlobalStat("gpuClauses") == 2
    assert s.getGlobalStat("gpuClauseLengthSum") == 6
    t.enqueue(lit(2))  # the solver propagates the imported clause
    rebuilt = s.deviceCompactions()
    s.reduceDb()
    # the kept clause moved on the device (no re-upload of the database)
    assert s.deviceCompactions() == rebuilt + 1
    assert s.getGlobalStat("gpuClauses") == 1
    assert s.getGlobalStat("gpuClauseLengthSum") == 3
    assert s.getGlobalStat("gpuReduceDbs") == 1
    t.enqueue(lit(1))  # would make the removed clause one-undefined
    assert t.send()
    execute(s)
    assert s.popAll(0) == []
    rep = s.getOneSolverStat(0, "reportedClauses")
    s.addClause(-1, [lit(0, True), lit(3, True)])
    assert t.send()
    execute(s)
    assert len(s.popAll(0)) == 1
    assert s.getOneSolverStat(0, "reportedClauses") == rep + 1


def test_rejects_long_and_empty_clauses(lib):
    """HostClauses::addClause (gpuShareLib/Clauses.cu:349-351): more than 100
    literals -> -1; ids of accepted clauses increase from 0."""
    s = make(lib, 300, 1)
    assert s.addClause(-1, list(range(0, 202, 2))) == -1
    assert s.addClause(-1, list(range(0, 200, 2))) == 0
    assert s.addClause(-1, []) == -1
    assert s.addClause(-1, [lit(1)]) == 1
    s.setMaxClauseLen(256)
    assert s.addClause(-1, list(range(0, 500, 2))) == 2
    assert s.getAddedClauseCount() == 0  # counted when moved to the GPU
    s.gpuRun()
    assert s.getAddedClauseCount() == 3


def test_stat_names_and_options(lib):
    import gpusharesat_gb300 as g
    s = make(lib, 1, 1)
    assert s.getGlobalStatCount() == 13
    assert [s.getGlobalStatName(i) for i in range(13)] == g.GLOBAL_STATS
    assert s.getOneSolverStatCount() == 6
    assert [s.getOneSolverStatName(i) for i in range(6)] == g.ONE_SOLVER_STATS
    free, total = s.getGpuMemInfo()
    assert 0 < free <= total
    with pytest.raises(g.GssError):
        g.ClauseSharer(clauseActivityDecay=1.5)
    with pytest.raises(g.GssError):
        g.ClauseSharer(initReportCountPerCategory=0)


def test_current_assignment_with_deferred_unsets(lib):
    """getCurrentAssignment (GpuClauseSharerImpl.cu:238-244) and unsets that
    arrive while the ring is full (:159-176)."""
    s = make(lib, 4, 1)
    s.addClause(-1, [lit(3)])
    assert s.trySetSolverValues(0, [lit(0), lit(1, True)])
    for i in range(32):
        assert s.trySendAssignment(0) == i
    s.unsetSolverValues(0, [lit(0)])  # ring full: deferred
    assert list(s.getCurrentAssignment(0, 4)) == [2, 1, 2, 2]
    assert not s.trySetSolverValues(0, [lit(2)])
    execute(s)  # frees the ring
    assert s.trySetSolverValues(0, [lit(2)])  # applies the deferred unset first
    assert list(s.getCurrentAssignment(0, 4)) == [2, 1, 0, 2]
    assert s.getLastAssigAllReported(0) == 0
    s.popAll(0)
    assert s.getLastAssigAllReported(0) == 32


# ------------------------------------------------------ differential tests

def _random_session(lib, seed, n_vars=24, n_solvers=3, steps=400, max_len=5, variant=None):
    rng = np.random.default_rng(seed)
    s = make(lib, n_vars, n_solvers)
    if variant is not None:
        s.setVariant(*variant)
    m = SharerModel()
    m.setVarCount(n_vars)
    m.setCpuSolverCount(n_solvers)
    trails = [[] for _ in range(n_solvers)]
    popped = 0
    for step in range(steps):
        op = rng.integers(0, 100)
        sid = int(rng.integers(0, n_solvers))
        if op < 15:
            L = int(rng.integers(1, max_len + 1))
            vs = rng.choice(n_vars, size=L, replace=False)
            lits = [int(2 * v + rng.integers(0, 2)) for v in vs]
            src = int(rng.integers(-1, n_solvers))
            assert s.addClause(src, lits) == m.addClause(src, lits), step
        elif op < 40:
            free = [v for v in range(n_vars) if all((l >> 1) != v for l in trails[sid])]
            if free:
                k = min(len(free), int(rng.integers(1, 4)))
                vs = rng.choice(free, size=k, replace=False)
                lits = [int(2 * v + rng.integers(0, 2)) for v in vs]
                a, b = s.trySetSolverValues(sid, lits), m.trySetSolverValues(sid, lits)
                assert a == b, step
                if a:
                    trails[sid].extend(lits)
        elif op < 55:
            if trails[sid]:
                cut = int(rng.integers(0, len(trails[sid])))
                lits = trails[sid][cut:]
                s.unsetSolverValues(sid, lits)
                m.unsetSolverValues(sid, lits)
                del trails[sid][cut:]
        elif op < 75:
            assert s.trySendAssignment(sid) == m.trySendAssignment(sid), step
        elif op < 88:
            s.gpuRun()
            m.gpuRun()
        else:
            a = sorted((tuple(l), c) for l, c in s.popAll(sid))
            b = sorted((tuple(l), c) for l, c in m.popAll(sid))
            assert a == b, (step, a, b)
            popped += len(a)
            assert s.getLastAssigAllReported(sid) == m.getLastAssigAllReported(sid), step
        if step % 50 == 0:
            for q in range(n_solvers):
                assert list(s.getCurrentAssignment(q, n_vars)) == m.getCurrentAssignment(q), step
    for _ in range(2):
        s.gpuRun()
        m.gpuRun()
    for q in range(n_solvers):
        a = sorted((tuple(l), c) for l, c in s.popAll(q))
        b = sorted((tuple(l), c) for l, c in m.popAll(q))
        assert a == b
        popped += len(a)
        for name in ("reportedClauses", "reportedClausesUnit", "reportedClausesBinary", "assigsSentToGpu",
                     "failuresToFindAssig", "varUpdatesSentToGpu"):
            assert s.getOneSolverStat(q, name) == m.getOneSolverStat(q, name), name
    assert s.getGlobalStat("gpuRuns") == m.gpu_runs
    assert popped > 0  # the session exercised delivery


@pytest.mark.parametrize("seed", range(6))
def test_random_sessions_match_model(lib, seed):
    _random_session(lib, seed)


@pytest.mark.parametrize("n_solvers,variant", [(9, None), (33, None), (12, (0, 16, 2, 0)), (20, (2, 4, 1, 0))])
def test_random_sessions_many_solvers(lib, n_solvers, variant):
    """More solvers than one 32-slot word per lane group, other kernel variants."""
    _random_session(lib, 100 + n_solvers, n_vars=20, n_solvers=n_solvers, steps=600, max_len=4, variant=variant)


def test_many_solvers_full_rings_match_oracle(lib):
    """32 solvers x 32 random assignments in one pass over 20000 clauses: the
    first imports of every solver are exactly the (clause, solver) pairs the
    C oracle reports."""
    from gpusharesat_gb300 import workloads as W
    rng = np.random.default_rng(77)
    n_vars, n_solvers, n_cl = 3000, 32, 20000
    lengths = W.lengths_small(rng, n_cl)
    lits, offsets = W.distinct_var_clauses(rng, lengths, n_vars)
    s = make(lib, n_vars, n_solvers)
    for c in range(n_cl):
        assert s.addClause(-1, lits[offsets[c]:offsets[c + 1]].tolist()) == c
    state = np.zeros((n_vars, n_solvers, 2), np.uint32)
    for q in range(n_solvers):
        for a in range(32):
            assigned = rng.random(n_vars) < 0.7
            val = rng.random(n_vars) < 0.5
            s.unsetSolverValues(q, [2 * v for v in range(n_vars)])
            sel = np.nonzero(assigned)[0]
            assert s.trySetSolverValues(q, [int(2 * v + (0 if val[v] else 1)) for v in sel])
            assert s.trySendAssignment(q) == a
            state[sel, q, 0] |= np.uint32(1 << a)
            state[sel[val[sel]], q, 1] |= np.uint32(1 << a)
    execute(s)
    ref = oracle.check(lits, offsets, state, np.full(n_solvers, 0xFFFFFFFF, np.uint32), n_threads=8)
    want = {(int(r["word"]), int(r["clause"])) for r in ref}
    got = set()
    for q in range(n_solvers):
        for l, c in s.popAll(q):
            got.add((q, c))
            assert l == lits[offsets[c]:offsets[c + 1]].tolist()
    assert got == want
    assert s.getGlobalStat("gpuReports") == len(want)
    assert s.getGlobalStat("totalAssigClauseTested") == n_cl * 32 * n_solvers


@pytest.mark.parametrize("locality", [0, 11])
def test_range_order_reports_every_clause_with_the_solvers_literals(lib, locality):
    """With the device database in variable-range order (8 ranges of 2^11
    variables: device literals regrouped by range, clauses sorted by range)
    or in length order, an all-false assignment reports every clause, each
    handed back with its literals in the order the solver added them, and a
    reduceDb (rebuilt on the device) keeps that."""
    n_vars = 16384
    s = make(lib, n_vars, 2)
    s.setLocality(locality)
    rng = np.random.default_rng(40 + locality)
    added = {}
    for k in range(3000):
        L = int(rng.integers(1, 3))
        vs = rng.choice(n_vars, size=L, replace=False)
        cl = [lit(int(v)) for v in vs]
        added[s.addClause(-1, cl)] = cl
    s.gpuRun()  # uploads the database
    for solver in (0, 1):
        assert s.trySetSolverValues(solver, [lit(v, True) for v in range(n_vars)])
        assert s.trySendAssignment(solver) >= 0
        execute(s)
        got = {c: list(l) for l, c in s.popAll(solver)}
        assert got == added
        if solver == 0:
            s.reduceDb()  # unit and binary clauses: all kept
