"""The serving loop on the GPU: the HBM clause budget with oldest-unreported
eviction, device-side compaction, reports that are the same for a solver
alone and in a mix of solvers, and a short run of the load generator.

Clauses here are binary (x_a | x_b) with positive literals, so a solver that
sets both variables false gets the clause reported, and one that assigns
neither does not (two undefined literals)."""
import numpy as np
import pytest

from oracle.sharer_model import SharerModel

pytestmark = pytest.mark.gpu

GPU_CLAUSES = 0  # GlobalStats index of gpuClauses (live clauses)


def lit(v, neg=False):
    return 2 * v + (1 if neg else 0)


def make(n_vars, n_solvers, budget):
    import gpusharesat_gb300 as g
    s = g.ClauseSharer(minGpuLatencyMicros=0, verbosity=0)
    s.setVarCount(n_vars)
    s.setCpuSolverCount(n_solvers)
    s.setClauseBudget(budget)
    return s


def execute(s):
    s.gpuRun()
    s.gpuRun()


def popped_ids(s, solver):
    return sorted(cid for _, cid in s.popAll(solver))


def all_false(s, solver, n_vars):
    """Sends one assignment of `solver` with every variable false."""
    assert s.trySetSolverValues(solver, [lit(v, True) for v in range(n_vars)])
    assert s.trySendAssignment(solver) >= 0


def test_budget_keeps_recently_reported(lib):
    n_vars = 400
    s = make(n_vars, 2, budget=100)
    # ids 0..4: hot, reported to solver 0; ids 5..99: cold
    ids = [s.addClause(-1, [lit(0), lit(1 + k)]) for k in range(5)]
    ids += [s.addClause(-1, [lit(10 + 2 * k), lit(11 + 2 * k)]) for k in range(95)]
    assert ids == list(range(100))
    assert s.trySetSolverValues(0, [lit(v, True) for v in range(6)])
    assert s.trySendAssignment(0) == 0
    execute(s)
    assert popped_ids(s, 0) == [0, 1, 2, 3, 4]
    assert s.evictedCount() == 0
    # 50 more cold clauses: the 50 oldest unreported ones (5..54) go
    ids = [s.addClause(-1, [lit(200 + 2 * k), lit(201 + 2 * k)]) for k in range(50)]
    assert ids == list(range(100, 150))
    all_false(s, 1, n_vars)
    execute(s)
    assert s.evictedCount() == 50
    assert s.getGlobalStat(GPU_CLAUSES) == 100
    assert popped_ids(s, 1) == [0, 1, 2, 3, 4] + list(range(55, 150))


def test_budget_takes_recent_when_it_must(lib):
    n_vars = 64
    s = make(n_vars, 2, budget=3)
    for k in range(5):
        s.addClause(-1, [lit(0), lit(1 + k)])
    # the budget applies at the first pass already: ids 0, 1 go (oldest)
    assert s.trySetSolverValues(0, [lit(v, True) for v in range(6)])
    assert s.trySendAssignment(0) == 0
    execute(s)
    assert s.evictedCount() == 2
    assert popped_ids(s, 0) == [2, 3, 4]
    # budget 1 and 5 cold clauses: round one takes the cold ones (never
    # reported), round two the two oldest of the recently reported ones
    s.setClauseBudget(1)
    for k in range(5):
        s.addClause(-1, [lit(20 + 2 * k), lit(21 + 2 * k)])
    all_false(s, 1, n_vars)
    execute(s)
    assert s.evictedCount() == 2 + 7
    assert popped_ids(s, 1) == [4]


def test_eviction_with_device_compaction_matches_model(lib):
    """Many passes of clause churn under a budget: the device database is
    compacted on the GPU several times; at the end an all-false assignment
    must report exactly the newest `budget` clauses (nothing was reported
    before, so eviction is oldest first)."""
    n_vars = 3000
    budget = 1000
    s = make(n_vars, 2, budget)
    rng = np.random.default_rng(3)
    next_id = 0
    assert s.trySetSolverValues(0, [lit(0)])  # x0 true: no clause reports for solver 0
    for step in range(12):
        for _ in range(300 if step else 1000):
            a, b = rng.choice(n_vars, size=2, replace=False)
            assert s.addClause(-1, [lit(int(a)), lit(int(b))]) == next_id
            next_id += 1
        assert s.trySendAssignment(0) >= 0
        execute(s)
        assert s.getGlobalStat(GPU_CLAUSES) == budget
    assert s.deviceCompactions() >= 2
    assert s.evictedCount() == next_id - budget
    all_false(s, 1, n_vars)
    execute(s)
    assert popped_ids(s, 1) == list(range(next_id - budget, next_id))


def _session(lib, n_mix, seed, n_vars=48, steps=60):
    """Solver 0 runs the same seeded sequence of assignments; n_mix other
    solvers send their own random assignments in the same passes. Every call
    also goes to the plain-Python model of the API, and solver 0's imports
    are compared with the model's after each pass. Returns what solver 0
    popped after each pass."""
    import gpusharesat_gb300 as g
    s = g.ClauseSharer(minGpuLatencyMicros=0, verbosity=0)
    m = SharerModel()
    for x in (s, m):
        x.setVarCount(n_vars)
        x.setCpuSolverCount(1 + n_mix)
    db = np.random.default_rng(1000 + seed)
    for _ in range(400):
        L = int(db.integers(1, 5))
        vs = db.choice(n_vars, size=L, replace=False)
        cl = [lit(int(v), bool(db.integers(0, 2))) for v in vs]
        assert s.addClause(-1, cl) == m.addClause(-1, cl)
    r0 = np.random.default_rng(seed)
    rm = np.random.default_rng(seed + 77)
    trails = [[] for _ in range(1 + n_mix)]
    out = []
    for step in range(steps):
        for solver in range(1 + n_mix):
            r = r0 if solver == 0 else rm
            tr = trails[solver]
            k = int(r.integers(0, len(tr) + 1))
            if len(tr) > k:
                s.unsetSolverValues(solver, tr[k:])
                m.unsetSolverValues(solver, tr[k:])
                del tr[k:]
            free = [v for v in range(n_vars) if all((l >> 1) != v for l in tr)]
            add = [lit(int(v), bool(r.integers(0, 2))) for v in r.choice(free, size=min(3, len(free)), replace=False)]
            assert s.trySetSolverValues(solver, add) and m.trySetSolverValues(solver, add)
            tr.extend(add)
            assert s.trySendAssignment(solver) == m.trySendAssignment(solver) >= 0
        for x in (s, m):
            x.gpuRun()
            x.gpuRun()
        got = sorted((tuple(l), c) for l, c in s.popAll(0))
        assert got == sorted((tuple(l), c) for l, c in m.popAll(0)), step
        for solver in range(1, 1 + n_mix):
            s.popAll(solver)
            m.popAll(solver)
        done = s.getLastAssigAllReported(0)
        assert done == m.getLastAssigAllReported(0) == step + 1
        out.append(([c for _, c in got], done))
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_reports_same_alone_and_in_the_mix(lib, seed):
    """Solver 0's imports, pass by pass, are the same whether it is served
    alone or with 31 other solvers in the same passes (and the model's)."""
    alone = _session(lib, 0, seed)
    mixed = _session(lib, 31, seed)
    assert alone == mixed
    assert sum(len(ids) for ids, _ in alone) > 0


def test_serving_generator_short_run(lib):
    import gpusharesat_gb300 as g
    r = g.serving_run(seconds=2.0, warmup_seconds=0.5, assign_rate=2e4, n_solvers=16, n_vars=2 ** 16,
                      budget=150_000, initial_clauses=140_000, clause_rate=1e5, plant_rate=0.01, batch_max=16,
                      trail_fraction=0.3, trail_change=4, seed=3)
    assert r["assignments"] > 1000
    assert 0 < r["p50_ms"] <= r["p99_ms"] <= r["p999_ms"] <= r["max_ms"]
    assert r["passes"] > 10
    assert r["checks_per_s"] > 0
    assert r["evicted"] > 0
    assert r["live_clauses_end"] <= 150_000
    assert r["reports_popped"] > 0


def test_reduce_db_after_evictions(lib):
    """A reduceDb on a database with evicted clauses drops the tombstones:
    the clause count stays the live count, evicted clauses stay gone, and
    the clauses it keeps still report."""
    n_vars = 2000
    s = make(n_vars, 2, budget=300)
    for k in range(500):
        s.addClause(-1, [lit(2 * k), lit(2 * k + 1)])  # binary: reduceDb keeps them all
    assert s.trySetSolverValues(0, [lit(0)]) and s.trySendAssignment(0) >= 0
    execute(s)
    assert s.evictedCount() == 200 and s.getGlobalStat(GPU_CLAUSES) == 300
    rebuilt = s.deviceCompactions()
    s.reduceDb()
    assert s.deviceCompactions() == rebuilt + 1  # rebuilt on the device, evicted clauses dropped
    assert s.getGlobalStat(GPU_CLAUSES) == 300
    all_false(s, 1, n_vars)
    execute(s)
    assert popped_ids(s, 1) == list(range(200, 500))
