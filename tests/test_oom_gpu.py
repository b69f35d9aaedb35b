"""Out-of-memory recovery of the pass driver, as GpuRunner::wholeRun does it
(gpuShareLib/GpuRunner.cu:243-260): when a device buffer cannot grow, the
clause database is reduced (reduceDb), hasRunOutOfGpuMemoryOnce becomes
true, and the pass still runs with the assignments already cut.

The allocation failure is injected on the host (gss_debug_fail_device_alloc
makes the library's next large cudaMalloc report out-of-memory without
calling it), so no GPU fault is involved. Clauses here have one or two
literals, which reduceDb always keeps (Clauses.cu:249-282 only drops clauses
of length 3 and more), so every reported set is known exactly."""
import numpy as np
import pytest

from oracle.sharer_model import SharerModel

pytestmark = pytest.mark.gpu


def lit(v, neg=False):
    return 2 * v + (1 if neg else 0)


def _sharer(n_vars, n_solvers):
    import gpusharesat_gb300 as g
    s = g.ClauseSharer(minGpuLatencyMicros=0, verbosity=0)
    s.setVarCount(n_vars)
    s.setCpuSolverCount(n_solvers)
    return s


def _all_false(s, solver, n_vars):
    assert s.trySetSolverValues(solver, [lit(v, True) for v in range(n_vars)])
    assert s.trySendAssignment(solver) >= 0


def test_append_out_of_memory_reduces_and_runs(lib):
    """The database's literal buffer cannot grow for a large batch: the pass
    reduces the database, uploads it again and runs; every clause still
    reports under an all-false assignment."""
    import gpusharesat_gb300 as g
    n_vars = 40000
    s = _sharer(n_vars, 2)
    try:
        for k in range(2000):
            s.addClause(-1, [lit(2 * k), lit(2 * k + 1)])
        s.gpuRun()
        s.gpuRun()
        assert not s.hasRunOutOfGpuMemoryOnce()
        for k in range(2000, 20000):
            s.addClause(-1, [lit(2 * k), lit(2 * k + 1)])
        # the literal buffer grows from 16 KB to 256 KB: that allocation fails
        g.debug_fail_device_alloc(200_000, 1)
        _all_false(s, 1, n_vars)
        s.gpuRun()
        s.gpuRun()
        assert s.hasRunOutOfGpuMemoryOnce()
        assert s.getGlobalStat(7) >= 1  # gpuReduceDbs
        got = sorted(c for _, c in s.popAll(1))
        assert got == list(range(20000))
    finally:
        g.debug_fail_device_alloc(0, 0)
        s.close()


def test_update_buffer_out_of_memory_keeps_the_cut_assignments(lib):
    """The buffer of variable updates cannot grow after the solvers' rings
    were cut: the database is reduced and the same updates are sent, so the
    assignment is checked and reported in that pass (no assignment lost)."""
    import gpusharesat_gb300 as g
    n_vars = 30000
    s = _sharer(n_vars, 2)
    try:
        for k in range(n_vars // 2):
            s.addClause(-1, [lit(2 * k), lit(2 * k + 1)])
        s.gpuRun()
        s.gpuRun()
        # 30000 updates x 16 bytes: the update buffer needs 512 KB
        g.debug_fail_device_alloc(400_000, 1)
        _all_false(s, 0, n_vars)
        s.gpuRun()
        s.gpuRun()
        assert s.hasRunOutOfGpuMemoryOnce()
        assert sorted(c for _, c in s.popAll(0)) == list(range(n_vars // 2))
        assert s.getLastAssigAllReported(0) == 1
    finally:
        g.debug_fail_device_alloc(0, 0)
        s.close()


@pytest.mark.parametrize("seed", [0, 1])
def test_sessions_with_injected_failures_match_model(lib, seed):
    """A random session of unit and binary clauses, assignments and passes,
    compared with the plain-Python model of the API after every pass, with
    an allocation failure injected before some of the passes."""
    import gpusharesat_gb300 as g
    n_vars = 64
    s = g.ClauseSharer(minGpuLatencyMicros=0, verbosity=0)
    m = SharerModel()
    rng = np.random.default_rng(seed)
    try:
        for x in (s, m):
            x.setVarCount(n_vars)
            x.setCpuSolverCount(3)
        trails = [[] for _ in range(3)]
        for step in range(30):
            for _ in range(int(rng.integers(0, 200))):
                L = int(rng.integers(1, 3))
                vs = rng.choice(n_vars, size=L, replace=False)
                cl = [lit(int(v), bool(rng.integers(0, 2))) for v in vs]
                assert s.addClause(-1, cl) == m.addClause(-1, cl)
            for solver in range(3):
                tr = trails[solver]
                k = int(rng.integers(0, len(tr) + 1))
                if len(tr) > k:
                    s.unsetSolverValues(solver, tr[k:])
                    m.unsetSolverValues(solver, tr[k:])
                    del tr[k:]
                free = [v for v in range(n_vars) if all((l >> 1) != v for l in tr)]
                add = [lit(int(v), bool(rng.integers(0, 2)))
                       for v in rng.choice(free, size=min(4, len(free)), replace=False)]
                assert s.trySetSolverValues(solver, add) and m.trySetSolverValues(solver, add)
                tr.extend(add)
                assert s.trySendAssignment(solver) == m.trySendAssignment(solver)
            if step % 4 == 1:
                g.debug_fail_device_alloc(0, 1)  # the next device allocation of any size fails
            for x in (s, m):
                x.gpuRun()
                x.gpuRun()
            g.debug_fail_device_alloc(0, 0)
            for solver in range(3):
                got = sorted((tuple(l), c) for l, c in s.popAll(solver))
                assert got == sorted((tuple(l), c) for l, c in m.popAll(solver)), (step, solver)
                assert s.getLastAssigAllReported(solver) == m.getLastAssigAllReported(solver)
        assert s.hasRunOutOfGpuMemoryOnce()
    finally:
        g.debug_fail_device_alloc(0, 0)
        s.close()
