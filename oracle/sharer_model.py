"""Plain-Python model of the GpuClauseSharer API semantics (test oracle).

TEST INFRASTRUCTURE ONLY: the parity tests drive the CUDA-backed sharer and
this model with the same calls and compare what they return. Pure-Python
loops, for small cases.

It states the semantics directly rather than through the reference's bit
machinery: an assignment is a snapshot of the solver's values taken when
trySendAssignment succeeds (what OneSolverAssigs::setVarLocked /
copyUpdatesLocked implement with 32 slots, gpuShareLib/Assigs.cu:163-300),
every clause on the GPU at the cut of a pass is checked against every
assignment of that pass with the rule of gpuShareLib/GpuRunner.cu:34-57, and
the results of a pass are delivered by the next gpuRun. Delivery restates
Reported::fill / popReportedClause (gpuShareLib/Reported.cu:97-204) and the
deferred unsets of GpuClauseSharerImpl.cu:130-191. reduceDb is not modelled.
"""
from collections import deque

TRUE, FALSE, UNDEF = 0, 1, 2
SLOTS = 32


def reports(lits, vals):
    """The report rule for one clause under one assignment."""
    n_false = n_undef = 0
    for lit in lits:
        v = vals[lit >> 1] if (lit >> 1) < len(vals) else UNDEF
        if v == UNDEF:
            n_undef += 1
        elif (v == TRUE) == bool(lit & 1):  # negative literal of a true var, positive of a false one
            n_false += 1
    return n_false == len(lits) or (n_false == len(lits) - 1 and n_undef == 1)


class _Solver:
    def __init__(self, n_vars):
        self.vals = [UNDEF] * n_vars
        self.current_id = 0
        self.first_id_used = 0
        self.snapshots = []   # (id, values) sent since the last cut
        self.to_unset = []
        # delivery
        self.batches = deque()  # [assig_start, assig_count, [(id, lits)], next, which_knows]
        self.inter = 0          # batches[:inter] consumed (kept), batches[inter:] ready
        self.current = None
        self.not_again = set()
        self.dont_import = deque()
        self.last_sent = 0
        self.last_all = 0
        self.stats = {"varUpdatesSentToGpu": 0, "assigsSentToGpu": 0, "failuresToFindAssig": 0,
                      "reportedClauses": 0, "reportedClausesUnit": 0, "reportedClausesBinary": 0}

    def full(self):
        return self.current_id == self.first_id_used + SLOTS


class SharerModel:
    def __init__(self, max_len=100):
        self.max_len = max_len
        self.n_vars = 0
        self.solvers = [_Solver(0)]
        self.next_id = 0
        self.staged = []
        self.db = []
        self.pending = None
        self.gpu_runs = 0

    # --- setup ---
    def setVarCount(self, n):
        for s in self.solvers:
            if len(s.vals) < n:
                s.vals.extend([UNDEF] * (n - len(s.vals)))
        self.n_vars = max(self.n_vars, n)

    def setCpuSolverCount(self, n):
        while len(self.solvers) < n:
            self.solvers.append(_Solver(self.n_vars))

    # --- clause export ---
    def addClause(self, solver, lits):
        if len(lits) < 1 or len(lits) > self.max_len or solver >= len(self.solvers):
            return -1
        cid = self.next_id
        self.next_id += 1
        self.staged.append((cid, list(lits)))
        if solver >= 0:
            s = self.solvers[solver]
            s.not_again.add(cid)
            s.dont_import.append((cid, s.last_sent + 1))
        return cid

    # --- assignments ---
    def _unset_pending(self, s):
        for lit in s.to_unset:
            if (lit >> 1) < len(s.vals):
                s.vals[lit >> 1] = UNDEF
        s.stats["varUpdatesSentToGpu"] += len(s.to_unset)
        s.to_unset = []

    def trySetSolverValues(self, solver, lits):
        s = self.solvers[solver]
        if s.full():
            s.stats["failuresToFindAssig"] += 1
            return False
        self._unset_pending(s)
        for lit in lits:
            if (lit >> 1) < len(s.vals):
                s.vals[lit >> 1] = FALSE if lit & 1 else TRUE
        s.stats["varUpdatesSentToGpu"] += len(lits)
        return True

    def unsetSolverValues(self, solver, lits):
        s = self.solvers[solver]
        if not s.full():
            self._unset_pending(s)
            for lit in lits:
                if (lit >> 1) < len(s.vals):
                    s.vals[lit >> 1] = UNDEF
            s.stats["varUpdatesSentToGpu"] += len(lits)
        else:
            s.to_unset.extend(lits)

    def trySendAssignment(self, solver):
        s = self.solvers[solver]
        if s.full():
            s.stats["failuresToFindAssig"] += 1
            return -1
        aid = s.current_id
        s.snapshots.append((aid, list(s.vals)))
        s.current_id += 1
        s.stats["assigsSentToGpu"] += 1
        s.last_sent = aid
        return aid

    def getCurrentAssignment(self, solver):
        s = self.solvers[solver]
        out = list(s.vals)
        for lit in s.to_unset:
            if (lit >> 1) < len(out):
                out[lit >> 1] = UNDEF
        return out

    # --- passes ---
    def gpuRun(self):
        if self.pending is not None:
            self._gather()
        self._launch()

    def _launch(self):
        self.db.extend(self.staged)
        self.staged = []
        if not self.db:
            return
        per_solver = []
        for s in self.solvers:
            per_solver.append((s.first_id_used, s.current_id - s.first_id_used, s.snapshots))
            s.snapshots = []
            s.first_id_used = s.current_id
        self.pending = (per_solver, list(self.db))

    def _gather(self):
        per_solver, db = self.pending
        self.pending = None
        self.gpu_runs += 1
        for si, (start, count, snaps) in enumerate(per_solver):
            hits = [(cid, lits) for cid, lits in db if any(reports(lits, vals) for _, vals in snaps)]
            if count > 0 or hits:
                self.solvers[si].batches.append([start, count, hits, 0, 0])

    # --- import ---
    def popReportedClause(self, solver):
        s = self.solvers[solver]
        while True:
            if s.current is None:
                if s.inter < len(s.batches):
                    s.current = s.batches[s.inter]
                    s.inter += 1
                else:
                    return None
            b = s.current
            while b[3] < len(b[2]):
                cid, lits = b[2][b[3]]
                b[3] += 1
                if cid not in s.not_again:
                    s.not_again.add(cid)
                    s.stats["reportedClauses"] += 1
                    if len(lits) == 1:
                        s.stats["reportedClausesUnit"] += 1
                    if len(lits) == 2:
                        s.stats["reportedClausesBinary"] += 1
                    return list(lits), cid
            b[4] = s.last_sent + 1
            seen_until = b[0] + b[1]
            while s.inter > 0 and s.batches[0][4] <= seen_until:
                old = s.batches.popleft()
                s.inter -= 1
                for cid, _ in old[2]:
                    s.not_again.discard(cid)
            while s.dont_import and s.dont_import[0][1] < seen_until:
                s.not_again.discard(s.dont_import.popleft()[0])
            s.last_all = seen_until
            s.current = None

    def popAll(self, solver):
        out = []
        while True:
            r = self.popReportedClause(solver)
            if r is None:
                return out
            out.append(r)

    def getLastAssigAllReported(self, solver):
        return self.solvers[solver].last_all

    def getOneSolverStat(self, solver, name):
        return self.solvers[solver].stats[name]
