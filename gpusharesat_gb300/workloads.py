"""Seeded synthetic clause databases and assignment sets.

The reference publishes no dataset for its check path; these generators stand
in for the workloads the benchmark and the parity tests run, with the shapes
and value distributions stated in each function. Everything is derived from
one ``numpy.random.Generator`` seed, so the oracle and the CUDA engine see
identical inputs.

Data layout (the engine's host-facing layout):
  lits      int32 [n_lits], lit = 2*var + sign (sign 1 = negative literal)
  offsets   int64 [n_clauses + 1] (CSR)
  state     uint32 [n_vars, n_words, 2]: (isDef, isTrue) bit planes; bit j of
            word w is assignment slot 32*w + j
  start     uint32 [n_words]: the slots of each word that hold a sent assignment
  solver_of_word int32 [n_words]
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    n_vars: int
    lits: np.ndarray
    offsets: np.ndarray
    state: np.ndarray
    start: np.ndarray
    solver_of_word: np.ndarray
    n_solvers: int
    planted: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))

    @property
    def n_clauses(self):
        return int(self.offsets.shape[0] - 1)

    @property
    def n_words(self):
        return int(self.state.shape[1])

    @property
    def n_assignments(self):
        return int(sum(bin(int(m)).count("1") for m in self.start))

    @property
    def n_lits(self):
        return int(self.lits.shape[0])


def _truncated_geometric(rng, n, lo, hi, mean):
    """Integers in [lo, hi]: lo + Geometric with the given mean of (L - lo),
    conditioned on L <= hi (resampled)."""
    p = 1.0 / (mean - lo + 1.0)
    out = lo + rng.geometric(p, size=n) - 1
    bad = out > hi
    while bad.any():
        out[bad] = lo + rng.geometric(p, size=int(bad.sum())) - 1
        bad = out > hi
    return out.astype(np.int64)


def lengths_small(rng, n):
    """Clause lengths 2..30, geometric with mean 8 (truncated)."""
    return _truncated_geometric(rng, n, 2, 30, 8.0)


def lengths_scale(rng, n):
    """Clause lengths 2..100: 60% uniform on 2..16, 40% a geometric tail on
    17..100 whose offset above 16 has mean 16 (truncated at 100)."""
    tail = rng.random(n) >= 0.6
    out = rng.integers(2, 17, size=n).astype(np.int64)
    nt = int(tail.sum())
    out[tail] = _truncated_geometric(rng, nt, 17, 100, 32.0)
    return out


def lengths_zipf(rng, n, cap=256, a=1.2):
    """Clause lengths >= 1 from Zipf(a), capped (resampled) at cap."""
    out = rng.zipf(a, size=n)
    bad = out > cap
    while bad.any():
        out[bad] = rng.zipf(a, size=int(bad.sum()))
        bad = out > cap
    return out.astype(np.int64)


def distinct_var_clauses(rng, lengths, n_vars):
    """Random clauses: distinct variables chosen uniformly, fair-coin signs.
    Returns (lits int32, offsets int64)."""
    lengths = np.asarray(lengths, dtype=np.int64)
    n = lengths.shape[0]
    offsets = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    if int(lengths.max(initial=0)) > n_vars:
        raise ValueError("a clause is longer than the number of variables")
    var = rng.integers(0, n_vars, size=int(offsets[-1]), dtype=np.int64)
    # Re-draw repeated variables (only the repeats), one length class at a time.
    for L in np.unique(lengths):
        L = int(L)
        if L < 2:
            continue
        ids = np.nonzero(lengths == L)[0]
        while ids.size:
            rows = offsets[ids][:, None] + np.arange(L)[None, :]
            vals = var[rows]
            order = np.argsort(vals, axis=1, kind="stable")
            s = np.take_along_axis(vals, order, axis=1)
            dup_sorted = s[:, 1:] == s[:, :-1]
            has = dup_sorted.any(axis=1)
            if not has.any():
                break
            r, j = np.nonzero(dup_sorted)
            pos = rows[r, order[r, j + 1]]
            var[pos] = rng.integers(0, n_vars, size=pos.shape[0], dtype=np.int64)
            ids = ids[has]
    sign = rng.integers(0, 2, size=var.shape[0], dtype=np.int64)
    lits = (2 * var + sign).astype(np.int32)
    return lits, offsets


def random_state(rng, n_vars, n_words, assigned_frac):
    """Bit planes for 32*n_words assignment slots. Slot a assigns each
    variable independently with probability assigned_frac[a]; values are a
    fair coin (isTrue bits of unassigned variables are random too: the rule
    must ignore them)."""
    assigned_frac = np.asarray(assigned_frac, dtype=np.float64)
    state = np.empty((n_vars, n_words, 2), dtype=np.uint32)
    for w in range(n_words):
        thr = np.round(assigned_frac[32 * w: 32 * w + 32] * 65536.0).astype(np.uint32)
        r = rng.integers(0, 65536, size=(n_vars, 32), dtype=np.uint32)
        bits = (r < thr[None, :]).astype(np.uint8)
        packed = np.packbits(bits, axis=1, bitorder="little")
        state[:, w, 0] = packed.view("<u4").reshape(n_vars)
        state[:, w, 1] = rng.integers(0, 2 ** 32, size=n_vars, dtype=np.uint32)
    return state


def plant_reports(rng, lits, offsets, state, start, rate):
    """Plants reports in a fraction `rate` of clauses: pick a started slot a,
    make every literal but the last false under a, and make the last literal
    false (half of the planted clauses), unassigned (a quarter) or true (a
    quarter, a negative control that must not report for a). Variables are
    re-drawn where needed so the clause keeps distinct variables.
    Modifies lits in place; returns the planted clause indices."""
    n_clauses = offsets.shape[0] - 1
    n_vars = state.shape[0]
    n_plant = int(round(n_clauses * rate))
    if n_plant == 0:
        return np.zeros(0, dtype=np.int64)
    chosen = np.sort(rng.choice(n_clauses, size=n_plant, replace=False))
    started = [(w, b) for w in range(state.shape[1]) for b in range(32) if (int(start[w]) >> b) & 1]
    for c in chosen:
        b0, b1 = int(offsets[c]), int(offsets[c + 1])
        L = b1 - b0
        w, bit = started[int(rng.integers(0, len(started)))]
        kind = int(rng.integers(0, 4))  # 0,1: last false; 2: last undef; 3: last true
        used = set()
        new = []
        for i in range(L):
            want_undef = (i == L - 1 and kind == 2)
            while True:
                v = int(rng.integers(0, n_vars))
                if v in used:
                    continue
                d = (int(state[v, w, 0]) >> bit) & 1
                if want_undef and d == 0:
                    break
                if not want_undef and d == 1:
                    break
            used.add(v)
            t = (int(state[v, w, 1]) >> bit) & 1
            if want_undef:
                sign = int(rng.integers(0, 2))
            elif i == L - 1 and kind == 3:
                sign = 1 - t  # literal true: positive literal of a true variable
            else:
                sign = t  # literal false: positive literal of a false variable
            new.append(2 * v + sign)
        lits[b0:b1] = np.asarray(new, dtype=np.int32)
    return chosen


def make_small(seed=0, n_vars=2 ** 14, n_clauses=100_000, plant_rate=0.01):
    """Plain check, small: 2^14 variables; 1e5 clauses with lengths 2..30
    (geometric, mean 8); one solver sends 64 partial assignments, each
    assigning a uniform 60% of the variables with fair-coin values; 1% of
    the clauses carry planted reports."""
    rng = np.random.default_rng(seed)
    lengths = lengths_small(rng, n_clauses)
    lits, offsets = distinct_var_clauses(rng, lengths, n_vars)
    n_words = 2
    state = random_state(rng, n_vars, n_words, np.full(32 * n_words, 0.6))
    start = np.full(n_words, 0xFFFFFFFF, dtype=np.uint32)
    planted = plant_reports(rng, lits, offsets, state, start, plant_rate)
    return Workload("plain-small", n_vars, lits, offsets, state, start,
                    np.zeros(n_words, dtype=np.int32), 1, planted)


def make_scale(seed=1, n_vars=2 ** 20, n_clauses=4_000_000, n_solvers=32, plant_rate=0.001):
    """Plain check at scale: 2^20 variables; 4e6 clauses with lengths 2..100
    (60% uniform on 2..16, 40% geometric tail); 32 solvers x 32 partial
    assignments = 1024 slots, each assigning a uniform 40-90% of the
    variables with fair signs; 0.1% planted reports. One 32-slot word per
    solver."""
    rng = np.random.default_rng(seed)
    lengths = lengths_scale(rng, n_clauses)
    lits, offsets = distinct_var_clauses(rng, lengths, n_vars)
    n_words = n_solvers
    frac = rng.uniform(0.4, 0.9, size=32 * n_words)
    state = random_state(rng, n_vars, n_words, frac)
    start = np.full(n_words, 0xFFFFFFFF, dtype=np.uint32)
    planted = plant_reports(rng, lits, offsets, state, start, plant_rate)
    return Workload("plain-scale", n_vars, lits, offsets, state, start,
                    np.arange(n_words, dtype=np.int32), n_solvers, planted)


def lengths_batching(rng, n, cap=256, a=1.2):
    """Clause lengths 1 + Zipf(a), at most cap. The shift by one keeps the
    Zipf shape while leaving out unit clauses (solvers keep units on their
    trail), which would otherwise report under almost every assignment."""
    return 1 + lengths_zipf(rng, n, cap=cap - 1, a=a)


def batch_starts(rng, n_solvers, lo=4, hi=64):
    """Started-slot masks for one pass of uneven batches: solver s sends
    U[lo, hi] assignments, laid out in its two 32-slot words 2s and 2s+1.
    Returns (start uint32[2 * n_solvers], batch sizes)."""
    sizes = rng.integers(lo, hi + 1, size=n_solvers)
    start = np.zeros(2 * n_solvers, dtype=np.uint32)
    for s, b in enumerate(sizes):
        b0, b1 = min(int(b), 32), max(int(b) - 32, 0)
        start[2 * s] = np.uint32((1 << b0) - 1) if b0 < 32 else np.uint32(0xFFFFFFFF)
        start[2 * s + 1] = np.uint32((1 << b1) - 1)
    return start, sizes


def make_batching(seed=2, n_vars=2 ** 20, n_clauses=8_000_000, n_solvers=48, plant_rate=0.0005):
    """Batching, uneven: 2^20 variables; 8e6 clauses with lengths 1 + Zipf(1.2)
    capped at 256; 48 solvers with two 32-slot words each (up to 64
    assignments per pass), each assignment assigning a uniform 40-90% of the
    variables with fair signs; 0.05% planted reports. The batch sizes (started
    slots) are drawn per pass with batch_starts."""
    rng = np.random.default_rng(seed)
    lengths = lengths_batching(rng, n_clauses)
    lits, offsets = distinct_var_clauses(rng, lengths, n_vars)
    n_words = 2 * n_solvers
    frac = rng.uniform(0.4, 0.9, size=32 * n_words)
    state = random_state(rng, n_vars, n_words, frac)
    start = np.full(n_words, 0xFFFFFFFF, dtype=np.uint32)
    planted = plant_reports(rng, lits, offsets, state, start, plant_rate)
    return Workload("batching", n_vars, lits, offsets, state, start,
                    (np.arange(n_words) // 2).astype(np.int32), n_solvers, planted)


def churn_batch(rng, n_vars, n_new):
    """New clauses of a churn step, from the small workload's generator
    (lengths 2..30, geometric mean 8)."""
    return distinct_var_clauses(rng, lengths_small(rng, n_new), n_vars)


def model_clauses(rng, lengths, n_vars, model):
    """Clauses over a hidden total assignment `model` (uint8 per variable,
    1 = true): distinct variables, at least two literals true under the
    model, each other literal false under it with probability 1/2. Under an
    assignment that agrees with the model such a clause has a true or two
    unassigned literals, so it never reports unless planted."""
    lits, offsets = distinct_var_clauses(rng, lengths, n_vars)
    var = lits.astype(np.int64) >> 1
    m_true = rng.random(var.shape[0]) < 0.5
    lengths = np.diff(offsets)
    # two forced model-true literals per clause, at distinct random positions
    p0 = (rng.random(lengths.shape[0]) * lengths).astype(np.int64)
    p1 = (p0 + 1 + (rng.random(lengths.shape[0]) * (lengths - 1)).astype(np.int64)) % np.maximum(lengths, 1)
    m_true[offsets[:-1] + p0] = True
    m_true[offsets[:-1] + p1] = True
    true_sign = 1 - model[var].astype(np.int64)  # sign of the model-true literal
    sign = np.where(m_true, true_sign, 1 - true_sign)
    return (2 * var + sign).astype(np.int32), offsets


def make_learned(seed=4, n_vars=2 ** 21, n_clauses=4_000_000, n_words=64, stream=0, assigned=0.5):
    """Learned scan order: a pool of n_clauses + stream clauses (the first
    n_clauses are the database at the start, the rest arrive in order), with
    lengths 1 + Zipf(1.2) capped at 256 over a hidden model; each clause has
    a latent report rate r ~ Beta(0.5, 20) and LBD = round(length * U) with
    U in [0.3, 1] falling with r (U = 0.3 + 0.7 * clip(1 - 10 r + 0.15 N(0,1))).
    The base state: n_words words of 32 slots, each slot assigning each
    variable with probability `assigned`, always to its model value, so no
    clause reports unless planted (gss_bench_plant plants clause c at rate
    r_c). Returns a dict of numpy arrays."""
    rng = np.random.default_rng(seed)
    total = n_clauses + stream
    model = rng.integers(0, 2, size=n_vars).astype(np.uint8)
    lengths = lengths_batching(rng, total)
    lits, offsets = model_clauses(rng, lengths, n_vars, model)
    r = rng.beta(0.5, 20, size=total).astype(np.float32)
    u = np.clip(1 - 10 * r + 0.15 * rng.standard_normal(total), 0, 1)
    lens = np.diff(offsets)
    lbd = np.maximum(1, np.round(lens * (0.3 + 0.7 * u))).astype(np.uint16)
    state = np.empty((n_vars, n_words, 2), dtype=np.uint32)
    thr = np.uint32(int(assigned * 65536))
    for w in range(n_words):
        bits = (rng.integers(0, 65536, size=(n_vars, 32), dtype=np.uint32) < thr).astype(np.uint8)
        state[:, w, 0] = np.packbits(bits, axis=1, bitorder="little").view("<u4").reshape(n_vars)
    state[:, :, 1] = np.where(model[:, None] == 1, np.uint32(0xFFFFFFFF), np.uint32(0))
    return {"lits": lits, "offsets": offsets, "rate": r, "lbd": lbd, "state": state, "model": model,
            "n_vars": n_vars, "n_words": n_words, "n_clauses": n_clauses, "stream": stream}


# ---- dump format shared by the harnesses ----
#
# One .npz file per workload: the arrays of Workload (lits, offsets, state,
# start, solver_of_word, planted) plus its name, variable count and solver
# count. The oracle, the engine, bench.py and the tests can all load it.

def save(wl, path):
    """Writes a Workload to `path` (.npz)."""
    np.savez(path, name=np.array(wl.name), n_vars=np.int64(wl.n_vars), n_solvers=np.int64(wl.n_solvers),
             lits=wl.lits, offsets=wl.offsets, state=wl.state, start=wl.start,
             solver_of_word=wl.solver_of_word, planted=wl.planted)


def load(path):
    """Reads a Workload written by save()."""
    with np.load(path, allow_pickle=False) as z:
        return Workload(str(z["name"]), int(z["n_vars"]), z["lits"], z["offsets"], z["state"], z["start"],
                        z["solver_of_word"], int(z["n_solvers"]), z["planted"])


MAKERS = {"small": make_small, "scale": make_scale, "batching": make_batching}


def main(argv=None):
    """python -m gpusharesat_gb300.workloads {small|scale|batching} OUT.npz [--clauses N] [--seed S]"""
    import argparse
    p = argparse.ArgumentParser()
    p.add_argument("workload", choices=sorted(MAKERS))
    p.add_argument("out")
    p.add_argument("--clauses", type=int, default=None)
    p.add_argument("--seed", type=int, default=None)
    args = p.parse_args(argv)
    kw = {}
    if args.clauses is not None:
        kw["n_clauses"] = args.clauses
    if args.seed is not None:
        kw["seed"] = args.seed
    wl = MAKERS[args.workload](**kw)
    save(wl, args.out)
    print("%s: %d clauses, %d literals, %d variables, %d words -> %s"
          % (wl.name, wl.n_clauses, wl.n_lits, wl.n_vars, wl.n_words, args.out))


if __name__ == "__main__":
    main()
