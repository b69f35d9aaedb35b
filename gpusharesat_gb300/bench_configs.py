"""Measurements of the batching, serving and learned-order workloads.

bench.py measures the headline (the plain check at scale). This module
measures the other configurations of the same metric, each against its own
baseline, and prints one JSON line per pass plus a summary line:

    python -m gpusharesat_gb300.bench_configs batching [--clauses 8000000 --passes 6]
    python -m gpusharesat_gb300.bench_configs serving [--rates 5e4 1e5 2e5 --budget 16000000]

batching: 8e6 clauses (lengths 1 + Zipf(1.2), at most 256), 48 solvers sending
    uneven batches of 4..64 assignments per pass (two 32-slot words each), 5%
    clause churn per pass (deletes plus new clauses from the small workload's
    generator). Three ways to check a pass, all over the same database:
      per_solver  one launch of the default kernel per solver's batch
      single      one launch of the default kernel for all batches
      batched     the autotuned persistent kernel for all batches, replayed
                  as a captured CUDA graph
    The reports of `batched` and `single` are compared record for record on
    the first pass, and the union of the per-solver launches with `single`'s.

serving: 2^21 variables; 64 solver threads with trails of half the variables
    send assignments (each unsets and sets 1..8 literals) in Poisson batches
    of 1..32 at an aggregate 5e4, 1e5 and 2e5 assignments/s; a clause stream
    of 2e5 clauses/s (lengths 1 + Zipf(1.2), at most 256; 0.05% planted to
    report) flows into an HBM budget of 16e6 clauses, full from the start.
    Reports p50/p99/p999 latency from an assignment's arrival to the moment
    every report of it is delivered, and sustained checks/s.
"""
import argparse
import json
import sys
import time

import numpy as np

import gpusharesat_gb300 as g
from gpusharesat_gb300 import autotune, build
from gpusharesat_gb300 import workloads as W


def _sorted(rep):
    return np.sort(rep, order=["clause", "word"])


def _same(a, b):
    a, b = _sorted(a), _sorted(b)
    return len(a) == len(b) and all(np.array_equal(a[f], b[f]) for f in ("clause", "word", "mask"))


def _timed(eng, fn):
    """Runs fn (which launches passes), returns the summed CUDA-event time of
    its check kernels in ms."""
    eng.wait()
    eng.kernel_time()
    eng.set_timing(True)
    fn()
    eng.wait()
    ms, n = eng.kernel_time()
    eng.set_timing(False)
    return ms


def batching(args):
    t0 = time.time()
    wl = W.make_batching(seed=2, n_clauses=args.clauses)
    rng = np.random.default_rng(12)
    print(json.dumps({"config": "batching", "clauses": wl.n_clauses, "literals": wl.n_lits, "vars": wl.n_vars,
                      "solvers": wl.n_solvers, "words": wl.n_words, "setup_s": round(time.time() - t0, 1)}),
          flush=True)
    eng = g.Engine(0)
    eng.set_db(wl.lits, wl.offsets)
    eng.set_state(wl.state, wl.start, wl.solver_of_word)
    # batched form: tune over persistent variants on the first pass's batches
    start0, _ = W.batch_starts(rng, wl.n_solvers)
    P = g.VARIANT_PERSISTENT
    best, table = autotune.tune(eng, wl.state, start0, wl.solver_of_word, launches=3,
                                variants=[(g.KERNEL_WIDE4, 8, 2, P), (g.KERNEL_WIDE4, 8, 1, P),
                                          (g.KERNEL_WIDE4, 8, 4, P), (g.KERNEL_WIDE4, 4, 2, P),
                                          (g.KERNEL_WIDE4, 2, 2, P), (g.KERNEL_WIDE2, 16, 2, P)])
    print(json.dumps({"autotuned": best, "table": table}), flush=True)
    live = np.arange(wl.n_clauses, dtype=np.int64)
    next_id = wl.n_clauses
    rows = []
    for p in range(args.passes):
        if p > 0:
            # 5% churn: random deletes, then as many new clauses
            n_churn = int(0.05 * len(live))
            gone = rng.choice(len(live), size=n_churn, replace=False)
            eng.delete(live[gone].astype(np.uint32))
            live = np.delete(live, gone)
            lits, offs = W.churn_batch(rng, wl.n_vars, n_churn)
            eng.append_db(lits, offs)
            live = np.concatenate([live, np.arange(next_id, next_id + n_churn)])
            next_id += n_churn
            if eng.clause_count > 1.25 * len(live):
                eng.compact()
        start, sizes = W.batch_starts(rng, wl.n_solvers)
        checks = len(live) * int(sizes.sum())
        # single launch, default kernel
        eng.set_variant()
        eng.set_state(wl.state, start, wl.solver_of_word)
        ref = eng.check() if p == 0 else None
        single_ms = _timed(eng, eng.launch)
        # one launch per solver's batch
        per_solver_reps = []

        def per_solver():
            for s in range(wl.n_solvers):
                m = np.zeros_like(start)
                m[2 * s:2 * s + 2] = start[2 * s:2 * s + 2]
                eng.set_start(m)
                if p == 0:
                    per_solver_reps.append(eng.check())
                else:
                    eng.launch()
                    eng.wait()
        per_ms = _timed(eng, per_solver)
        eng.set_start(start)
        # batched: autotuned persistent kernel as a replayed graph
        eng.set_variant(*best)
        eng.set_state(wl.state, start, wl.solver_of_word)
        eng.set_graph(True)
        got = eng.check() if p == 0 else None
        batched_ms = _timed(eng, eng.launch)
        eng.set_graph(False)
        row = {"pass": p, "live_clauses": int(len(live)), "assignments": int(sizes.sum()),
               "checks": checks, "per_solver_ms": per_ms, "single_ms": single_ms, "batched_ms": batched_ms,
               "per_solver_checks_per_s": checks / (per_ms / 1e3), "single_checks_per_s": checks / (single_ms / 1e3),
               "batched_checks_per_s": checks / (batched_ms / 1e3), "graph_captures": eng.graph_captures}
        if p == 0:
            row["batched_equals_single"] = _same(got, ref)
            row["per_solver_union_equals_single"] = _same(np.concatenate(per_solver_reps), ref)
            row["reports"] = int(len(ref))
        rows.append(row)
        print(json.dumps(row), flush=True)
    steady = rows[1:] or rows
    summary = {"config": "batching", "passes": len(rows),
               "per_solver_checks_per_s": float(np.mean([r["per_solver_checks_per_s"] for r in steady])),
               "single_checks_per_s": float(np.mean([r["single_checks_per_s"] for r in steady])),
               "batched_checks_per_s": float(np.mean([r["batched_checks_per_s"] for r in steady])),
               "exact": bool(rows[0]["batched_equals_single"] and rows[0]["per_solver_union_equals_single"]),
               "autotuned_variant": best}
    print(json.dumps(summary), flush=True)
    eng.close()
    return summary


def serving(args):
    """The serving loop through the sharer's C ABI, driven by the C++ load
    generator (gss_serving_run): 64 solver threads, Poisson batches of 1..32
    assignments at an aggregate rate, a clause stream into an HBM budget.
    Each rate is a fresh sharer with the same seed."""
    rows = []
    for rate in args.rates:
        t0 = time.time()
        r = g.serving_run(seconds=args.seconds, warmup_seconds=args.warmup_seconds, assign_rate=rate,
                          n_solvers=64, n_vars=2 ** 21, budget=args.budget, initial_clauses=args.budget,
                          clause_rate=2e5, plant_rate=0.0005, batch_max=32, trail_fraction=0.5,
                          trail_change=8, seed=3)
        r.update({"config": "serving", "assign_rate": rate, "budget": args.budget,
                  "wall_s": round(time.time() - t0, 1)})
        rows.append(r)
        print(json.dumps(r), flush=True)
    summary = {"config": "serving", "rates": args.rates,
               "p50_ms": [r["p50_ms"] for r in rows], "p99_ms": [r["p99_ms"] for r in rows],
               "p999_ms": [r["p999_ms"] for r in rows], "checks_per_s": [r["checks_per_s"] for r in rows],
               "assignments_per_s": [r["assignments_per_s"] for r in rows]}
    print(json.dumps(summary), flush=True)
    return summary


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("config", choices=["batching", "serving"])
    p.add_argument("--clauses", type=int, default=8_000_000)
    p.add_argument("--passes", type=int, default=6)
    p.add_argument("--rates", type=float, nargs="+", default=[5e4, 1e5, 2e5])
    p.add_argument("--budget", type=int, default=16_000_000)
    p.add_argument("--seconds", type=float, default=10.0)
    p.add_argument("--warmup-seconds", type=float, default=2.0)
    args = p.parse_args(argv)
    build.build()
    if args.config == "batching":
        batching(args)
    elif args.config == "serving":
        serving(args)


if __name__ == "__main__":
    main(sys.argv[1:])
