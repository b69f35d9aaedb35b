"""Autotuner of the check kernel: times every variant on the caller's own
database and assignment state and keeps the fastest one that reports exactly
what the engine's default variant reports.

A variant is (kind, lanes per clause, depth, flags) as taken by
Engine.set_variant: how many 32-slot words a lane owns (kind), how many lanes
share a clause, how many state loads a lane keeps in flight. The engine's
automatic choice comes from a sweep of this kind on the at-scale workload;
tuning on a different workload (few words, short clauses...) can pick another.

    python -m gpusharesat_gb300.autotune --clauses 4000000 --vars-log2 20
"""
import argparse
import json
import time

import numpy as np

import gpusharesat_gb300 as g

# (kind, lanes per clause, depth, flags)
P, O = g.VARIANT_PIPELINED, g.VARIANT_OCCUPANCY
CANDIDATES_WIDE = [(g.KERNEL_WIDE4, 8, 2, P), (g.KERNEL_WIDE4, 8, 2, P | O), (g.KERNEL_WIDE4, 8, 1, P),
                   (g.KERNEL_WIDE4, 8, 4, P), (g.KERNEL_WIDE4, 8, 4, P | O), (g.KERNEL_WIDE4, 4, 2, P | O),
                   (g.KERNEL_WIDE2, 16, 2, P | O), (g.KERNEL_WIDE2, 16, 4, P | O),
                   (g.KERNEL_WIDE4, 8, 1, 0), (g.KERNEL_WIDE4, 8, 2, 0), (g.KERNEL_WIDE4, 8, 4, 0),
                   (g.KERNEL_WIDE4, 4, 2, 0), (g.KERNEL_WIDE4, 4, 4, 0), (g.KERNEL_WIDE4, 2, 2, 0),
                   (g.KERNEL_WIDE2, 16, 2, 2), (g.KERNEL_WIDE2, 8, 2, 2)]
CANDIDATES_DIRECT = [(g.KERNEL_DIRECT, l, d, 0) for l, ds in ((1, (1,)), (2, (1, 2)), (4, (2, 4)), (8, (2, 4)),
                                                              (16, (2, 4)), (32, (2, 4))) for d in ds]
CANDIDATES_TILED = [(g.KERNEL_TILED, 0, k, 0) for k in (2, 4)]


# length classes of the bucketed kernel: (1,4], (4,12], (12,32], (32,...)
LENGTH_CLASSES = (4, 12, 32, 1 << 30)


def tune_length_plan(engine, state, start, solver_of_word=None, classes=LENGTH_CLASSES, layouts=None, launches=4,
                     warmup=1, log=None):
    """Picks a lane layout per length class for the bucketed kernel: for each
    class, times every layout on that class alone (the other classes
    skipped) and keeps the fastest. The state is laid out in 32-word blocks
    (the wide kind, 8 lanes). Returns (layouts, table); the engine is left
    with the plan set, its report set checked against the default kernel's."""
    layouts = layouts or list(g.LAYOUTS)
    engine.set_length_plan()
    engine.set_variant(g.KERNEL_WIDE4, 8, 2, g.VARIANT_PERSISTENT)
    engine.set_state(state, start, solver_of_word)
    want = _key(engine.check())
    table = []
    best = []
    for k in range(len(classes)):
        times = {}
        for lay in layouts:
            plan = [g.LAYOUT_SKIP] * len(classes)
            plan[k] = lay
            engine.set_length_plan(classes, plan)
            for _ in range(warmup):
                engine.launch()
            engine.wait()
            engine.kernel_time()
            engine.set_timing(True)
            for _ in range(launches):
                engine.launch()
            engine.wait()
            ms, n = engine.kernel_time()
            engine.set_timing(False)
            times[lay] = ms / max(n, 1)
            row = {"class": k, "max_len": int(classes[k]), "layout": lay, "ms": times[lay]}
            table.append(row)
            if log:
                log(json.dumps(row))
        best.append(min(times, key=times.get))
    engine.set_length_plan(classes, best)
    same = _key(engine.check()) == want
    table.append({"plan": best, "same_reports": same})
    if not same:
        raise RuntimeError("the tuned length plan reports differently from the default kernel")
    return best, table


def candidates(n_words):
    c = list(CANDIDATES_DIRECT) + list(CANDIDATES_TILED)
    if n_words >= 8:
        c = list(CANDIDATES_WIDE) + c
    return c


def _key(rep):
    order = np.lexsort((rep["word"], rep["clause"]))
    r = rep[order]
    return len(r), hash(r["clause"].tobytes()), hash(r["word"].tobytes()), hash(r["mask"].tobytes())


def tune(engine, state, start, solver_of_word=None, launches=8, warmup=2, variants=None, log=None):
    """Times each variant on the engine's database against (state, start).
    Returns (best variant, table); the engine is left on the best variant."""
    n_words = state.shape[1]
    table = []
    engine.set_variant()
    engine.set_state(state, start, solver_of_word)
    want = _key(engine.check())
    for v in (variants or candidates(n_words)):
        try:
            engine.set_variant(*v)
            engine.set_state(state, start, solver_of_word)
            same = _key(engine.check()) == want
        except g.GssError as e:
            table.append({"variant": v, "error": str(e)})
            continue
        for _ in range(warmup):
            engine.launch()
        engine.wait()
        engine.kernel_time()
        engine.set_timing(True)
        for _ in range(launches):
            engine.launch()
        engine.wait()
        ms, n = engine.kernel_time()
        engine.set_timing(False)
        row = {"variant": v, "ms": ms / max(n, 1), "same_reports": same}
        table.append(row)
        if log:
            log(json.dumps(row))
    ok = [r for r in table if r.get("same_reports")]
    best = min(ok, key=lambda r: r["ms"])["variant"]
    engine.set_variant(*best)
    engine.set_state(state, start, solver_of_word)
    return best, table


def main():
    from gpusharesat_gb300 import build, workloads as W
    p = argparse.ArgumentParser()
    p.add_argument("--clauses", type=int, default=4_000_000)
    p.add_argument("--vars-log2", type=int, default=20)
    p.add_argument("--solvers", type=int, default=32)
    p.add_argument("--launches", type=int, default=8)
    args = p.parse_args()
    build.build()
    t0 = time.time()
    wl = W.make_scale(seed=1, n_vars=2 ** args.vars_log2, n_clauses=args.clauses, n_solvers=args.solvers)
    eng = g.Engine(0)
    eng.set_db(wl.lits, wl.offsets)
    print(json.dumps({"workload": "plain check at scale", "clauses": wl.n_clauses, "vars": wl.n_vars,
                      "words": wl.n_words, "setup_s": round(time.time() - t0, 1)}), flush=True)
    best, table = tune(eng, wl.state, wl.start, wl.solver_of_word, launches=args.launches,
                       log=lambda s: print(s, flush=True))
    print(json.dumps({"best": best, "checks_per_s": wl.n_clauses * wl.n_assignments /
                      (min(r["ms"] for r in table if r.get("same_reports")) / 1e3)}))
    eng.close()


if __name__ == "__main__":
    main()
