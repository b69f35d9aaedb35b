"""Measurements of the batching, serving and learned-order workloads.

bench.py measures the headline (the plain check at scale). This module
measures the other configurations of the same metric, each against its own
baseline, and prints one JSON line per pass plus a summary line:

    python -m gpusharesat_gb300.bench_configs batching [--clauses 8000000 --passes 6]
    python -m gpusharesat_gb300.bench_configs serving [--rates 5e4 1e5 2e5 --budget 16000000]
    python -m gpusharesat_gb300.bench_configs learned [--clauses 4000000 --passes 3000 --retrain 1000]
    python -m gpusharesat_gb300.bench_configs gather [--passes 20]

batching: 8e6 clauses (lengths 1 + Zipf(1.2), at most 256), 48 solvers sending
    uneven batches of 4..64 assignments per pass (two 32-slot words each), 5%
    clause churn per pass (deletes plus new clauses from the small workload's
    generator). Three ways to check a pass, all over the same database:
      per_solver  one launch of the grid-stride wide kernel per solver's batch
      single      one launch of the grid-stride wide kernel for all batches
      batched     the autotuned persistent kernel for all batches, replayed
                  as a captured CUDA graph
      bucketed    the bucketed persistent kernel with a lane layout per
                  length class (tuned class by class), replayed as a graph
    The report sets of `batched`, `bucketed` and `single`, and the union of
    the per-solver launches, are compared on the first pass through an
    order-independent hash sum of their (clause, word, mask) records.

serving: 2^21 variables; 64 solver threads with trails of half the variables
    send assignments (each unsets and sets 1..8 literals) in Poisson batches
    of 1..32 at an aggregate 5e4, 1e5 and 2e5 assignments/s; a clause stream
    of 2e5 clauses/s (lengths 1 + Zipf(1.2), at most 256; 0.05% planted to
    report) flows into an HBM budget of 16e6 clauses, full from the start.
    Reports p50/p99/p999 latency from an assignment's arrival to the moment
    every report of it is delivered, and sustained checks/s, for the sharer's
    default form (persistent kernel over the variable-range order) and, with
    --compare-plain 1, for the plain single-launch scan (grid-stride wide
    kernel, length order) at the same rates.

learned: 2^21 variables; 4e6 clauses at the start (lengths 1 + Zipf(1.2),
    at most 256) plus a stream of 500 new clauses per pass (as many of the
    oldest deleted), 64 words x 32 slots per pass. Clauses are built over a
    hidden model and the slots agree with it, so a clause reports only when
    planted; clause c is planted in a pass with latent probability
    r_c ~ Beta(0.5, 20), and its LBD falls with r_c. The order retrains every
    1000 passes; the head (delivered early) is the first 25% of the scan.
    The ordered passes run the persistent kernel (head and tail launches);
    every compare_every passes the plain single launch (grid-stride wide
    kernel, no order) checks the same state. Reports the share of report
    bits in the first 10% of the learned scan against the plain order's
    first 10%, the delivery latency of report bits (from the launch call to
    the moment the host has them, and on the device clock), sustained
    checks/s of both forms over back-to-back passes, and that each compared
    pass reports what the plain scan reports.

gather: the bound of the check kernels. Random 256-byte row gathers
    (gss_probe_gather: 8 lanes x 32 bytes a row, 2 rows in flight per group,
    8 blocks of 256 threads per SM) over buffers of 32 MB to 1 GB, the host
    link's pinned copy rates (each direction, then both at once), then the
    default check kernel on the at-scale workload (4e6 clauses x 1024
    assignments) with 2^17 variables (a 32 MB state, resident in L2) and
    with 2^20 variables (256 MB, the benchmark's): the kernel time with the
    state in L2 is the floor its instruction issue and latency set; the
    difference at 2^20 is what the misses to DRAM cost.
"""
import argparse
import json
import sys
import time

import numpy as np

import gpusharesat_gb300 as g
from gpusharesat_gb300 import autotune, build
from gpusharesat_gb300 import workloads as W


def _mix64(z):
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _digest(reps, chunk=1 << 24):
    """(records, order-independent 64-bit hash sum) of one or more report
    arrays, for comparing report sets of hundreds of millions of records
    without sorting them."""
    n, total = 0, np.uint64(0)
    with np.errstate(over="ignore"):
        for rep in reps:
            for b in range(0, len(rep), chunk):
                r = rep[b:b + chunk]
                key = (r["clause"].astype(np.uint64) << np.uint64(32)) | r["word"].astype(np.uint64)
                total = total + np.add.reduce(_mix64(_mix64(key) ^ r["mask"].astype(np.uint64)), dtype=np.uint64)
            n += len(rep)
    return n, int(total)


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
    # bucketed form: a lane layout per length class, tuned class by class
    plan, ptable = autotune.tune_length_plan(eng, wl.state, start0, wl.solver_of_word)
    eng.set_length_plan()
    print(json.dumps({"length_plan": plan, "classes": list(autotune.LENGTH_CLASSES), "table": ptable}), flush=True)
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
        # single launch: the plain grid-stride wide kernel
        eng.set_variant(g.KERNEL_WIDE4, 8, 2, 0)
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
                    per_solver_reps.append(_digest([eng.check()]))
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
        # bucketed: the tuned length plan in one persistent launch, as a graph
        eng.set_variant(g.KERNEL_WIDE4, 8, 2, g.VARIANT_PERSISTENT)
        eng.set_state(wl.state, start, wl.solver_of_word)
        eng.set_length_plan(autotune.LENGTH_CLASSES, plan)
        got_b = eng.check() if p == 0 else None
        bucketed_ms = _timed(eng, eng.launch)
        eng.set_length_plan()
        eng.set_graph(False)
        row = {"pass": p, "live_clauses": int(len(live)), "assignments": int(sizes.sum()),
               "checks": checks, "per_solver_ms": per_ms, "single_ms": single_ms, "batched_ms": batched_ms,
               "per_solver_checks_per_s": checks / (per_ms / 1e3), "single_checks_per_s": checks / (single_ms / 1e3),
               "batched_checks_per_s": checks / (batched_ms / 1e3), "bucketed_ms": bucketed_ms,
               "bucketed_checks_per_s": checks / (bucketed_ms / 1e3), "graph_captures": eng.graph_captures}
        if p == 0:
            dref = _digest([ref])
            row["batched_equals_single"] = _digest([got]) == dref
            row["bucketed_equals_single"] = _digest([got_b]) == dref
            union = (sum(x[0] for x in per_solver_reps), int(sum(x[1] for x in per_solver_reps) % (1 << 64)))
            row["per_solver_union_equals_single"] = union == dref
            row["reports"] = int(len(ref))
        rows.append(row)
        print(json.dumps(row), flush=True)
    steady = rows[1:] or rows
    summary = {"config": "batching", "passes": len(rows),
               "per_solver_checks_per_s": float(np.mean([r["per_solver_checks_per_s"] for r in steady])),
               "single_checks_per_s": float(np.mean([r["single_checks_per_s"] for r in steady])),
               "batched_checks_per_s": float(np.mean([r["batched_checks_per_s"] for r in steady])),
               "bucketed_checks_per_s": float(np.mean([r["bucketed_checks_per_s"] for r in steady])),
               "exact": bool(rows[0]["batched_equals_single"] and rows[0]["per_solver_union_equals_single"]
                             and rows[0]["bucketed_equals_single"]),
               "autotuned_variant": best, "length_plan": plan}
    print(json.dumps(summary), flush=True)
    eng.close()
    return summary


def serving(args):
    """The serving loop through the sharer's C ABI, driven by the C++ load
    generator (gss_serving_run): 64 solver threads, Poisson batches of 1..32
    assignments at an aggregate rate, a clause stream into an HBM budget.
    Each rate is a fresh sharer with the same seed."""
    rows = []
    plain_rows = []
    for rate in args.rates:
        for plain in ((0, 1) if args.compare_plain else (0,)):
            t0 = time.time()
            r = g.serving_run(seconds=args.seconds, warmup_seconds=args.warmup_seconds, assign_rate=rate,
                              n_solvers=64, n_vars=2 ** 21, budget=args.budget, initial_clauses=args.budget,
                              clause_rate=2e5, plant_rate=0.0005, batch_max=32, trail_fraction=0.5,
                              trail_change=8, seed=3, plain_scan=plain)
            r.update({"config": "serving", "assign_rate": rate, "budget": args.budget,
                      "form": "plain single launch (grid-stride wide kernel, length order)" if plain
                      else "persistent kernel over the variable-range order, two-pass pipeline",
                      "wall_s": round(time.time() - t0, 1)})
            (plain_rows if plain else rows).append(r)
            print(json.dumps(r), flush=True)
    summary = {"config": "serving", "rates": args.rates,
               "p50_ms": [r["p50_ms"] for r in rows], "p99_ms": [r["p99_ms"] for r in rows],
               "p999_ms": [r["p999_ms"] for r in rows], "checks_per_s": [r["checks_per_s"] for r in rows],
               "assignments_per_s": [r["assignments_per_s"] for r in rows]}
    if plain_rows:
        summary["plain"] = {"p50_ms": [r["p50_ms"] for r in plain_rows], "p99_ms": [r["p99_ms"] for r in plain_rows],
                            "p999_ms": [r["p999_ms"] for r in plain_rows],
                            "checks_per_s": [r["checks_per_s"] for r in plain_rows]}
    print(json.dumps(summary), flush=True)
    return summary


_POP16 = np.array([bin(i).count("1") for i in range(1 << 16)], dtype=np.uint8)


def _bits(rep):
    """Report bits (clause x slot pairs) of a report array."""
    if not len(rep):
        return 0
    m = np.ascontiguousarray(rep["mask"]).astype(np.uint32)
    if hasattr(np, "bitwise_count"):
        return int(np.bitwise_count(m).sum(dtype=np.int64))
    return int(_POP16[m & 0xFFFF].sum(dtype=np.int64) + _POP16[m >> 16].sum(dtype=np.int64))


def _weighted_quantile(values, weights, q):
    order = np.argsort(values)
    v, w = np.asarray(values)[order], np.asarray(weights, dtype=np.float64)[order]
    c = np.cumsum(w)
    if c[-1] <= 0:
        return 0.0
    return float(v[np.searchsorted(c, q * c[-1])])


def learned(args):
    """Learned scan order against the plain scan on one stream of passes.

    Per pass: plant reports at the clauses' latent rates into the base state
    (device), then the ordered pass (scoring, head launch, tail launch) with
    its head delivered early, and, every compare_every passes, the plain
    single-launch pass over the same state, whose report set must equal the
    ordered pass's. The stream appends stream_per_pass new clauses and
    deletes as many of the oldest before each pass."""
    import torch
    t0 = time.time()
    P, k = args.passes, args.stream_per_pass
    d = W.make_learned(seed=4, n_vars=2 ** 21, n_clauses=args.clauses, n_words=64, stream=k * P)
    n0, n_vars, n_words = d["n_clauses"], d["n_vars"], d["n_words"]
    lits, offsets = d["lits"], d["offsets"]
    print(json.dumps({"config": "learned", "clauses": n0, "stream_per_pass": k, "passes": P,
                      "literals": int(offsets[n0]), "vars": n_vars, "slots": 32 * n_words,
                      "setup_s": round(time.time() - t0, 1)}), flush=True)
    dev = torch.device("cuda:0")
    d_lits = torch.from_numpy(lits).to(dev)
    d_off = torch.from_numpy(offsets).to(dev)
    rate_all = torch.from_numpy(d["rate"]).to(dev)
    d_rate = torch.zeros_like(rate_all)
    d_rate[:n0] = rate_all[:n0]
    base = torch.from_numpy(d["state"].view(np.int32)).to(dev)
    state = base.clone()
    start = torch.full((n_words,), -1, dtype=torch.int32, device=dev)
    eng = g.Engine(0)
    # the composed form: the persistent kernel under the learned order; the
    # comparison pass: the plain single launch (grid-stride wide kernel) on
    # the same database and state (the state layout is the same for both)
    composed = (g.KERNEL_WIDE4, 8, 2, g.VARIANT_PERSISTENT)
    plain_variant = (g.KERNEL_WIDE4, 8, 2, 0)
    eng.set_variant(*composed)
    eng.set_db(lits[:offsets[n0]], offsets[:n0 + 1])
    eng.order_enable(head_fraction=args.head_fraction, retrain_interval=args.retrain, train_epochs=2, seed=4,
                     overlap=args.overlap, rescore_interval=args.rescore)
    eng.set_lbd(np.arange(n0, dtype=np.uint32), d["lbd"][:n0])
    # room for the planted reports of a pass (about 0.75 records per clause at 64 words)
    eng.set_capacity(max(1 << 22, 2 * n0))
    lo, nxt = 0, n0
    rows = []
    # report buffers reused across passes (their pages stay mapped)
    bufs = [np.ones(1 << 22, dtype=g.REPORT_DTYPE) for _ in range(3)]
    for p in range(P):
        if p > 0 and k:
            ids = np.arange(nxt, nxt + k, dtype=np.uint32)
            b0, b1 = int(offsets[nxt]), int(offsets[nxt + k])
            eng.append_db(lits[b0:b1], offsets[nxt:nxt + k + 1] - b0, ids)
            eng.set_lbd(ids, d["lbd"][nxt:nxt + k])
            eng.delete(np.arange(lo, lo + k, dtype=np.uint32))
            d_rate[nxt:nxt + k] = rate_all[nxt:nxt + k]
            d_rate[lo:lo + k] = 0
            nxt += k
            lo += k
        g.bench_plant(d_lits.data_ptr(), d_off.data_ptr(), nxt, d_rate.data_ptr(), state.data_ptr(),
                      base.data_ptr(), n_vars, n_words, 4, p, 0)
        torch.cuda.synchronize()
        eng.set_state_device(state.data_ptr(), n_vars, n_words, start.data_ptr())
        eng.wait()
        ta = time.perf_counter()
        eng.launch()
        tl = time.perf_counter()
        head = eng.wait_head(cap=bufs[0].shape[0], out=bufs[0])
        tb = time.perf_counter()
        tail = eng.copy_tail(cap=bufs[1].shape[0], out=bufs[1])
        tc = time.perf_counter()
        st = eng.order_stats()
        head_bits = _bits(head)
        row = {"pass": p, "head_bits": head_bits, "bits": head_bits + _bits(tail), "launch_call_ms": (tl - ta) * 1e3,
               "head_ms": (tb - ta) * 1e3,
               "all_ms": (tc - ta) * 1e3, "score_dev_ms": st["score_ms"], "head_dev_ms": st["head_ms"],
               "tail_dev_ms": st["tail_ms"], "trainings": st["trainings"]}
        if p % args.compare_every == 0:
            # the plain pass starts on an idle GPU (the order's scoring of the
            # next pass, on its own stream, is not charged to it)
            torch.cuda.synchronize()
            eng.order_set_active(False)
            eng.set_variant(*plain_variant)
            eng.set_timing(True)
            eng.kernel_time()
            td = time.perf_counter()
            eng.launch()
            tl2 = time.perf_counter()
            plain = eng.reports(out=bufs[2])
            te = time.perf_counter()
            row["plain_launch_call_ms"] = (tl2 - td) * 1e3
            row["plain_all_ms"] = (te - td) * 1e3
            row["plain_dev_ms"] = eng.kernel_time()[0]
            eng.set_timing(False)
            eng.set_variant(*composed)
            eng.order_set_active(True)
            # report sets compared by an order-independent hash sum (no sort
            # of millions of records per compared pass)
            row["same_reports"] = _digest([head, tail]) == _digest([plain])
            # share of report bits in the first 10% of each scan order
            n_scan = eng.clause_count
            first10 = int(np.ceil(0.1 * n_scan))
            row["plain_first10_bits"] = _bits(plain[eng.positions(plain["clause"]) < first10])
            row["learned_first10_bits"] = (_bits(head[eng.scan_ranks(head["clause"]) < first10]) +
                                           _bits(tail[eng.scan_ranks(tail["clause"]) < first10]))
        rows.append(row)
        g.bench_plant(d_lits.data_ptr(), d_off.data_ptr(), nxt, d_rate.data_ptr(), state.data_ptr(),
                      base.data_ptr(), n_vars, n_words, 4, p, 1)
        torch.cuda.synchronize()
        if p % 100 == 0:
            print(json.dumps(row), flush=True)
    # sustained passes, back to back on the last pass's state, with no report
    # handling on the host: the ordered form (scoring of the next pass on its
    # own stream, head and tail launches, history) against the plain single
    # launch; wall clock over K passes, each waited for before the next
    thr = {}
    if args.throughput_passes > 0:
        K = args.throughput_passes
        live = nxt - lo
        for name in ("learned", "plain", "persistent", "learned"):
            learned_form = name == "learned"
            eng.order_set_active(learned_form)
            eng.set_variant(*(plain_variant if name == "plain" else composed))
            for _ in range(3):
                eng.launch()
                eng.wait()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(K):
                eng.launch()
                eng.wait()
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / K
            thr[name] = {"ms_per_pass": dt * 1e3, "checks_per_s": live * 32 * n_words / dt}
        eng.set_variant(*composed)
        eng.order_set_active(True)
        print(json.dumps({"throughput_passes": K, **{k: v for k, v in thr.items()}}), flush=True)
    trained = [r for r in rows if r["trainings"] >= 1 and r["bits"]]
    cmp_rows = [r for r in trained if "plain_all_ms" in r]
    cmp_bits = max(1, np.sum([r["bits"] for r in cmp_rows]))
    head_share = float(np.sum([r["head_bits"] for r in trained]) / max(1, np.sum([r["bits"] for r in trained])))
    recall = float(np.sum([r["learned_first10_bits"] for r in cmp_rows]) / cmp_bits)
    plain_recall = float(np.sum([r["plain_first10_bits"] for r in cmp_rows]) / cmp_bits)
    # delivery latency of each report bit, from the pass's launch call
    lv, lw, pv, pw = [], [], [], []
    for r in cmp_rows:
        lv += [r["head_ms"], r["all_ms"]]
        lw += [r["head_bits"], r["bits"] - r["head_bits"]]
        pv.append(r["plain_all_ms"])
        pw.append(r["bits"])
    # the same on the device clock: head bits when the head launch ends, the
    # rest when the tail ends (the scoring ran during the previous pass),
    # against the plain launch's end
    dv, dw, dp = [], [], []
    for r in cmp_rows:
        dv += [r["head_dev_ms"], r["head_dev_ms"] + r["tail_dev_ms"]]
        dw += [r["head_bits"], r["bits"] - r["head_bits"]]
        dp.append(r["plain_dev_ms"])
    checks_ordered = [(nxt - lo) * 32 * n_words / (r["all_ms"] / 1e3) for r in cmp_rows]
    checks_plain = [(nxt - lo) * 32 * n_words / (r["plain_all_ms"] / 1e3) for r in cmp_rows]
    summary = {"config": "learned", "passes": P, "trained_passes": len(trained), "compared_passes": len(cmp_rows),
               "head_fraction": args.head_fraction, "head_share_of_report_bits": head_share,
               "recall_first_10pct_learned": recall, "recall_first_10pct_plain": plain_recall,
               "latency_mean_ms_learned": float(np.average(lv, weights=lw)) if cmp_rows else None,
               "latency_mean_ms_plain": float(np.average(pv, weights=pw)) if cmp_rows else None,
               "latency_p50_ms_learned": _weighted_quantile(lv, lw, 0.5) if cmp_rows else None,
               "latency_p50_ms_plain": _weighted_quantile(pv, pw, 0.5) if cmp_rows else None,
               "latency_p99_ms_learned": _weighted_quantile(lv, lw, 0.99) if cmp_rows else None,
               "latency_p99_ms_plain": _weighted_quantile(pv, pw, 0.99) if cmp_rows else None,
               "device_latency_p50_ms_learned": _weighted_quantile(dv, dw, 0.5) if cmp_rows else None,
               "device_latency_p99_ms_learned": _weighted_quantile(dv, dw, 0.99) if cmp_rows else None,
               "device_latency_p50_ms_plain": _weighted_quantile(dp, pw, 0.5) if cmp_rows else None,
               "device_latency_p99_ms_plain": _weighted_quantile(dp, pw, 0.99) if cmp_rows else None,
               "launch_call_ms_learned": float(np.mean([r["launch_call_ms"] for r in cmp_rows])) if cmp_rows else None,
               "launch_call_ms_plain": float(np.mean([r["plain_launch_call_ms"] for r in cmp_rows]))
               if cmp_rows else None,
               "pass_ms_learned": float(np.mean([r["all_ms"] for r in cmp_rows])) if cmp_rows else None,
               "pass_ms_plain": float(np.mean([r["plain_all_ms"] for r in cmp_rows])) if cmp_rows else None,
               "score_dev_ms": float(np.mean([r["score_dev_ms"] for r in trained])) if trained else None,
               "device_ms_learned": float(np.mean([r["score_dev_ms"] + r["head_dev_ms"] + r["tail_dev_ms"]
                                                   for r in cmp_rows])) if cmp_rows else None,
               "device_ms_plain": float(np.mean([r["plain_dev_ms"] for r in cmp_rows])) if cmp_rows else None,
               "overlap": args.overlap, "rescore_interval": args.rescore,
               "checks_per_s_learned": float(np.mean(checks_ordered)) if cmp_rows else None,
               "checks_per_s_plain": float(np.mean(checks_plain)) if cmp_rows else None,
               "sustained_ms_per_pass_learned": thr["learned"]["ms_per_pass"] if thr else None,
               "sustained_ms_per_pass_plain": thr["plain"]["ms_per_pass"] if thr else None,
               "sustained_checks_per_s_learned": thr["learned"]["checks_per_s"] if thr else None,
               "sustained_checks_per_s_plain": thr["plain"]["checks_per_s"] if thr else None,
               "sustained_ms_per_pass_persistent_no_order": thr["persistent"]["ms_per_pass"] if thr else None,
               "same_reports_every_compared_pass": all(r["same_reports"] for r in rows if "same_reports" in r),
               "trainings": rows[-1]["trainings"] if rows else 0}
    print(json.dumps(summary), flush=True)
    eng.close()
    return summary


def _host_link(mb=256, reps=5):
    """Pinned host <-> device copy rates: one direction at a time, then both
    at once on two streams (best of `reps`, wall clock around synchronize)."""
    import torch
    n = mb << 20
    dev = torch.device("cuda:0")
    h_in = torch.ones(n, dtype=torch.uint8).pin_memory()
    h_out = torch.empty(n, dtype=torch.uint8).pin_memory()
    d_in = torch.empty(n, dtype=torch.uint8, device=dev)
    d_out = torch.ones(n, dtype=torch.uint8, device=dev)
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()
    rows = []
    for name, up, down in (("host->device", True, False), ("device->host", False, True), ("both", True, True)):
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if up:
                with torch.cuda.stream(s_up):
                    d_in.copy_(h_in, non_blocking=True)
            if down:
                with torch.cuda.stream(s_down):
                    h_out.copy_(d_out, non_blocking=True)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        moved = n * (int(up) + int(down))
        row = {"host_link": name, "mb_each_way": mb, "ms": best * 1e3, "gb_per_s": moved / best / 1e9}
        rows.append(row)
        print(json.dumps(row), flush=True)
    return rows


def gather(args):
    """Row-gather probe over several working sets, then the default check
    kernel with its state in L2 and in DRAM (see the module docstring)."""
    rows = []
    for mb in (32, 64, 96, 128, 192, 256, 1024):
        rps, ms = g.probe_gather(mb << 20, depth=2, blocks_per_sm=8)
        row = {"probe": "random 256-byte rows", "buffer_mb": mb, "rows_per_s": rps, "ms_per_launch": ms,
               "tb_per_s": rps * 256 / 1e12}
        rows.append(row)
        print(json.dumps(row), flush=True)
    rows += _host_link()
    for vl in (17, 20):
        wl = W.make_scale(seed=1, n_vars=2 ** vl)
        eng = g.Engine(0)
        try:
            eng.set_db(wl.lits, wl.offsets)
            eng.set_state(wl.state, wl.start, wl.solver_of_word)
            n = len(eng.check())
            for _ in range(5):
                eng.launch()
            ms = _timed(eng, lambda: [eng.launch() for _ in range(args.passes)]) / args.passes
        finally:
            eng.close()
        row = {"kernel": "default check kernel", "variables": 2 ** vl, "state_mb": (2 ** vl) * 256 / 2 ** 20,
               "clauses": wl.n_clauses, "slots": 1024, "reports": n, "ms_per_pass": ms,
               "literal_visits_note": "about 8.4 state-row gathers per clause"}
        rows.append(row)
        print(json.dumps(row), flush=True)
    return rows


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("config", choices=["batching", "serving", "learned", "gather"])
    p.add_argument("--clauses", type=int, default=8_000_000)
    p.add_argument("--passes", type=int, default=6)
    p.add_argument("--rates", type=float, nargs="+", default=[5e4, 1e5, 2e5])
    p.add_argument("--budget", type=int, default=16_000_000)
    p.add_argument("--seconds", type=float, default=10.0)
    p.add_argument("--warmup-seconds", type=float, default=2.0)
    p.add_argument("--stream-per-pass", type=int, default=500)
    p.add_argument("--retrain", type=int, default=1000)
    p.add_argument("--head-fraction", type=float, default=0.25)
    p.add_argument("--compare-every", type=int, default=5)
    p.add_argument("--overlap", type=int, default=1)
    p.add_argument("--rescore", type=int, default=1,
                   help="learned: passes per scoring and sort (the passes between keep the last order)")
    p.add_argument("--throughput-passes", type=int, default=50,
                   help="learned: back-to-back passes of each form for the sustained checks/s (0: skip)")
    p.add_argument("--compare-plain", type=int, default=1,
                   help="serving: also run each rate with the plain single-launch scan")
    args = p.parse_args(argv)
    if args.config == "learned" and "--clauses" not in (argv or sys.argv):
        args.clauses = 4_000_000
    if args.config == "learned" and "--passes" not in (argv or sys.argv):
        args.passes = 3000
    build.build()
    if args.config == "batching":
        batching(args)
    elif args.config == "serving":
        serving(args)
    elif args.config == "learned":
        learned(args)
    elif args.config == "gather":
        if "--passes" not in (argv or sys.argv):
            args.passes = 20
        gather(args)


if __name__ == "__main__":
    main(sys.argv[1:])
