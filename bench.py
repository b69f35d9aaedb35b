"""Benchmark: clause x assignment checks/s of the GB300 check pass.

Workload (one "step" = one pass): the plain check at scale - 2^20 variables,
4e6 clauses with lengths 2..100 (60% uniform on 2..16, 40% geometric tail),
1024 partial assignments from 32 solvers (32 each) assigning 40-90% of the
variables with fair signs, 0.1% planted reports; seeded synthetic data of
those shapes (the reference publishes no dataset).

value: checks/s with the clause database and the assignment planes resident
       in HBM (kernel passes back to back, CUDA events on the launch stream).
e2e:   the same metric through the C ABI call gss_check_passes_host_cells
       with host buffers: every step's assignment planes go host->device from
       pinned memory and its reports come back device->host as 8-byte
       records {clause * words + word, mask}; the copies of neighbouring
       steps overlap the current step's check.
latency: submit-to-report p50/p99/p999 through the GpuClauseSharer C ABI
       (the serving shape; see serving_leg).
learned_order: the learned scan order against the plain single launch on
       its own workload (see learned_leg).
batching: uneven batches with churn, the persistent and bucketed forms
       against the plain single launch (see batching_leg).
The inputs (about 0.6 GB) are larger than the 129 MB L2, so no flush is
needed between steps.

--impl reference times the CPU restatement of the reference's check (the
reference has no CPU implementation of its own and its CUDA build cannot run
on the benchmark host) on all host cores, on a bounded sample of the same
workload.

Multi-GPU: clauses are independent, so with N ranks each rank checks its own
database shard of the same size (weak scaling) with no collective on the
data path; value = all ranks' checks / the slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "clause\u00d7assignment checks/s on 1 GB300, bit-exact"
UNIT = "checks/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="scale", choices=["scale", "small"],
                   help="scale: 4e6 clauses x 1024 assignments (the headline); small: 1e5 clauses x 64 assignments")
    p.add_argument("--clauses", type=int, default=None)
    p.add_argument("--vars-log2", type=int, default=20)
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--kind", type=int, default=None, help="check kernel kind (0 direct, 1 tiled)")
    p.add_argument("--lpc", type=int, default=0, help="lanes per clause (0 = automatic)")
    p.add_argument("--depth", type=int, default=4, help="loads in flight (direct) or clause slots (tiled)")
    p.add_argument("--flags", type=int, default=0, help="variant flags (1: L2 hint, 2: occupancy)")
    p.add_argument("--locality", type=int, default=-1,
                   help="database order: -1 automatic variable ranges, 0 length order, 11..31 ranges of 2^n vars")
    p.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    p.add_argument("--serving-seconds", type=float, default=3.0,
                   help="measured seconds per rate of the serving leg (0: skip it)")
    p.add_argument("--learned-passes", type=int, default=120,
                   help="passes of the learned-order leg (0: skip it)")
    p.add_argument("--batching-passes", type=int, default=3,
                   help="passes of the batching leg (0: skip it)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def config_dict(args, world):
    if args.workload == "small":
        return {
            "workload": "plain check, small: %d clauses (lengths 2-30, geometric mean 8) x 64 assignments "
                        "(1 solver), 2^14 variables, 1%% planted reports" % args.clauses,
            "clauses_per_gpu": args.clauses, "assignments": 64, "variables": 2 ** 14, "solvers": 1,
            "l2": "inputs fit in L2 (about 4 MB): no roofline claim",
            "parallelism": "clause shards, %d replica(s)" % world,
        }
    return {
        "workload": "plain check at scale: %d clauses (lengths 2-100) x 1024 assignments (32 solvers x 32), "
                    "2^%d variables, 0.1%% planted reports" % (args.clauses, args.vars_log2),
        "clauses_per_gpu": args.clauses,
        "assignments": 1024,
        "variables": 2 ** args.vars_log2,
        "solvers": 32,
        "l2": "inputs larger than L2 (no flush)",
        "parallelism": "clause shards, %d replica(s)" % world,
    }


def algorithmic_bytes(wl, n_reports):
    """4*sum(L) + 8*V*ceil(A/32) + 16*R per pass."""
    words = (wl.n_assignments + 31) // 32
    return 4 * wl.n_lits + 8 * wl.n_vars * words + 16 * n_reports


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    """Per-launch DRAM bytes (read + write) of the check kernel on this
    workload, from the committed ncu summary (its `traffic_bytes_per_launch`
    line), or None."""
    import re
    path = os.path.join(ROOT, "profiles", "check_wide_persist_kernel_plain_scale.md")
    if os.path.exists(path):
        with open(path) as f:
            m = re.search(r"traffic_bytes_per_launch\s*[|:]\s*([0-9]+)", f.read())
            if m:
                return int(m.group(1))
    return None


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for i, n in enumerate(names):
                    if r[5 + i].lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def shard_seed(rank):
    """Each rank checks its own clause shard of the same size (weak scaling)."""
    return 1 + 1000 * rank


def make_workload(args, rank):
    from gpusharesat_gb300 import workloads as W
    if args.workload == "small":
        return W.make_small(seed=shard_seed(rank) - 1, n_clauses=args.clauses)
    return W.make_scale(seed=shard_seed(rank), n_vars=2 ** args.vars_log2, n_clauses=args.clauses)


def max_over_ranks(value, world, device):
    """The slowest rank's value (all_reduce MAX over the process group)."""
    if world == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank_per_step, world, max_seconds_per_step):
    """Whole-job units/s: all ranks' units over the slowest rank's time."""
    return units_per_rank_per_step * world / max_seconds_per_step


SERVING_RATES = (5e4, 1e5, 2e5)


def serving_leg(seconds):
    """Submit-to-report latency through the GpuClauseSharer C ABI
    (gss_sharer_*: addClause, trySendAssignment, gpuRun, popReportedClause,
    getLastAssigAllReported), driven by the C++ load generator
    gss_serving_run in the serving shape: 2^21 variables, a 16e6-clause HBM
    budget filled at the start, a clause stream of 2e5 clauses/s with
    oldest-unreported eviction, 64 solver threads sending Poisson batches of
    1..32 assignments at an aggregate 5e4, 1e5 and 2e5 assignments/s, 0.05%
    planted reports. Latency of an assignment: its arrival (batch time) to
    the moment getLastAssigAllReported passes it for its solver."""
    import gpusharesat_gb300 as g
    rows = []
    for rate in SERVING_RATES:
        r = g.serving_run(seconds=seconds, warmup_seconds=1.0, assign_rate=rate, n_solvers=64, n_vars=2 ** 21,
                          budget=16_000_000, initial_clauses=16_000_000, clause_rate=2e5, plant_rate=0.0005,
                          batch_max=32, trail_fraction=0.5, trail_change=8, seed=3)
        rows.append({"rate_assignments_per_s": rate, "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"],
                     "p999_ms": r["p999_ms"], "mean_ms": r["mean_ms"], "assignments": r["assignments"],
                     "checks_per_s": r["checks_per_s"], "passes": r["passes"], "retries": r["retries"],
                     "evicted": r["evicted"]})
    return {"endpoints": "trySendAssignment arrival -> getLastAssigAllReported (GpuClauseSharer.h:151)",
            "workload": "2^21 variables, 16e6-clause budget, 2e5 clauses/s stream, 64 solvers, batches of 1-32, "
                        "0.05%% planted reports, %.0f s measured per rate after 1 s warm-up" % seconds,
            "rates": rows}


def learned_leg(passes):
    """The composed form against the plain single launch on the learned-order
    workload (bench_configs.learned): 2^21 variables, 4e6 clauses plus a
    stream of 500 a pass, 2048 slots, reports planted at latent per-clause
    rates; the persistent kernel with the learned head (25% of the scan) and
    tail, the history every pass, the order rebuilt every 4 passes, retrained
    halfway. Reports recall in the first 10% of the scan, delivery latency on
    the device clock, sustained checks/s of back-to-back passes, and whether
    every compared pass reported exactly the plain scan's set."""
    import contextlib
    import io
    from gpusharesat_gb300 import bench_configs
    args = argparse.Namespace(clauses=4_000_000, passes=passes, retrain=max(1, passes // 2), head_fraction=0.25,
                              compare_every=10, throughput_passes=20, rescore=4, overlap=1, stream_per_pass=500)
    with contextlib.redirect_stdout(io.StringIO()):
        r = bench_configs.learned(args)
    return {
        "workload": "2^21 variables, 4e6 clauses + 500 a pass, 2048 slots, latent report rates Beta(0.5, 20); "
                    "%d passes, retrained after %d, order rebuilt every 4 passes, head 25%% of the scan" % (
                        passes, args.retrain),
        "recall_first_10pct": {"learned": r["recall_first_10pct_learned"], "plain": r["recall_first_10pct_plain"]},
        "device_latency_ms": {"learned_p50": r["device_latency_p50_ms_learned"],
                              "learned_p99": r["device_latency_p99_ms_learned"],
                              "plain_p50": r["device_latency_p50_ms_plain"],
                              "plain_p99": r["device_latency_p99_ms_plain"]},
        "sustained_checks_per_s": {"learned": r["sustained_checks_per_s_learned"],
                                   "plain_single_launch": r["sustained_checks_per_s_plain"]},
        "sustained_ms_per_pass": {"learned": r["sustained_ms_per_pass_learned"],
                                  "plain_single_launch": r["sustained_ms_per_pass_plain"],
                                  "persistent_without_order": r["sustained_ms_per_pass_persistent_no_order"]},
        "same_reports_every_compared_pass": r["same_reports_every_compared_pass"],
        "compared_passes": r["compared_passes"],
    }


def batching_leg(passes):
    """Uneven batches with churn (bench_configs.batching) at 2e6 clauses:
    48 solvers with U[4,64] assignments each, 5% clause churn per pass; the
    autotuned persistent kernel replayed as a captured graph and the bucketed
    kernel against one launch of the plain grid-stride kernel for all
    batches and against one launch per solver; report sets compared on the
    first pass."""
    import contextlib
    import io
    from gpusharesat_gb300 import bench_configs
    args = argparse.Namespace(clauses=2_000_000, passes=passes)
    with contextlib.redirect_stdout(io.StringIO()):
        r = bench_configs.batching(args)
    return {
        "workload": "2^20 variables, 2e6 clauses (lengths 1 + Zipf(1.2), at most 256), 48 solvers x U[4,64] "
                    "assignments, 5%% churn per pass, %d passes" % passes,
        "checks_per_s": {"batched_persistent_graph": r["batched_checks_per_s"],
                         "bucketed_length_plan": r["bucketed_checks_per_s"],
                         "plain_single_launch": r["single_checks_per_s"],
                         "one_launch_per_solver": r["per_solver_checks_per_s"]},
        "autotuned_variant": r["autotuned_variant"],
        "exact": r["exact"],
    }


def cpu_parity(wl, gpu_reports, threads=None):
    """CPU leg, part 1: the oracle (C restatement, all host cores) checks the
    whole workload once, outside the timed region, and its records are
    compared field by field with the GPU's sizing pass (clause, word, mask,
    and the solver of the word)."""
    import oracle
    import gpusharesat_gb300 as g
    threads = threads or os.cpu_count() or 1
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=threads)
    got = g.sort_reports(gpu_reports)
    mism = abs(len(got) - len(ref))
    if len(got) == len(ref):
        bad = (got["clause"] != ref["clause"]) | (got["word"] != ref["word"]) | (got["mask"] != ref["mask"]) | \
            (got["solver"] != wl.solver_of_word[ref["word"]].astype(np.uint32))
        mism = int(bad.sum())
    return {"records": int(len(ref)), "gpu_records": int(len(got)), "mismatches": int(mism),
            "checker": "oracle/check.c (C restatement of gpuShareLib/GpuRunner.cu:34-89), full workload"}


def cpu_baseline(wl, seconds, threads=None):
    """CPU leg, part 2: times the oracle (C restatement, all host cores) on a
    prefix of the clause database sized to take about `seconds`. Returns
    checks/s and the sample description."""
    import oracle
    threads = threads or os.cpu_count() or 1
    n = min(wl.n_clauses, 20000)
    while True:
        t0 = time.perf_counter()
        oracle.check(wl.lits, wl.offsets[:n + 1], wl.state, wl.start, n_threads=threads)
        dt = time.perf_counter() - t0
        if dt >= seconds / 4 or n >= wl.n_clauses:
            break
        n = min(wl.n_clauses, int(n * max(2.0, (seconds / 4) / max(dt, 1e-3))))
    reps = max(1, int(seconds / max(dt, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.check(wl.lits, wl.offsets[:n + 1], wl.state, wl.start, n_threads=threads)
    dt = (time.perf_counter() - t0) / reps
    return n * wl.n_assignments / dt, threads, "%d of %d clauses x %d assignments, %d rep(s)" % (
        n, wl.n_clauses, wl.n_assignments, reps)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    wl = make_workload(args, 0)
    threads = os.cpu_count() or 1
    # size one step's sample to about 2 s of CPU work
    n = 20000
    t0 = time.perf_counter()
    oracle.check(wl.lits, wl.offsets[:n + 1], wl.state, wl.start, n_threads=threads)
    dt = time.perf_counter() - t0
    n = int(min(wl.n_clauses, max(n, n * 2.0 / max(dt, 1e-3))))
    for _ in range(args.warmup):
        oracle.check(wl.lits, wl.offsets[:n + 1], wl.state, wl.start, n_threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.check(wl.lits, wl.offsets[:n + 1], wl.state, wl.start, n_threads=threads)
        times.append(time.perf_counter() - t0)
    per_step = float(np.mean(times))
    value = n * wl.n_assignments / per_step
    sample = "%d of %d clauses x %d assignments per step" % (n, wl.n_clauses, wl.n_assignments)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded)",
        "config": config_dict(args, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference's check rule (the reference has no CPU path; its CUDA build "
                "cannot run here), all host threads",
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    import gpusharesat_gb300 as g
    from gpusharesat_gb300 import build as b
    b.build()

    wl = make_workload(args, rank)
    stream = torch.cuda.Stream()
    eng = g.Engine(local)
    eng.set_stream(stream.cuda_stream)
    if args.kind is not None:
        eng.set_variant(args.kind, args.lpc, args.depth, args.flags)
    eng.set_locality(args.locality)
    eng.set_db(wl.lits, wl.offsets)
    eng.set_state(wl.state, wl.start, wl.solver_of_word)
    # size the queues: run once (grows on overflow); its reports are checked
    # against the oracle in the CPU leg, after the timed regions
    sizing_reports = eng.check()
    n_reports = len(sizing_reports)

    # ---- device-resident timing (value) ----
    for _ in range(args.warmup):
        eng.launch()
    torch.cuda.synchronize()
    eng.kernel_time()  # drop warm-up events
    eng.set_timing(True)
    sampler = ClockSampler(local) if rank == 0 else None
    barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
        time.sleep(0.3)
    launches0 = eng.launch_count
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        eng.launch()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop() if sampler else None
    gpu_launches = eng.launch_count - launches0
    eng.set_timing(False)
    n_last = eng.wait()
    assert n_last == n_reports, (n_last, n_reports)
    kern_ms, kern_n = eng.kernel_time()
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1), world, "cuda")
    ms_per_step = elapsed_ms / args.steps
    checks_per_pass = wl.n_clauses * wl.n_assignments
    value = job_throughput(checks_per_pass, world, ms_per_step / 1e3)

    # ---- end to end through host buffers (e2e) ----
    # gss_check_passes_host: K passes in one call, each copying its state in
    # from pinned host memory and its reports out to pinned host memory, the
    # copies of neighbouring passes overlapping the check of the current one.
    states_h = [torch.from_numpy(wl.state.reshape(-1)).pin_memory() for _ in range(2)]
    start_h = torch.from_numpy(wl.start).pin_memory()
    sow_h = torch.from_numpy(wl.solver_of_word).pin_memory()
    cap = n_reports + 1024
    outs_h = [torch.empty(cap * 2, dtype=torch.int32).pin_memory() for _ in range(2)]
    lib = g.load()

    def e2e_run(k):
        sp = (ctypes.c_void_p * k)(*[states_h[i % 2].data_ptr() for i in range(k)])
        op = (ctypes.c_void_p * k)(*[outs_h[i % 2].data_ptr() for i in range(k)])
        caps = (ctypes.c_int64 * k)(*([cap] * k))
        nrep = (ctypes.c_int64 * k)()
        rc = lib.gss_check_passes_host_cells(eng.h, k, sp, wl.n_vars, wl.n_words,
                                             ctypes.c_void_p(start_h.data_ptr()), ctypes.c_void_p(sow_h.data_ptr()),
                                             op, caps, nrep)
        g._check(rc)
        assert all(nrep[i] == n_reports for i in range(k)), list(nrep)

    e2e_s = float("nan")
    e2e_parity = None
    if not args.no_e2e:
        e2e_run(max(2, args.warmup))
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_run(args.e2e_steps)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, world, "cuda")
        if rank == 0:
            # the last timed step's host records against the sizing pass (outside the timed region)
            cells = outs_h[(args.e2e_steps - 1) % 2].numpy().view(g.CELL_REPORT_DTYPE)[:n_reports]
            got = g.sort_reports(g.cells_to_reports(cells, wl.n_words))
            ref = g.sort_reports(sizing_reports)
            e2e_parity = {"records": int(n_reports), "mismatches": int(
                ((got["clause"] != ref["clause"]) | (got["word"] != ref["word"]) | (got["mask"] != ref["mask"])).sum())}
    h2d = wl.state.nbytes + wl.start.nbytes + wl.solver_of_word.nbytes
    d2h = n_reports * 8 + 16 * 4  # {clause * words + word, mask} records, and the counters

    if rank == 0:
        peak, peak_kind = load_peaks()
        kern_avg_s = (kern_ms / max(kern_n, 1)) / 1e3
        B = algorithmic_bytes(wl, n_reports)
        achieved = B / kern_avg_s / 1e9
        traffic = load_traffic() if (args.workload == "scale" and args.clauses == 4_000_000
                                     and args.kind is None and args.locality == -1) else None
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak,
                    "traffic": traffic,
                    "traffic_source": ("ncu capture of this kernel on this workload, committed summary "
                                       "profiles/check_wide_persist_kernel_plain_scale.md (not measured in this "
                                       "run)")
                    if traffic else None,
                    "algorithmic_bytes_per_launch": B, "kernel_ms": kern_avg_s * 1e3,
                    "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                    else "fallback"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded)",
            "config": config_dict(args, world),
            "reports_per_pass": n_reports,
            "e2e": {"value": job_throughput(checks_per_pass, world, e2e_s), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                    "host_link_gbs": (h2d + d2h) / e2e_s / 1e9,
                    "call": "gss_check_passes_host_cells (8-byte {clause * words + word, mask} report records "
                            "packed on the device)",
                    "parity_vs_sizing_pass": e2e_parity}
            if not args.no_e2e else None,
            "database_order": {"locality_shift": eng.locality_shift},
            "roofline": roofline,
            "gpu_launches": gpu_launches,
            "clocks": clocks,
        }
        # the other configurations' legs measure one GPU: they run at N = 1
        # (in a multi-GPU run they would hold every rank's GPU for minutes)
        one_gpu = world == 1 and args.workload == "scale"
        if args.serving_seconds > 0 and one_gpu:
            line["latency"] = serving_leg(args.serving_seconds)
        if args.learned_passes > 0 and one_gpu:
            line["learned_order"] = learned_leg(args.learned_passes)
        if args.batching_passes > 0 and one_gpu:
            line["batching"] = batching_leg(args.batching_passes)
        if not args.no_cpu_baseline:
            line["parity"] = cpu_parity(wl, sizing_reports)
            if world == 1:  # the CPU baseline is timed at N = 1 only
                v, cores, sample = cpu_baseline(wl, args.cpu_seconds)
                line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.clauses is None:
        args.clauses = 100_000 if args.workload == "small" else 4_000_000
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
