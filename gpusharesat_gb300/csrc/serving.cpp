// Load generator for the serving loop: simulated solver threads submitting
// assignments to a GpuClauseSharer while a GPU thread runs passes and a
// clause stream flows in against an HBM budget. Host C++ over the C ABI; it
// measures submit-to-delivery latency and sustained checks/s.
//
// Solvers behave like CDCL threads (what GpuHelpedSolver does through the
// API, glucose-syrup/gpu/GpuHelpedSolver.cc:109-157): each keeps a trail;
// an assignment is a small backtrack (unsetSolverValues), a few new literals
// (trySetSolverValues) and trySendAssignment. Assignments arrive in batches
// of 1..batch_max at Poisson times. A request that finds its solver's 32
// slots taken waits for the next pass to free them: continuous batching, each
// pass admits whatever arrived while the previous one ran.
//
// Latency of an assignment: from its arrival time to the moment its solver
// sees getLastAssigAllReported pass it (every report of the assignment
// delivered and popped).
//
// Clauses and trails follow a hidden total assignment M, as learned clauses
// and trails of solvers working on one satisfiable formula would: every trail
// literal is true under M, and every clause of the database and of the
// stream has at least two literals true under M (each other literal is false
// under M with probability 1/2). Such a clause never reports: under any trail
// its M-true literals are true or unassigned. Planted clauses (plant_rate of
// the stream) do: their literals are the negations of literals on some
// solver's current trail, plus one literal of a variable that trail leaves
// unassigned.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

#include "gpusharesat.h"

namespace {

using Clock = std::chrono::steady_clock;

double now_s(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

// splitmix64
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    uint32_t below(uint32_t n) { return (uint32_t) ((next() >> 32) * (uint64_t) n >> 32); }
    double exponential(double rate) { return -log(1.0 - uniform()) / rate; }
};

// Clause lengths 1 + Zipf(a) capped at `cap`, by inverse CDF.
struct LengthTable {
    std::vector<double> cdf;
    LengthTable(double a, int cap) {
        double total = 0;
        for (int k = 1; k < cap; k++) total += pow((double) k, -a);
        double acc = 0;
        for (int k = 1; k < cap; k++) {
            acc += pow((double) k, -a) / total;
            cdf.push_back(acc);
        }
    }
    int draw(Rng &r) const {
        const double u = r.uniform();
        const int k = (int) (std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
        return 1 + std::min<int>(k, (int) cdf.size());
    }
};

// Random clauses with distinct variables, at least two literals true under
// the hidden assignment M (model[v] = 1: v is true in M).
struct ClauseGen {
    const LengthTable &lt;
    const std::vector<uint8_t> &model;
    std::vector<uint32_t> seen;  // epoch of the clause that last used each variable
    uint32_t epoch = 0;
    ClauseGen(const LengthTable &t, const std::vector<uint8_t> &m) : lt(t), model(m), seen(m.size(), 0) {}
    void draw(Rng &r, std::vector<int> &out) {
        const int len = std::min<int>(lt.draw(r), (int) seen.size());
        out.clear();
        epoch++;
        while ((int) out.size() < len) {
            const int v = (int) r.below((uint32_t) seen.size());
            if (seen[v] == epoch) continue;
            seen[v] = epoch;
            const bool m_true = out.size() < 2 || (r.next() & 1);
            out.push_back(m_true ? true_lit(v) : true_lit(v) ^ 1);
        }
        // the guaranteed M-true literals at random positions
        for (int k = 0; k < 2 && k < len; k++) std::swap(out[k], out[k + r.below((uint32_t) (len - k))]);
    }
    int true_lit(int v) const { return 2 * v + (model[v] ? 0 : 1); }
};

struct Solver {
    std::mutex lock;  // guards trail and assigned against the planting reader
    std::vector<int> trail;
    std::vector<uint8_t> assigned;
    std::vector<double> arrival;  // arrival time of each sent assignment, by id
    int64_t completed = 0;        // assignments whose reports were all delivered
    int64_t popped = 0;
    int64_t retries = 0;
    std::vector<float> latency_ms;
};

}  // namespace

extern "C" {

int gss_serving_run(const gss_serving_params *p, gss_serving_result *res) {
    if (!p || !res || p->n_solvers < 1 || p->n_vars < 2 || p->assign_rate <= 0 || p->batch_max < 1)
        return GSS_ERR_INVALID;
    memset(res, 0, sizeof *res);
    gss_sharer_options o;
    gss_sharer_options_default(&o);
    o.verbosity = 0;
    o.min_gpu_latency_micros = 0;
    gss_sharer *sh = nullptr;
    int rc = gss_sharer_create(&o, nullptr, nullptr, -1, &sh);
    if (rc != GSS_OK) return rc;
    gss_sharer_set_var_count(sh, p->n_vars);
    gss_sharer_set_cpu_solver_count(sh, p->n_solvers);
    gss_sharer_set_max_clause_len(sh, 256);
    gss_sharer_set_clause_budget(sh, p->budget);
    if (p->plain_scan) {
        gss_sharer_set_variant(sh, GSS_KERNEL_WIDE4, 8, 2, 0);
        gss_sharer_set_locality(sh, 0);
    }
    const LengthTable lt(1.2, 256);
    std::vector<uint8_t> model(p->n_vars);
    {
        Rng r(p->seed * 6151 + 9);
        for (auto &m : model) m = (uint8_t) (r.next() & 1);
    }
    auto true_lit = [&](int v) { return 2 * v + (model[v] ? 0 : 1); };

    // initial database
    {
        Rng r(p->seed * 7919 + 1);
        ClauseGen gen(lt, model);
        std::vector<int> cl;
        for (int64_t i = 0; i < p->initial_clauses; i++) {
            gen.draw(r, cl);
            gss_sharer_add_clause(sh, -1, cl.data(), (int) cl.size());
        }
    }
    // solvers with their initial trails
    std::vector<Solver> solvers(p->n_solvers);
    for (int s = 0; s < p->n_solvers; s++) {
        Solver &sv = solvers[s];
        Rng r(p->seed * 104729 + 17 * s + 3);
        sv.assigned.assign(p->n_vars, 0);
        const int n0 = (int) (p->trail_fraction * p->n_vars);
        while ((int) sv.trail.size() < n0) {
            const int v = (int) r.below((uint32_t) p->n_vars);
            if (sv.assigned[v]) continue;
            sv.assigned[v] = 1;
            sv.trail.push_back(true_lit(v));
        }
        if (!sv.trail.empty() && !gss_sharer_try_set_solver_values(sh, s, sv.trail.data(), (int) sv.trail.size())) {
            gss_sharer_destroy(sh);
            return GSS_ERR_STATE;
        }
    }
    rc = gss_sharer_gpu_run(sh);  // the first pass uploads the database
    if (rc == GSS_OK) rc = gss_sharer_gpu_run(sh);
    if (rc != GSS_OK) {
        gss_sharer_destroy(sh);
        return rc;
    }

    const auto t0 = Clock::now();
    const double t_measure = p->warmup_seconds;
    const double t_end = p->warmup_seconds + p->seconds;
    std::atomic<bool> stop{false};
    std::atomic<int> gpu_error{0};
    std::atomic<int64_t> streamed{0}, passes{0};
    // Solver threads sleep until the next pass ends or their next arrival,
    // instead of polling: 64 polling threads on a 16-core host would take the
    // CPU from the thread that runs the passes.
    std::mutex pass_lock;
    std::condition_variable pass_done;
    int64_t pass_seq = 0;
    auto notify_pass = [&]() {
        {
            std::lock_guard<std::mutex> g(pass_lock);
            pass_seq++;
        }
        pass_done.notify_all();
    };
    // waits for a pass after `seen`, or until `deadline_s` (seconds since t0)
    auto wait_pass = [&](int64_t seen, double deadline_s) {
        std::unique_lock<std::mutex> g(pass_lock);
        const auto until = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(deadline_s));
        pass_done.wait_until(g, until, [&]() { return pass_seq != seen || stop.load(); });
        return pass_seq;
    };
    auto pass_now = [&]() {
        std::lock_guard<std::mutex> g(pass_lock);
        return pass_seq;
    };
    int64_t tested_at_measure = -1;
    double time_at_measure = 0;
    std::mutex measure_lock;

    // GPU thread: clause stream and passes
    std::vector<float> run_ms;  // gpuRun call durations in the measured window (GPU thread only)
    double long_ms[4] = {0, 0, 0, 0};
    std::thread gpu([&]() {
        Rng r(p->seed * 31 + 5);
        ClauseGen gen(lt, model);
        std::vector<int> cl;
        int64_t produced = 0;
        bool measured = false;
        while (!stop.load()) {
            const double t = now_s(t0);
            if (!measured && t >= t_measure) {
                std::lock_guard<std::mutex> g(measure_lock);
                tested_at_measure = gss_sharer_global_stat(sh, 6 /* totalAssigClauseTested */);
                time_at_measure = t;
                measured = true;
            }
            const int64_t due = (int64_t) (t * p->clause_rate);
            for (; produced < due; produced++) {
                if (r.uniform() < p->plant_rate) {
                    // the negations of literals on a solver's current trail (false
                    // under it, and under M), plus the M-true literal of a
                    // variable the trail leaves unassigned
                    Solver &sv = solvers[r.below((uint32_t) p->n_solvers)];
                    std::lock_guard<std::mutex> g(sv.lock);
                    const int len = std::min<int>(lt.draw(r), 1 + (int) sv.trail.size());
                    cl.clear();
                    for (int k = 0; k + 1 < len; k++) {
                        const int l = sv.trail[r.below((uint32_t) sv.trail.size())];
                        bool dup = false;
                        for (int x : cl)
                            if ((x >> 1) == (l >> 1)) dup = true;
                        if (!dup) cl.push_back(l ^ 1);
                    }
                    for (int tries = 0; tries < 64; tries++) {
                        const int v = (int) r.below((uint32_t) p->n_vars);
                        if (!sv.assigned[v]) {
                            cl.push_back(true_lit(v));
                            break;
                        }
                    }
                } else {
                    gen.draw(r, cl);
                }
                if (!cl.empty()) gss_sharer_add_clause(sh, -1, cl.data(), (int) cl.size());
            }
            streamed = produced;
            const double r0 = now_s(t0);
            // the sharer's time statistics (microseconds): timeSpentTestingClauses (9),
            // timeSpentFillingAssigs (10), timeSpentFillingReported (11)
            int64_t st0[3];
            for (int k = 0; k < 3; k++) st0[k] = gss_sharer_global_stat(sh, 9 + k);
            const int rc_run = gss_sharer_gpu_run(sh);
            if (r0 >= t_measure && r0 < t_end) {
                const double ms = (now_s(t0) - r0) * 1e3;
                run_ms.push_back((float) ms);
                if (ms > 20.0) {
                    double parts = 0;
                    for (int k = 0; k < 3; k++) {
                        const double d = (gss_sharer_global_stat(sh, 9 + k) - st0[k]) * 1e-3;
                        long_ms[k] += d;
                        parts += d;
                    }
                    long_ms[3] += ms - parts;
                }
            }
            if (rc_run != GSS_OK) {
                gpu_error = 1;
                stop = true;
                notify_pass();
                break;
            }
            passes++;
            notify_pass();
        }
    });

    // solver threads
    const double mean_batch = (1 + p->batch_max) / 2.0;
    const double batch_rate = p->assign_rate / (p->n_solvers * mean_batch);
    std::vector<std::thread> threads;
    for (int s = 0; s < p->n_solvers; s++) {
        threads.emplace_back([&, s]() {
            Solver &sv = solvers[s];
            Rng r(p->seed * 1000003 + 7 * s + 11);
            double next_arrival = r.exponential(batch_rate);
            int pending_batch = 0;
            double batch_time = 0;
            std::vector<int> add, del;
            auto poll = [&]() {
                int *lits;
                int count;
                int64_t id;
                while (gss_sharer_pop_reported_clause(sh, s, &lits, &count, &id)) sv.popped++;
                const int64_t upto = gss_sharer_last_assig_all_reported(sh, s);
                const double t = now_s(t0);
                for (; sv.completed < upto && sv.completed < (int64_t) sv.arrival.size(); sv.completed++) {
                    const double arr = sv.arrival[sv.completed];
                    if (arr >= t_measure && t <= t_end) sv.latency_ms.push_back((float) ((t - arr) * 1e3));
                }
            };
            while (!stop.load()) {
                const double t = now_s(t0);
                if (t >= t_end) break;
                if (pending_batch == 0 && t >= next_arrival) {
                    pending_batch = 1 + (int) r.below((uint32_t) p->batch_max);
                    batch_time = next_arrival;
                    next_arrival += r.exponential(batch_rate);
                }
                if (pending_batch > 0) {
                    // next assignment: backtrack a little, then a few new literals
                    del.clear();
                    add.clear();
                    {
                        std::lock_guard<std::mutex> g(sv.lock);
                        int u = 1 + (int) r.below((uint32_t) p->trail_change);
                        u = std::min<int>(u, (int) sv.trail.size());
                        for (int k = 0; k < u; k++) {
                            const int l = sv.trail.back();
                            sv.trail.pop_back();
                            sv.assigned[l >> 1] = 0;
                            del.push_back(l);
                        }
                        const int d = 1 + (int) r.below((uint32_t) p->trail_change);
                        while ((int) add.size() < d) {
                            const int v = (int) r.below((uint32_t) p->n_vars);
                            if (sv.assigned[v]) continue;
                            sv.assigned[v] = 1;
                            const int l = true_lit(v);
                            add.push_back(l);
                            sv.trail.push_back(l);
                        }
                    }
                    if (!del.empty()) gss_sharer_unset_solver_values(sh, s, del.data(), (int) del.size());
                    // a full ring frees at the next pass's cut: wait for it
                    int64_t seen = pass_now();
                    while (!gss_sharer_try_set_solver_values(sh, s, add.data(), (int) add.size())) {
                        sv.retries++;
                        poll();
                        if (stop.load()) break;
                        seen = wait_pass(seen, now_s(t0) + 0.002);
                    }
                    int64_t id;
                    while ((id = gss_sharer_try_send_assignment(sh, s)) < 0) {
                        sv.retries++;
                        poll();
                        if (stop.load()) break;
                        seen = wait_pass(seen, now_s(t0) + 0.002);
                    }
                    if (id >= 0) {
                        if ((int64_t) sv.arrival.size() <= id) sv.arrival.resize(id + 1);
                        sv.arrival[id] = batch_time;
                    }
                    pending_batch--;
                } else {
                    // deliveries come with passes: sleep until the next one
                    // ends or the next batch arrives
                    const int64_t seen = pass_now();
                    poll();
                    wait_pass(seen, std::min(next_arrival, t_end));
                }
            }
        });
    }
    while (now_s(t0) < t_end && !stop.load()) std::this_thread::sleep_for(std::chrono::milliseconds(5));
    const double t_stop = now_s(t0);
    const int64_t tested_end = gss_sharer_global_stat(sh, 6);
    stop = true;
    notify_pass();
    for (auto &t : threads) t.join();
    gpu.join();

    std::vector<float> all;
    for (auto &sv : solvers) {
        all.insert(all.end(), sv.latency_ms.begin(), sv.latency_ms.end());
        res->reports_popped += sv.popped;
        res->retries += sv.retries;
    }
    std::sort(all.begin(), all.end());
    auto pct = [&](double q) -> double {
        if (all.empty()) return 0;
        size_t i = (size_t) (q * (all.size() - 1));
        return all[i];
    };
    res->p50_ms = pct(0.50);
    res->p99_ms = pct(0.99);
    res->p999_ms = pct(0.999);
    res->max_ms = all.empty() ? 0 : all.back();
    double sum = 0;
    for (float x : all) sum += x;
    res->mean_ms = all.empty() ? 0 : sum / all.size();
    res->assignments = (int64_t) all.size();
    res->passes = passes;
    res->elapsed_s = t_stop - time_at_measure;
    res->checks_per_s = tested_at_measure >= 0 && res->elapsed_s > 0
                            ? (double) (tested_end - tested_at_measure) / res->elapsed_s
                            : 0;
    res->assignments_per_s = res->elapsed_s > 0 ? all.size() / res->elapsed_s : 0;
    res->evicted = gss_sharer_evicted_count(sh);
    res->clauses_streamed = streamed;
    res->live_clauses_end = gss_sharer_global_stat(sh, 0 /* gpuClauses */);
    res->device_compactions = gss_sharer_device_compactions(sh);
    std::sort(run_ms.begin(), run_ms.end());
    if (!run_ms.empty()) {
        res->run_ms_p50 = run_ms[(size_t) (0.5 * (run_ms.size() - 1))];
        res->run_ms_p99 = run_ms[(size_t) (0.99 * (run_ms.size() - 1))];
        res->run_ms_max = run_ms.back();
        for (float x : run_ms) res->long_runs += x > 20.0f;
    }
    res->long_wait_ms = long_ms[0];
    res->long_launch_ms = long_ms[1];
    res->long_deliver_ms = long_ms[2];
    res->long_other_ms = long_ms[3];
    gss_sharer_destroy(sh);
    return gpu_error ? GSS_ERR_CUDA : GSS_OK;
}

}  // extern "C"
