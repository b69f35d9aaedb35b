"""Parity at the benchmark's full sizes.

- The plain check at scale, exactly as the benchmark runs it: 4e6 clauses
  (lengths 2..100) x 1024 assignments (32 solvers x 32), 2^20 variables, the
  default kernel and the default database order (variable ranges). Every
  one of the ~19.6M (clause, word, mask) records is compared with the oracle.
- The uneven-batching workload at full size: 8e6 clauses (1 + Zipf(1.2)
  lengths up to 256) x 48 solvers with two words each and uneven batches,
  after a 5% churn step (400k deletes, 400k appended clauses), checked by the
  persistent kernel with a per-length-class lane plan, replayed as a CUDA
  graph. That pass has ~3.5e8 records, so it is compared through the
  oracle's order-independent digest (record count and a 64-bit hash sum of
  (clause id, word, mask)).
"""
import os

import numpy as np
import pytest

import oracle
from gpusharesat_gb300 import workloads as W

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_scale_workload_full_size_parity(lib):
    import gpusharesat_gb300 as g
    wl = W.make_scale(seed=1)
    assert (wl.n_clauses, wl.n_assignments, wl.n_vars) == (4_000_000, 1024, 2 ** 20)
    eng = g.Engine(0)
    try:
        eng.set_db(wl.lits, wl.offsets)
        assert eng.locality_shift == 17
        eng.set_state(wl.state, wl.start, wl.solver_of_word)
        gpu = g.sort_reports(eng.check())
    finally:
        eng.close()
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=THREADS)
    assert len(ref) > 19_000_000
    assert len(gpu) == len(ref), (len(gpu), len(ref))
    for f in ("clause", "word", "mask"):
        np.testing.assert_array_equal(gpu[f], ref[f], err_msg=f)
    np.testing.assert_array_equal(gpu["solver"], wl.solver_of_word[gpu["word"]])


def test_batching_workload_full_size_after_churn(lib):
    import gpusharesat_gb300 as g
    rng = np.random.default_rng(202)
    wl = W.make_batching(seed=2)
    assert (wl.n_clauses, wl.n_words) == (8_000_000, 96)
    n_churn = wl.n_clauses // 20
    eng = g.Engine(0)
    try:
        eng.set_variant(g.KERNEL_WIDE4, 8, 2, g.VARIANT_PERSISTENT)
        eng.set_graph(True)
        eng.set_db(wl.lits, wl.offsets)
        eng.set_state(wl.state, wl.start, wl.solver_of_word)
        eng.set_length_plan((4, 12, 32, 1 << 30),
                            [g.LAYOUT_4x8_G1, g.LAYOUT_4x8_G2, g.LAYOUT_4x8_G2, g.LAYOUT_4x8_G2])
        # 5% churn: random deletes, then new clauses from the small-workload generator
        gone = np.sort(rng.choice(wl.n_clauses, size=n_churn, replace=False)).astype(np.uint32)
        eng.delete(gone)
        new_lits, new_off = W.distinct_var_clauses(rng, W.lengths_small(rng, n_churn), wl.n_vars)
        eng.append_db(new_lits, new_off)
        assert eng.live_count == wl.n_clauses
        rep = eng.check()
    finally:
        eng.set_graph(False)
        eng.close()
    got = oracle.report_digest(rep["clause"], rep["word"], rep["mask"])
    del rep
    # the live database in id order: the kept clauses, then the appended ones
    keep = np.ones(wl.n_clauses, bool)
    keep[gone] = False
    lens = np.diff(wl.offsets)
    kept_lits = wl.lits[np.repeat(keep, lens)]
    live_lits = np.concatenate([kept_lits, new_lits])
    live_len = np.concatenate([lens[keep], np.diff(new_off)])
    live_off = np.zeros(live_len.shape[0] + 1, np.int64)
    np.cumsum(live_len, out=live_off[1:])
    live_ids = np.concatenate([np.nonzero(keep)[0], wl.n_clauses + np.arange(n_churn)]).astype(np.uint32)
    want = oracle.check_digest(live_lits, live_off, wl.state, wl.start, ids=live_ids, n_threads=THREADS)
    assert want[0] > 100_000_000
    assert got == want, (got, want)
