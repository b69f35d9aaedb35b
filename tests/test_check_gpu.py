"""Parity of the CUDA check pass with the CPU oracle, through the C ABI.

Bit-exact: the set of (clause, word, slot-mask) records must equal the
oracle's. Covers the small plain-check workload in full, the at-scale
workload at reduced size and edge cases (unit clauses, the longest clause,
partial words, unstarted slots, empty inputs, queue overflow).
"""
import numpy as np
import pytest

import oracle
from gpusharesat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _gpu_reports(engine, wl, capacity=0):
    import gpusharesat_gb300 as g
    engine.set_db(wl.lits, wl.offsets)
    engine.set_state(wl.state, wl.start, wl.solver_of_word)
    engine.set_capacity(capacity)
    rep = engine.check()
    return g.sort_reports(rep)


def _assert_same(gpu, ref, wl=None):
    assert len(gpu) == len(ref), (len(gpu), len(ref))
    for f in ("clause", "word", "mask"):
        np.testing.assert_array_equal(gpu[f], ref[f], err_msg=f)
    if wl is not None and len(gpu):
        np.testing.assert_array_equal(gpu["solver"], wl.solver_of_word[gpu["word"]])


def test_small_workload_parity(engine):
    wl = W.make_small(seed=0)
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=8)
    gpu = _gpu_reports(engine, wl)
    _assert_same(gpu, ref, wl)
    # planted clauses whose last literal is false or undefined must report
    assert len(ref) > 0


def test_scale_workload_reduced_parity(engine):
    wl = W.make_scale(seed=1, n_vars=2 ** 16, n_clauses=200_000)
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=8)
    gpu = _gpu_reports(engine, wl)
    _assert_same(gpu, ref, wl)


@pytest.mark.parametrize("n_words", [1, 3, 33, 70])
def test_word_counts(engine, n_words):
    rng = np.random.default_rng(100 + n_words)
    n_vars = 3000
    lengths = W.lengths_small(rng, 5000)
    lits, offsets = W.distinct_var_clauses(rng, lengths, n_vars)
    state = W.random_state(rng, n_vars, n_words, rng.uniform(0.3, 0.95, 32 * n_words))
    start = rng.integers(0, 2 ** 32, size=n_words, dtype=np.uint32)  # ragged started slots
    start[0] = 0xFFFFFFFF
    wl = W.Workload("words", n_vars, lits, offsets, state, start,
                    (np.arange(n_words) // 2).astype(np.int32), (n_words + 1) // 2)
    ref = oracle.check(lits, offsets, state, start)
    gpu = _gpu_reports(engine, wl)
    _assert_same(gpu, ref, wl)


def test_unit_and_long_clauses(engine, lib):
    rng = np.random.default_rng(7)
    n_vars = 20000
    maxlen = lib.gss_max_clause_len()
    lengths = np.array([1] * 500 + [2] * 500 + [maxlen, maxlen - 1, 100, 101, 255, 256, 257], dtype=np.int64)
    lits, offsets = W.distinct_var_clauses(rng, lengths, n_vars)
    # mostly-false assignments so that long clauses survive a while
    state = W.random_state(rng, n_vars, 4, np.full(128, 0.999))
    # make every long clause all-false under slot 5 of word 2
    for c in range(1000, len(lengths)):
        for i in range(offsets[c], offsets[c + 1]):
            v = lits[i] >> 1
            state[v, 2, 0] |= np.uint32(1 << 5)
            t = (int(state[v, 2, 1]) >> 5) & 1
            lits[i] = 2 * v + t
    start = np.full(4, 0xFFFFFFFF, dtype=np.uint32)
    wl = W.Workload("edge", n_vars, lits, offsets, state, start, np.arange(4, dtype=np.int32), 4)
    ref = oracle.check(lits, offsets, state, start)
    gpu = _gpu_reports(engine, wl)
    _assert_same(gpu, ref, wl)
    long_ids = set(range(1000, len(lengths)))
    hit = {int(r["clause"]) for r in ref if r["word"] == 2 and (int(r["mask"]) >> 5) & 1}
    assert long_ids <= hit


def test_unstarted_slots_never_report(engine):
    rng = np.random.default_rng(3)
    n_vars = 500
    lits, offsets = W.distinct_var_clauses(rng, np.ones(400, dtype=np.int64), n_vars)
    state = np.zeros((n_vars, 2, 2), dtype=np.uint32)  # everything undefined: units report everywhere
    start = np.array([0x0000F00F, 0], dtype=np.uint32)
    wl = W.Workload("unstarted", n_vars, lits, offsets, state, start, np.zeros(2, np.int32), 1)
    gpu = _gpu_reports(engine, wl)
    assert len(gpu) == 400
    assert set(gpu["mask"].tolist()) == {0x0000F00F}
    assert set(gpu["word"].tolist()) == {0}


def test_empty_inputs(engine):
    wl = W.Workload("empty", 10, np.zeros(0, np.int32), np.zeros(1, np.int64),
                    np.zeros((10, 1, 2), np.uint32), np.full(1, 0xFFFFFFFF, np.uint32), np.zeros(1, np.int32), 1)
    assert len(_gpu_reports(engine, wl)) == 0
    rng = np.random.default_rng(1)
    lits, offsets = W.distinct_var_clauses(rng, np.full(10, 3), 10)
    wl0 = W.Workload("nowords", 10, lits, offsets, np.zeros((10, 0, 2), np.uint32), np.zeros(0, np.uint32),
                     np.zeros(0, np.int32), 0)
    assert len(_gpu_reports(engine, wl0)) == 0


def test_wait_before_any_launch(lib):
    """A fresh engine has no pass to wait for: wait and copy give nothing."""
    import gpusharesat_gb300 as g
    eng = g.Engine(0)
    assert eng.wait() == 0
    assert len(eng.reports()) == 0
    eng.close()


def test_overflow_reruns_to_same_result(engine):
    wl = W.make_small(seed=5, n_clauses=20000)
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    gpu = _gpu_reports(engine, wl, capacity=64)  # far too small: the engine grows and reruns
    _assert_same(gpu, ref, wl)


def test_rejects_bad_database(engine):
    import gpusharesat_gb300 as g
    with pytest.raises(g.GssError):
        engine.set_db(np.array([-2], np.int32), np.array([0, 1], np.int64))
    with pytest.raises(g.GssError):
        engine.set_db(np.zeros(0, np.int32), np.array([0, 0], np.int64))  # empty clause
    # a database with variables beyond the state is refused at launch
    engine.set_db(np.array([2 * 50], np.int32), np.array([0, 1], np.int64))
    engine.set_state(np.zeros((10, 1, 2), np.uint32), np.full(1, 1, np.uint32))
    with pytest.raises(g.GssError):
        engine.launch()


def test_pass_through_host_buffers(engine):
    wl = W.make_small(seed=9, n_clauses=30000)
    import gpusharesat_gb300 as g
    engine.set_db(wl.lits, wl.offsets)
    engine.set_capacity(0)
    rep = g.sort_reports(engine.pass_host(wl.state, wl.start, wl.solver_of_word))
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    _assert_same(rep, ref, wl)


@pytest.mark.parametrize("records", ["full", "packed", "cells"])
def test_pipelined_passes_through_host_buffers(engine, records):
    """Several passes with different states, pipelined over three streams, each
    equal to the oracle; small output capacities force the overflow path.
    packed: the 12-byte records packed on the device; cells: the 8-byte
    {clause * n_words + word, mask} records."""
    import gpusharesat_gb300 as g
    rng = np.random.default_rng(17)
    base = W.make_scale(seed=17, n_vars=2 ** 12, n_clauses=30000, n_solvers=32)
    states = [W.random_state(rng, base.n_vars, 32, rng.uniform(0.4, 0.9, 1024)) for _ in range(5)]
    engine.set_db(base.lits, base.offsets)
    for caps in (None, [100] * 5):
        engine.set_capacity(0 if caps is None else 50)
        got = g.passes_host(engine, states, base.start, base.solver_of_word, caps=caps, records=records)
        for st, rep in zip(states, got):
            if records == "cells":
                rep = g.cells_to_reports(rep, 32)
            ref = oracle.check(base.lits, base.offsets, st, base.start)
            _assert_same(g.sort_reports(rep), ref)
    engine.set_capacity(0)


def test_cell_records_refuse_ids_past_32_bits(engine):
    """Cell records need (largest id + 1) x words <= 2^32: a clause id of 2^22
    over 1024 words is refused, not wrapped."""
    import gpusharesat_gb300 as g
    engine.set_db(np.array([2, 4], np.int32), np.array([0, 2], np.int64))
    engine.append_db(np.array([2, 6], np.int32), np.array([0, 2], np.int64), np.array([1 << 22], np.uint32))
    n_words = 1024
    state = np.zeros((8, n_words, 2), np.uint32)
    with pytest.raises(g.GssError):
        g.passes_host(engine, [state], np.full(n_words, 0xFFFFFFFF, np.uint32), np.arange(n_words, dtype=np.int32),
                      records="cells")


import kat  # noqa: E402


@pytest.mark.parametrize("case", kat.load_cases(), ids=lambda c: c["name"])
def test_reference_known_answers_on_gpu(engine, case):
    """The reference's own known-answer cases, through the C ABI on the GPU."""
    lits, offsets, state, start, sow = kat.case_inputs(case)
    wl = W.Workload(case["name"], case["n_vars"], lits, offsets, state, start, sow, int(sow.max()) + 1)
    gpu = _gpu_reports(engine, wl)
    got = oracle.expand(gpu)
    np.testing.assert_array_equal(got, kat.expected_triples(case))


DIRECT_VARIANTS = [(0, l, g, h) for l, gs in ((1, (1,)), (2, (1, 2)), (4, (1, 2, 4)), (8, (1, 2, 4, 8)), (16, (1, 2, 4, 8)),
                                                (32, (1, 2, 4, 8))) for g in gs for h in (0, 1)]
TILED_VARIANTS = [(1, l, k, h) for l in (0, 1, 2, 4, 8, 16, 32) for k in (2, 4, 8) for h in (0, 1)]
WIDE_VARIANTS = [(kind, l, d, occ * 2) for kind, l, ds in ((2, 8, (1, 2, 4)), (2, 4, (1, 2, 4)), (2, 2, (1, 2)),
                                                             (3, 16, (1, 2, 4)), (3, 8, (1, 2, 4)))
                 for d in ds for occ in (0, 1)]
PERSISTENT_VARIANTS = [(2, 8, d, 8) for d in (1, 2, 4)] + [(2, 4, 2, 8), (2, 2, 2, 8), (3, 16, 2, 8), (3, 8, 2, 8)]
PIPELINED_VARIANTS = [(kind, l, d, 4 | occ * 2) for kind, l, ds in ((2, 8, (1, 2, 4)), (2, 4, (2, 4)), (3, 16, (2, 4)))
                      for d in ds for occ in (0, 1)]


@pytest.mark.parametrize("locality", [0, 11])
@pytest.mark.parametrize("kind,lpc,depth,hints",
                         DIRECT_VARIANTS + TILED_VARIANTS + WIDE_VARIANTS + PIPELINED_VARIANTS + PERSISTENT_VARIANTS)
def test_every_kernel_variant_matches_oracle(engine, kind, lpc, depth, hints, locality):
    """Each kernel variant (kind, lanes per clause, loads in flight or clause
    slots, cache hints) is bit-exact, including slot counts that do not fill
    the last slot block and clauses longer than a tile, in length order and
    in variable-range order (8 ranges of 2^11 variables)."""
    wl = W.make_scale(seed=11, n_vars=2 ** 14, n_clauses=20_000, n_solvers=13)
    # a few clauses longer than a staged tile (512 literals)
    rng = np.random.default_rng(5)
    extra_l, extra_o = W.distinct_var_clauses(rng, np.array([513, 700, 2000]), wl.n_vars)
    lits = np.concatenate([wl.lits, extra_l])
    offsets = np.concatenate([wl.offsets, wl.offsets[-1] + extra_o[1:]])
    wl = W.Workload(wl.name, wl.n_vars, lits, offsets, wl.state, wl.start, wl.solver_of_word, wl.n_solvers)
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    engine.set_variant(kind, lpc, depth, hints)
    engine.set_locality(locality)
    try:
        gpu = _gpu_reports(engine, wl)
        assert engine.locality_shift == locality
    finally:
        engine.set_variant()
        engine.set_locality(-1)
    _assert_same(gpu, ref, wl)


def _live_reference(live, state, start):
    """Oracle reports of a {id: literals} database, with clause = id."""
    ids = sorted(live)
    lits = np.concatenate([np.asarray(live[i], np.int32) for i in ids])
    offsets = np.zeros(len(ids) + 1, np.int64)
    offsets[1:] = np.cumsum([len(live[i]) for i in ids])
    ref = oracle.check(lits, offsets, state, start)
    ref["clause"] = np.asarray(ids, np.uint32)[ref["clause"]]
    return np.sort(ref, order=["clause", "word"])


@pytest.mark.parametrize("locality", [0, 11])
@pytest.mark.parametrize("kind", [-1, 0, 2])
def test_database_churn_matches_oracle(engine, kind, locality):
    """Deletes (tombstones), appends with ids, and a compaction: every pass
    reports exactly the live clauses' reports, keyed by clause id, in length
    order and in variable-range order (2 ranges of 2^11 variables)."""
    import gpusharesat_gb300 as g
    rng = np.random.default_rng(31)
    base = W.make_scale(seed=31, n_vars=2 ** 12, n_clauses=20000, n_solvers=32)
    live = {c: base.lits[base.offsets[c]:base.offsets[c + 1]].tolist() for c in range(base.n_clauses)}
    engine.set_variant(kind, 0, 2, 0)
    engine.set_locality(locality)
    engine.set_db(base.lits, base.offsets)
    engine.set_state(base.state, base.start, base.solver_of_word)
    next_id = base.n_clauses
    for step in range(4):
        gone = rng.choice(sorted(live), size=1000, replace=False)
        engine.delete(gone)
        for i in gone:
            del live[int(i)]
        lengths = W.lengths_small(rng, 1000)
        lits, offs = W.distinct_var_clauses(rng, lengths, base.n_vars)
        ids = np.arange(next_id, next_id + 1000) if step % 2 else None
        engine.append_db(lits, offs, ids)
        for k in range(1000):
            live[next_id + k] = lits[offs[k]:offs[k + 1]].tolist()
        next_id += 1000
        if step == 2:
            engine.compact()
            assert engine.clause_count == len(live)
        assert engine.live_count == len(live)
        got = np.sort(engine.check(), order=["clause", "word"])
        ref = _live_reference(live, base.state, base.start)
        assert len(got) == len(ref)
        for f in ("clause", "word", "mask"):
            np.testing.assert_array_equal(got[f], ref[f])
    with pytest.raises(g.GssError):
        engine.delete([10 ** 8])
    engine.set_variant()
    engine.set_locality(-1)


def test_persistent_graph_replays_across_passes(engine):
    """The persistent kernel run as a captured graph: one capture serves
    passes whose database and assignments change; every pass is exact."""
    import gpusharesat_gb300 as g
    rng = np.random.default_rng(41)
    base = W.make_scale(seed=41, n_vars=2 ** 12, n_clauses=20000, n_solvers=40)
    live = {c: base.lits[base.offsets[c]:base.offsets[c + 1]].tolist() for c in range(base.n_clauses)}
    engine.set_variant(g.KERNEL_WIDE4, 8, 2, g.VARIANT_PERSISTENT)
    engine.set_graph(True)
    try:
        engine.set_db(base.lits, base.offsets)
        engine.set_capacity(1 << 22)
        captures0 = engine.graph_captures
        next_id = base.n_clauses
        for step in range(3):
            state = W.random_state(rng, base.n_vars, base.n_words, rng.uniform(0.4, 0.9, 32 * base.n_words))
            start = rng.integers(0, 2 ** 32, size=base.n_words, dtype=np.uint32)
            engine.set_state(state, start, base.solver_of_word)
            gone = rng.choice(sorted(live), size=500, replace=False)
            engine.delete(gone)
            for i in gone:
                del live[int(i)]
            lits, offs = W.distinct_var_clauses(rng, W.lengths_small(rng, 500), base.n_vars)
            engine.append_db(lits, offs)
            for k in range(500):
                live[next_id + k] = lits[offs[k]:offs[k + 1]].tolist()
            next_id += 500
            got = np.sort(engine.check(), order=["clause", "word"])
            ref = _live_reference(live, state, start)
            assert len(got) == len(ref)
            for f in ("clause", "word", "mask"):
                np.testing.assert_array_equal(got[f], ref[f])
        assert engine.graph_captures - captures0 == 1
    finally:
        engine.set_graph(False)
        engine.set_capacity(0)
        engine.set_variant()


# ---- the bucketed kernel: a lane layout per length class ----

def _plan_engine(wl, locality=-1):
    import gpusharesat_gb300 as g
    eng = g.Engine(0)
    eng.set_locality(locality)
    eng.set_db(wl.lits, wl.offsets)
    eng.set_variant(g.KERNEL_WIDE4, 8, 2, g.VARIANT_PERSISTENT)
    eng.set_state(wl.state, wl.start, wl.solver_of_word)
    return eng


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_length_plan_matches_oracle(lib, seed):
    """Random layouts per length class, 32 and 96 words: the bucketed pass
    reports exactly what the oracle reports."""
    import gpusharesat_gb300 as g
    rng = np.random.default_rng(seed)
    n_solvers = 16 if seed < 2 else 48
    wl = W.make_scale(seed=40 + seed, n_vars=2 ** 13, n_clauses=30000, n_solvers=n_solvers)
    if seed == 2:  # two words per solver, as the batching workload
        wl = W.make_batching(seed=42, n_vars=2 ** 13, n_clauses=30000, n_solvers=48)
    eng = _plan_engine(wl, locality=11 if seed else 0)  # variable ranges: 4 ranges of 2^11
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    for _ in range(3):
        layouts = rng.choice(g.LAYOUTS, size=4).tolist()
        eng.set_length_plan((4, 12, 32, 1 << 30), layouts)
        _assert_same(g.sort_reports(eng.check()), ref, wl)
    eng.set_length_plan()
    _assert_same(g.sort_reports(eng.check()), ref, wl)
    eng.close()


def test_length_plan_skips_classes(lib):
    import gpusharesat_gb300 as g
    wl = W.make_scale(seed=44, n_vars=2 ** 13, n_clauses=30000, n_solvers=32)
    eng = _plan_engine(wl)
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    lens = np.diff(wl.offsets)
    eng.set_length_plan((4, 12, 32, 1 << 30), [g.LAYOUT_SKIP, g.LAYOUT_4x8_G2, g.LAYOUT_SKIP, g.LAYOUT_1x32_G1])
    keep = ((lens > 4) & (lens <= 12)) | (lens > 32)
    _assert_same(g.sort_reports(eng.check()), ref[keep[ref["clause"]]], wl)
    eng.close()


def test_length_plan_with_churn_and_graph(lib):
    """Appended batches (each sorted) make many position ranges; deletes are
    skipped in the kernel; the plan is rebuilt after each change and the
    pass graph replays it."""
    import gpusharesat_gb300 as g
    rng = np.random.default_rng(45)
    base = W.make_scale(seed=45, n_vars=2 ** 12, n_clauses=20000, n_solvers=32)
    live = {c: base.lits[base.offsets[c]:base.offsets[c + 1]].tolist() for c in range(base.n_clauses)}
    eng = _plan_engine(base, locality=11)  # 2 ranges of 2^11 variables: a run per (range pair, class)
    eng.set_graph(True)
    eng.set_length_plan((3, 8, 20, 1 << 30), [g.LAYOUT_1x32_G2, g.LAYOUT_2x16_G1, g.LAYOUT_4x8_G2, g.LAYOUT_4x8_G1])
    next_id = base.n_clauses
    for step in range(4):
        gone = rng.choice(sorted(live), size=800, replace=False)
        eng.delete(gone)
        for i in gone:
            del live[int(i)]
        lits, offs = W.distinct_var_clauses(rng, W.lengths_small(rng, 900), base.n_vars)
        eng.append_db(lits, offs)
        for k in range(900):
            live[next_id + k] = lits[offs[k]:offs[k + 1]].tolist()
        next_id += 900
        got = np.sort(eng.check(), order=["clause", "word"])
        ref = _live_reference(live, base.state, base.start)
        assert len(got) == len(ref)
        for f in ("clause", "word", "mask"):
            np.testing.assert_array_equal(got[f], ref[f])
    assert eng.graph_captures >= 1
    eng.close()
