"""The CPU oracle against the reference's known-answer cases (CPU only)."""
import numpy as np
import pytest

import kat
import oracle
from gpusharesat_gb300 import workloads as W


@pytest.mark.parametrize("case", kat.load_cases(), ids=lambda c: c["name"])
def test_oracle_matches_reference_known_answers(oracle_lib, case):
    lits, offsets, state, start, sow = kat.case_inputs(case)
    got = oracle.expand(oracle.check(lits, offsets, state, start))
    np.testing.assert_array_equal(got, kat.expected_triples(case))


def test_rule_truth_table(oracle_lib):
    # every (value, sign) pair for a 2-literal clause, one slot per combination
    vals = ["T", "F", "U"]
    combos = [(a, b) for a in vals for b in vals]
    is_def = np.zeros(2, np.uint32)
    is_true = np.zeros(2, np.uint32)
    for s, (a, b) in enumerate(combos):
        for i, ch in enumerate((a, b)):
            if ch != "U":
                is_def[i] |= np.uint32(1 << s)
            if ch == "T":
                is_true[i] |= np.uint32(1 << s)
    m = oracle.check_one([0, 2], is_def, is_true, (1 << len(combos)) - 1)
    for s, (a, b) in enumerate(combos):
        n_false = (a == "F") + (b == "F")
        n_undef = (a == "U") + (b == "U")
        want = n_false == 2 or (n_false == 1 and n_undef == 1)
        assert bool((m >> s) & 1) == want, (a, b)


def test_threads_agree(oracle_lib):
    wl = W.make_small(seed=4, n_clauses=30000)
    a = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=1)
    b = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=7)
    assert len(a) == len(b)
    for f in ("clause", "word", "mask"):
        np.testing.assert_array_equal(a[f], b[f])


def test_planted_clauses_behave(oracle_lib):
    """Planted clauses: all-false or one-undefined plants report for their slot."""
    wl = W.make_small(seed=0)
    rep = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    reported = set(rep["clause"].tolist())
    # at least half the plants are 'last literal false' and must report
    assert sum(int(c) in reported for c in wl.planted) >= len(wl.planted) // 2


def test_unstarted_slots_are_ignored(oracle_lib):
    lits = np.array([0], np.int32)
    offsets = np.array([0, 1], np.int64)
    state = np.zeros((1, 1, 2), np.uint32)  # undefined everywhere: a unit reports
    got = oracle.check(lits, offsets, state, np.array([0x5], np.uint32))
    assert len(got) == 1 and got["mask"][0] == 0x5


def test_digest_matches_records_and_sees_a_changed_record(oracle_lib):
    """The order-independent digest the full-size GPU tests compare: the
    oracle's in-C digest equals the digest of its own records (in any order,
    with clause ids mapped), and one changed record changes it."""
    wl = W.make_small(seed=3, n_clauses=20000)
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=4)
    ids = (np.arange(wl.n_clauses, dtype=np.uint32) * 7 + 3).astype(np.uint32)
    want = oracle.check_digest(wl.lits, wl.offsets, wl.state, wl.start, ids=ids, n_threads=3)
    perm = np.random.default_rng(0).permutation(len(ref))
    shuffled = ref[perm]
    assert oracle.report_digest(ids[shuffled["clause"]], shuffled["word"], shuffled["mask"]) == want
    assert want[0] == len(ref)
    bad = shuffled.copy()
    bad["mask"][5] ^= np.uint32(1 << 7)
    assert oracle.report_digest(ids[bad["clause"]], bad["word"], bad["mask"]) != want
    assert oracle.check_digest(wl.lits, wl.offsets, wl.state, wl.start, n_threads=1) == \
        oracle.report_digest(ref["clause"], ref["word"], ref["mask"])
