"""Properties of the seeded workload generators that the measurements rely
on, checked with the C oracle on small sizes (CPU)."""
import numpy as np

import oracle
from gpusharesat_gb300 import workloads as W


def test_model_clauses_never_report_under_the_base_state(oracle_lib):
    d = W.make_learned(seed=9, n_vars=2 ** 13, n_clauses=8000, n_words=2, stream=500)
    n = d["n_clauses"] + d["stream"]
    lits, offsets = d["lits"], d["offsets"]
    assert offsets.shape[0] == n + 1
    # at least two literals true under the model in every clause
    var, sign = lits >> 1, lits & 1
    true_lit = sign == (1 - d["model"][var])
    per_clause = np.add.reduceat(true_lit.astype(np.int64), offsets[:-1])
    assert per_clause.min() >= 2
    rep = oracle.check(lits, offsets, d["state"], np.full(d["n_words"], 0xFFFFFFFF, np.uint32))
    assert len(rep) == 0
    # rates and LBD
    assert 0 < d["rate"].mean() < 0.05
    lens = np.diff(offsets)
    assert np.all((d["lbd"] >= 1) & (d["lbd"] <= lens))
    hi = d["rate"] > np.quantile(d["rate"], 0.9)
    assert (d["lbd"][hi] / lens[hi]).mean() < (d["lbd"][~hi] / lens[~hi]).mean()


def test_dump_round_trip(tmp_path, oracle_lib):
    wl = W.make_small(seed=4, n_clauses=3000)
    path = str(tmp_path / "small.npz")
    W.save(wl, path)
    back = W.load(path)
    assert back.name == wl.name and back.n_vars == wl.n_vars and back.n_solvers == wl.n_solvers
    for f in ("lits", "offsets", "state", "start", "solver_of_word", "planted"):
        assert np.array_equal(getattr(back, f), getattr(wl, f)), f
    a = oracle.check(wl.lits, wl.offsets, wl.state, wl.start)
    b = oracle.check(back.lits, back.offsets, back.state, back.start)
    assert np.array_equal(a, b)
