"""The learned order's lazy history against the eager one, on the CPU.

The device keeps a clause's 8-pass report history as of the pass of its last
report and writes a record only in the passes that reported the clause
(order.cu: fold_kernel, hist_at); readers shift the history to the pass they
need. This restates that representation in Python and checks that it gives,
at every pass, the same history bytes, totals, last-report passes and
features as the eager history of the oracle (oracle/mlp.py History, which
shifts every clause's history every pass).
"""
import numpy as np

from oracle import mlp


def hist_at(hist, last, t):
    """The history word with byte 0 = pass t from one whose byte 0 is pass
    `last` (no report after it); all zero for a clause that never reported."""
    if last < 0:
        return 0
    d = t - last
    if d >= 8:
        return 0
    if d <= 0:
        return hist
    return (hist << (8 * d)) & 0xFFFFFFFFFFFFFFFF


class Lazy:
    def __init__(self):
        self.hist, self.total, self.last = {}, {}, {}

    def born(self, ids):
        for i in ids:
            self.hist.setdefault(i, 0)
            self.total.setdefault(i, 0)
            self.last.setdefault(i, -1)

    def fold(self, p, counts):
        """Only the clauses reported in pass p are written."""
        for i, c in counts.items():
            if c:
                self.hist[i] = hist_at(self.hist[i], self.last[i], p) | min(c, 255)
                self.total[i] += c
                self.last[i] = p

    def bytes_at(self, i, t):
        h = hist_at(self.hist[i], self.last[i], t)
        return [(h >> (8 * k)) & 0xFF for k in range(8)]


def test_lazy_history_equals_eager_history():
    rng = np.random.default_rng(3)
    n, passes = 300, 40
    eager, lazy = mlp.History(), Lazy()
    eager.born(range(n), -1)
    lazy.born(range(n))
    lengths = rng.integers(2, 40, size=n)
    lbd = rng.integers(0, 30, size=n)
    rate = rng.beta(0.5, 4, size=n)
    for p in range(passes):
        # sparse reports, some above 255 slots (saturated bytes), long gaps
        counts = {int(i): int(rng.integers(1, 400)) for i in range(n) if rng.random() < rate[i] * (p % 11 != 3)}
        eager.record(p, counts)
        lazy.fold(p, counts)
        now = p + 1  # features of a prediction for the pass after `now`, history through pass now - 1
        for i in range(n):
            assert lazy.bytes_at(i, now - 1) == eager.hist[i], (p, i)
            assert lazy.total[i] == eager.total[i] and lazy.last[i] == eager.last[i]
            last = lazy.last[i]
            got = mlp.features(int(lengths[i]), int(lbd[i]), now - eager.birth[i], lazy.bytes_at(i, now - 1),
                               lazy.total[i], -1 if last < 0 else now - last)
            want = eager.features(i, int(lengths[i]), int(lbd[i]), now)
            assert np.array_equal(got, want), (p, i)


def test_hist_at_shifts_out_after_eight_passes():
    assert hist_at(0x05, 3, 3) == 0x05
    assert hist_at(0x05, 3, 4) == 0x0500
    assert hist_at(0x0102, 3, 10) == 0x02 << 56
    assert hist_at(0x0102, 3, 11) == 0
    assert hist_at(0xFF, -1, 5) == 0
