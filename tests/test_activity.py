"""The reduceDb policy (clause activity and removal thresholds) against the
reference's known answers, glucose-syrup/test/ClauseActivityLbdTest.cu.
Host code only: runs without a GPU."""
import math

import pytest

RESCALE = 1e19


@pytest.fixture(scope="module")
def G(lib):
    import gpusharesat_gb300 as g
    return g


def _set_lbd_and_act(a, lbd, act):
    """setLbdAndAct (ClauseActivityLbdTest.cu:97-111): a clause with that lbd,
    bumped act - 1 times."""
    i = a.add(lbd)
    for _ in range(act - 1):
        a.bump(i)
    return i


def test_init_act(G):  # :59-67
    a = G.ClauseActivity(1.0)
    assert abs(1.0 - a.get(a.add(1))) < 0.01


def test_bump_act(G):  # :69-81
    a = G.ClauseActivity(1.0)
    i = a.add(1)
    a.bump(i)
    assert abs(2.0 - a.get(i)) < 0.01


def test_decay(G):  # :83-100
    a = G.ClauseActivity(0.5)
    i = a.add(1)
    assert abs(2.0 - a.get(i)) < 0.01
    a.decay()
    a.bump(i)
    assert abs(6.0 - a.get(i)) < 0.01


@pytest.mark.parametrize("acts,lo,hi,n", [
    ([1, 2, 3], 2.0, 2.1, 2), ([1, 2, 3], -0.1, 0.1, 0), ([1, 2, 3], 3.0, 3.1, 3),   # :164-172
    ([1, 1, 1, 3, 3, 100], 1.0, 1.1, 3),                                            # :174-183
    ([1, 1, 1, 1, 10], 1.0, 1.1, 2),                                                # :185-193
])
def test_approx_nth_act(G, acts, lo, hi, n):
    a = G.ClauseActivity(1.0)
    for x in acts:
        _set_lbd_and_act(a, 3, x)
    v = a.approx_nth(3, 4, n)
    assert lo < v <= hi


@pytest.mark.parametrize("lbd_acts,lo,hi,min_lim,max_lim,act_only", [
    ([(2, 1), (2, 2), (3, 4), (4, 6)], -0.1, 1.0, 2, 3, False),                      # testRemLbdAct :195-203
    ([(2, 1), (3, 4), (3, 9), (4, 15)], 4.0, 9.0, 3, 4, False),                      # testRemLbdAct2 :205-212
    ([(2, 1), (2, 3), (2, 4), (2, 5), (3, 1)], -0.1, 1.0, 2, 3, False),              # testDontRemoveLbd2Clauses :214-222
    ([(2, 1), (8, 5)], 1, 5, 0, 100, True),                                          # testActOnly :224-229
])
def test_removing_thresholds(G, lbd_acts, lo, hi, min_lim, max_lim, act_only):
    a = G.ClauseActivity(1.0)
    for lbd, act in lbd_acts:
        _set_lbd_and_act(a, lbd, act)
    mn, mx, act = a.removing_thresholds(act_only, len(lbd_acts))
    assert (mn, mx) == (min_lim, max_lim)
    assert lo < act <= hi


def test_act_only_huge_differences(G):  # :231-254
    decay = 0.5
    a = G.ClauseActivity(decay)
    _set_lbd_and_act(a, 3, 1)  # activity 2
    _set_lbd_and_act(a, 3, 2)  # activity 4
    c = int(math.log(RESCALE / 100) / math.log(1 / decay))
    for _ in range(c):
        a.decay()
    _set_lbd_and_act(a, 3, 1)
    _, _, act = a.removing_thresholds(True, 3)
    assert 2 < act <= 4


def test_rescale(G):  # :256-274
    a = G.ClauseActivity(1 / (RESCALE * 10))
    i = a.add(1)
    assert abs(10 - a.get(i)) < 0.1
    a.decay()
    a.bump(i)
    assert abs(100 - a.get(i)) < 0.1
    a.bump(i)
    assert abs(200 - a.get(i)) < 0.1
