"""Turns the known-answer cases of tests/golden/kat_check.json into engine inputs."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_cases():
    with open(os.path.join(HERE, "golden", "kat_check.json")) as f:
        return json.load(f)["cases"]


def case_inputs(case):
    """(lits, offsets, state, start, solver_of_word) for a case."""
    n_vars = case["n_vars"]
    clauses = case["clauses"]
    lits = np.array([l for c in clauses for l in c], dtype=np.int32)
    offsets = np.zeros(len(clauses) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(c) for c in clauses])
    words = case["words"]
    state = np.zeros((n_vars, len(words), 2), dtype=np.uint32)
    # undefined variables get random isTrue bits: the rule must ignore them
    rng = np.random.default_rng(12345)
    state[:, :, 1] = rng.integers(0, 2 ** 32, size=(n_vars, len(words)), dtype=np.uint32)
    start = np.zeros(len(words), dtype=np.uint32)
    for w, word in enumerate(words):
        for slot, vals in enumerate(word["slots"]):
            if vals is None:
                continue
            start[w] |= np.uint32(1 << slot)
            for v, ch in enumerate(vals):
                bit = np.uint32(1 << slot)
                if ch in "TF":
                    state[v, w, 0] |= bit
                    if ch == "T":
                        state[v, w, 1] |= bit
                    else:
                        state[v, w, 1] &= ~bit
    sow = np.array([word["solver"] for word in words], dtype=np.int32)
    return lits, offsets, state, start, sow


def expected_triples(case):
    e = np.array(case["expected"], dtype=np.int64).reshape(-1, 3)
    order = np.lexsort((e[:, 2], e[:, 1], e[:, 0]))
    return e[order]
