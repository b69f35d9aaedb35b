"""CPU oracle for the clause-check pass (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker. The shipped
library (``gpusharesat_gb300``) never imports it and has no CPU fallback.

``check()`` wraps ``oracle/check.c``, a C restatement of the report rule of
gpuShareLib/GpuRunner.cu:34-89 (see that file's header for the mapping).
``sharer_model`` restates the host-side state machine of the
``GpuClauseSharer`` API in plain Python for small cases. ``mlp`` restates
the learned scan order's scorer (forward, loss, gradient, Adam, BF16
inference) and its per-clause features in float64 numpy.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

REPORT_DTYPE = np.dtype([("clause", "<u4"), ("word", "<u4"), ("mask", "<u4"), ("pad", "<u4")])


def build():
    """Compiles liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.oracle_check.restype = ctypes.c_int64
        lib.oracle_check.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
            ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
        ]
        lib.oracle_check_one.restype = ctypes.c_uint32
        lib.oracle_check_one.argtypes = [
            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
        ]
        lib.oracle_check_digest.restype = ctypes.c_int
        lib.oracle_check_digest.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
        ]
        _LIB = lib
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def check(lits, offsets, state, start_mask, n_threads=1):
    """Reports of every clause against every started slot.

    lits: int32 [n_lits]; offsets: int64 [n_clauses + 1];
    state: uint32 [n_vars, n_words, 2] (isDef, isTrue);
    start_mask: uint32 [n_words].
    Returns a structured array (clause, word, mask, pad) in (clause, word) order.
    """
    lits = np.ascontiguousarray(lits, dtype=np.int32)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    state = np.ascontiguousarray(state, dtype=np.uint32)
    start_mask = np.ascontiguousarray(start_mask, dtype=np.uint32)
    n_vars, n_words = state.shape[0], state.shape[1]
    n_clauses = offsets.shape[0] - 1
    cap = max(1024, n_clauses // 16)
    while True:
        out = np.zeros(cap, dtype=REPORT_DTYPE)
        n = _lib().oracle_check(_ptr(lits), _ptr(offsets), n_clauses, _ptr(state), n_vars,
                                n_words, _ptr(start_mask), int(n_threads), _ptr(out), cap)
        if n < 0:
            raise RuntimeError("oracle_check failed")
        if n <= cap:
            return out[:n]
        cap = int(n)


def check_one(lits, is_def, is_true, start=0xFFFFFFFF):
    """The rule for one clause and one 32-slot word (values given per literal)."""
    lits = np.ascontiguousarray(lits, dtype=np.int32)
    is_def = np.ascontiguousarray(is_def, dtype=np.uint32)
    is_true = np.ascontiguousarray(is_true, dtype=np.uint32)
    return int(_lib().oracle_check_one(_ptr(lits), lits.shape[0], _ptr(is_def), _ptr(is_true),
                                       ctypes.c_uint32(start)))


def expand(reports):
    """(clause, word, mask) records -> sorted int64 array of (clause, word, slot)."""
    if len(reports) == 0:
        return np.zeros((0, 3), dtype=np.int64)
    masks = reports["mask"].astype(np.uint64)
    bits = ((masks[:, None] >> np.arange(32, dtype=np.uint64)[None, :]) & 1).astype(bool)
    rows, slots = np.nonzero(bits)
    out = np.stack([reports["clause"][rows].astype(np.int64),
                    reports["word"][rows].astype(np.int64),
                    slots.astype(np.int64)], axis=1)
    order = np.lexsort((out[:, 2], out[:, 1], out[:, 0]))
    return out[order]


def check_digest(lits, offsets, state, start_mask, ids=None, n_threads=1):
    """(record count, digest) of the oracle's reports, for passes too large to
    compare record by record: the digest is the wrapping uint64 sum over
    (clause, word, mask) records of mix(mix((id << 32) | word) ^ mask), mix =
    the SplitMix64 finaliser, id = ids[clause] (the clause index when ids is
    None). It does not depend on record order; report_digest() computes the
    same from any report array."""
    lits = np.ascontiguousarray(lits, dtype=np.int32)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    state = np.ascontiguousarray(state, dtype=np.uint32)
    start_mask = np.ascontiguousarray(start_mask, dtype=np.uint32)
    ids_a = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
    count = ctypes.c_uint64()
    digest = ctypes.c_uint64()
    rc = _lib().oracle_check_digest(_ptr(lits), _ptr(offsets), offsets.shape[0] - 1,
                                    None if ids_a is None else _ptr(ids_a), _ptr(state), state.shape[1],
                                    _ptr(start_mask), int(n_threads), ctypes.byref(count), ctypes.byref(digest))
    if rc != 0:
        raise RuntimeError("oracle_check_digest failed")
    return int(count.value), int(digest.value)


def _mix64(z):
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def report_digest(clause, word, mask, chunk=1 << 25):
    """(record count, digest) of report records given as arrays of clause ids,
    words and masks, in any order (see check_digest)."""
    n = int(len(clause))
    total = np.uint64(0)
    with np.errstate(over="ignore"):
        for b in range(0, n, chunk):
            c = np.asarray(clause[b:b + chunk]).astype(np.uint64)
            w = np.asarray(word[b:b + chunk]).astype(np.uint64)
            m = np.asarray(mask[b:b + chunk]).astype(np.uint64)
            h = _mix64(_mix64((c << np.uint64(32)) | w) ^ m)
            total = total + np.add.reduce(h, dtype=np.uint64)
    return n, int(total)
