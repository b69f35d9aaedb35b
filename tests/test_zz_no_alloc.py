"""gss_check_noalloc, the check pass for callers that cannot allocate device
memory: a solver process that hands its whole GPU budget to its own pool at
start-up (a cudaMalloc would then fail or eat into that budget), or a
latency-bound loop that must not stall in the allocator.

The test allocates every input and output itself (torch), calls the entry
point through the C ABI twice in a row, and each time compares the reports,
record by record, with the CPU oracle. It also covers the documented overflow
contract (a count above the capacity means overflow, and the records written
are a subset of the full set), the empty pass (all counts zero) and the
refused arguments. Kept in its own file, collected last, so that a run that
stops at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

vp = ctypes.c_void_p
u32 = ctypes.c_uint32


def _bind(lib):
    lib.gss_check_noalloc.restype = ctypes.c_int
    lib.gss_check_noalloc.argtypes = [vp, vp, u32, vp, u32, u32, vp, vp, vp, u32, u32, vp, vp]
    return lib.gss_check_noalloc


def _sorted(clause, word, mask):
    order = np.lexsort((word, clause))
    return clause[order], word[order], mask[order]


class _Inputs:
    """The workload in the wide layout, on the device."""

    def __init__(self, wl):
        import torch
        self.wl = wl
        self.n_blocks = (wl.n_words + 31) // 32
        wide = np.zeros((wl.n_vars, self.n_blocks * 32, 2), np.uint32)
        wide[:, :wl.n_words] = wl.state
        wide = np.ascontiguousarray(wide.reshape(wl.n_vars, self.n_blocks, 32, 2).transpose(1, 0, 2, 3))
        start = np.zeros(self.n_blocks * 32, np.uint32)
        start[:wl.n_words] = wl.start
        sow = np.zeros(self.n_blocks * 32, np.int32)
        sow[:wl.n_words] = wl.solver_of_word
        self.dev = torch.device("cuda", 0)
        self.lits = torch.from_numpy(wl.lits).to(self.dev)
        self.offsets = torch.from_numpy(wl.offsets).to(self.dev)
        self.state = torch.from_numpy(wide.view(np.int32)).to(self.dev)
        self.start = torch.from_numpy(start.view(np.int32)).to(self.dev)
        self.sow = torch.from_numpy(sow).to(self.dev)

    def run(self, fn, n_parts, cap, n_clauses=None):
        """One call; returns (counts, out[n_parts, cap] records)."""
        import torch
        import gpusharesat_gb300 as g
        out = torch.zeros(max(n_parts * cap * 4, 4), dtype=torch.int32, device=self.dev)
        counts = torch.full((n_parts,), -1, dtype=torch.int32, device=self.dev)
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        n = self.wl.n_clauses if n_clauses is None else n_clauses
        rc = fn(vp(self.lits.data_ptr()), vp(self.offsets.data_ptr()), n, vp(self.state.data_ptr()),
                self.wl.n_vars, self.n_blocks, vp(self.start.data_ptr()), vp(self.sow.data_ptr()),
                vp(out.data_ptr()), n_parts, cap, vp(counts.data_ptr()), vp(stream))
        assert rc == 0, g.load().gss_last_error()
        torch.cuda.synchronize(self.dev)
        recs = out.cpu().numpy().view(g.REPORT_DTYPE)[:n_parts * cap].reshape(n_parts, cap)
        return counts.cpu().numpy().astype(np.int64), recs


def _workload():
    from gpusharesat_gb300 import workloads as W
    # 40 solvers: two blocks of 32 words, the second one partly padding
    return W.make_scale(seed=21, n_vars=2 ** 14, n_clauses=40_000, n_solvers=40)


def test_noalloc_matches_oracle_on_two_calls(lib):
    fn = _bind(lib)
    wl = _workload()
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=8)
    assert len(ref) > 0
    inp = _Inputs(wl)
    n_parts = 16
    cap = (2 * len(ref)) // n_parts + 1024
    for call in range(2):
        counts, recs = inp.run(fn, n_parts, cap)
        assert (counts >= 0).all() and (counts <= cap).all(), counts
        got = np.concatenate([recs[p, :counts[p]] for p in range(n_parts)])
        c, w, m = _sorted(got["clause"], got["word"], got["mask"])
        assert len(c) == len(ref), (call, len(c), len(ref))
        np.testing.assert_array_equal(c, ref["clause"], err_msg="call %d clause" % call)
        np.testing.assert_array_equal(w, ref["word"], err_msg="call %d word" % call)
        np.testing.assert_array_equal(m, ref["mask"], err_msg="call %d mask" % call)
        np.testing.assert_array_equal(got["solver"], wl.solver_of_word[got["word"]])


def test_noalloc_overflow_then_rerun(lib):
    """A capacity far below the report count: counts above the capacity show
    the overflow, the records written are real reports, and a rerun with
    room for every partition's count gives the oracle's set."""
    fn = _bind(lib)
    wl = _workload()
    ref = oracle.check(wl.lits, wl.offsets, wl.state, wl.start, n_threads=8)
    key = lambda c, w, m: set(zip(c.tolist(), w.tolist(), m.tolist()))
    ref_set = key(ref["clause"], ref["word"], ref["mask"])
    inp = _Inputs(wl)
    n_parts = 8
    counts, recs = inp.run(fn, n_parts, 64)
    assert counts.sum() == len(ref)
    assert (counts > 64).any()
    part = np.concatenate([recs[p, :min(counts[p], 64)] for p in range(n_parts)])
    assert key(part["clause"], part["word"], part["mask"]) <= ref_set
    cap = int(counts.max())
    counts2, recs2 = inp.run(fn, n_parts, cap)
    assert (counts2 <= cap).all()
    got = np.concatenate([recs2[p, :counts2[p]] for p in range(n_parts)])
    assert len(got) == len(ref)
    assert key(got["clause"], got["word"], got["mask"]) == ref_set


def test_noalloc_empty_pass_counts_zero(lib):
    fn = _bind(lib)
    inp = _Inputs(_workload())
    counts, _ = inp.run(fn, 4, 16, n_clauses=0)
    np.testing.assert_array_equal(counts, np.zeros(4, np.int64))


def test_noalloc_rejects_bad_arguments(lib):
    fn = _bind(lib)
    rc = fn(None, None, 0, None, 0, 0, None, None, None, 65, 0, None, None)
    assert rc == -1
    assert b"64" in lib.gss_last_error()
    dummy = ctypes.c_uint32()
    p = vp(ctypes.addressof(dummy))
    rc = fn(p, p, 1, p, 0, 1, p, p, p, 1, 1, p, None)  # clauses over zero variables
    assert rc == -1
    assert b"0 variables" in lib.gss_last_error()
