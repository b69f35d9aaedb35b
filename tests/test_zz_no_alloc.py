"""gss_check_noalloc, the check pass for callers that cannot allocate device
memory (for instance a solver that gave its whole GPU budget to its own pool
at start-up): the test allocates every input and output itself, calls the
entry point twice in a row, and each time gets exactly the reports of the
engine's own pass with the same kernel. Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted(rep):
    order = np.lexsort((rep["word"], rep["clause"]))
    return rep[order]


def test_noalloc_matches_engine_on_two_calls(lib):
    import torch

    import gpusharesat_gb300 as g
    from gpusharesat_gb300 import workloads as W

    # 40 solvers: two blocks of 32 words, the second one partly padding
    wl = W.make_scale(seed=21, n_vars=2 ** 14, n_clauses=40_000, n_solvers=40)
    eng = g.Engine(0)
    try:
        eng.set_variant(g.KERNEL_WIDE4, 8, 2, 0)
        eng.set_db(wl.lits, wl.offsets)
        eng.set_state(wl.state, wl.start, wl.solver_of_word)
        ref = _sorted(eng.check())
    finally:
        eng.close()
    assert len(ref) > 0

    n_blocks = (wl.n_words + 31) // 32
    wide = np.zeros((wl.n_vars, n_blocks * 32, 2), np.uint32)
    wide[:, :wl.n_words] = wl.state
    wide = np.ascontiguousarray(wide.reshape(wl.n_vars, n_blocks, 32, 2).transpose(1, 0, 2, 3))
    start = np.zeros(n_blocks * 32, np.uint32)
    start[:wl.n_words] = wl.start
    sow = np.zeros(n_blocks * 32, np.int32)
    sow[:wl.n_words] = wl.solver_of_word

    dev = torch.device("cuda", 0)
    d_lits = torch.from_numpy(wl.lits).to(dev)
    d_offsets = torch.from_numpy(wl.offsets).to(dev)
    d_state = torch.from_numpy(wide.view(np.int32)).to(dev)
    d_start = torch.from_numpy(start.view(np.int32)).to(dev)
    d_sow = torch.from_numpy(sow).to(dev)
    n_parts = 16
    cap = (2 * len(ref)) // n_parts + 1024
    d_out = torch.zeros(n_parts * cap * 4, dtype=torch.int32, device=dev)
    d_counts = torch.zeros(n_parts, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    lib.gss_check_noalloc.restype = ctypes.c_int
    vp = ctypes.c_void_p
    u32 = ctypes.c_uint32
    lib.gss_check_noalloc.argtypes = [vp, vp, u32, vp, u32, u32, vp, vp, vp, u32, u32, vp, vp]

    for call in range(2):
        d_out.zero_()
        d_counts.fill_(-1)
        rc = lib.gss_check_noalloc(vp(d_lits.data_ptr()), vp(d_offsets.data_ptr()), wl.n_clauses,
                                   vp(d_state.data_ptr()), wl.n_vars, n_blocks, vp(d_start.data_ptr()),
                                   vp(d_sow.data_ptr()), vp(d_out.data_ptr()), n_parts, cap,
                                   vp(d_counts.data_ptr()), vp(stream))
        assert rc == 0, lib.gss_last_error()
        torch.cuda.synchronize(dev)
        counts = d_counts.cpu().numpy().astype(np.int64)
        assert (counts <= cap).all(), counts
        out = d_out.cpu().numpy().view(g.REPORT_DTYPE).reshape(n_parts, cap)
        got = _sorted(np.concatenate([out[p, :counts[p]] for p in range(n_parts)]))
        assert len(got) == len(ref), (call, len(got), len(ref))
        for f in ("clause", "word", "mask", "solver"):
            np.testing.assert_array_equal(got[f], ref[f], err_msg="call %d field %s" % (call, f))


def test_noalloc_rejects_too_many_partitions(lib):
    vp = ctypes.c_void_p
    lib.gss_check_noalloc.restype = ctypes.c_int
    lib.gss_check_noalloc.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp,
                                      ctypes.c_uint32, ctypes.c_uint32, vp, vp]
    rc = lib.gss_check_noalloc(None, None, 0, None, 0, 0, None, None, None, 65, 0, None, None)
    assert rc == -1
    assert b"64" in lib.gss_last_error()
