"""GB300-native clause checking for GpuShareSat-style clause sharing.

Python binding of the C ABI in include/gpusharesat.h, through ctypes. The
compute path is the CUDA library libgpusharesat.so built in-tree by
``gpusharesat_gb300.build``; there is no CPU fallback: loading fails loudly
when the library is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpusharesat.so")

GSS_OK = 0
GSS_ERR_INVALID = -1
GSS_ERR_CUDA = -2
GSS_ERR_NOMEM = -3
GSS_ERR_OVERFLOW = -4
GSS_ERR_STATE = -5
GSS_ERR_NOT_FOUND = -6

KERNEL_AUTO = -1
KERNEL_DIRECT = 0
KERNEL_TILED = 1
KERNEL_WIDE4 = 2
KERNEL_WIDE2 = 3
VARIANT_L2_HINT = 1
VARIANT_OCCUPANCY = 2
VARIANT_PIPELINED = 4
VARIANT_PERSISTENT = 8
# lane layouts of the bucketed kernel (Engine.set_length_plan)
LAYOUT_SKIP = -1
LAYOUT_4x8_G1 = 0
LAYOUT_4x8_G2 = 1
LAYOUT_2x16_G1 = 2
LAYOUT_2x16_G2 = 3
LAYOUT_1x32_G1 = 4
LAYOUT_1x32_G2 = 5
LAYOUTS = (LAYOUT_4x8_G1, LAYOUT_4x8_G2, LAYOUT_2x16_G1, LAYOUT_2x16_G2, LAYOUT_1x32_G1, LAYOUT_1x32_G2)

REPORT_DTYPE = np.dtype([("clause", "<u4"), ("word", "<u4"), ("mask", "<u4"), ("solver", "<u4")])
PACKED_REPORT_DTYPE = np.dtype([("clause", "<u4"), ("word", "<u4"), ("mask", "<u4")])
CELL_REPORT_DTYPE = np.dtype([("cell", "<u4"), ("mask", "<u4")])

_lib = None


class GssError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gpusharesat error %d: %s" % (code, msg))
        self.code = code


def _vp(x):
    return ctypes.c_void_p(x)


def _sig(lib, name, restype, *argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = list(argtypes)


def load():
    """Loads libgpusharesat.so (built by gpusharesat_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgpusharesat.so is not built (run gpusharesat_gb300.build.build()); "
                           "there is no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    c_int, c_i64, vp = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    _sig(lib, "gss_last_error", ctypes.c_char_p)
    _sig(lib, "gss_version", ctypes.c_char_p)
    _sig(lib, "gss_debug_fail_device_alloc", c_int, c_i64, c_int)
    _sig(lib, "gss_max_clause_len", c_int)
    _sig(lib, "gss_engine_create", c_int, c_int, vp)
    _sig(lib, "gss_engine_destroy", c_int, vp)
    _sig(lib, "gss_engine_set_stream", c_int, vp, vp)
    _sig(lib, "gss_engine_launch_count", c_i64, vp)
    _sig(lib, "gss_engine_set_timing", c_int, vp, c_int)
    _sig(lib, "gss_engine_set_graph", c_int, vp, c_int)
    _sig(lib, "gss_engine_graph_captures", c_i64, vp)
    _sig(lib, "gss_engine_kernel_time", c_int, vp, vp, vp)
    _sig(lib, "gss_engine_set_variant", c_int, vp, c_int, c_int, c_int, c_int)
    _sig(lib, "gss_db_set", c_int, vp, vp, vp, c_i64)
    _sig(lib, "gss_db_clause_count", c_i64, vp)
    _sig(lib, "gss_db_append", c_int, vp, vp, vp, c_i64, vp)
    _sig(lib, "gss_db_delete", c_int, vp, vp, c_i64)
    _sig(lib, "gss_db_compact", c_int, vp)
    _sig(lib, "gss_db_set_locality", c_int, vp, c_int)
    _sig(lib, "gss_db_locality_shift", c_int, vp)
    _sig(lib, "gss_db_live_count", c_i64, vp)
    _sig(lib, "gss_db_literal_count", c_i64, vp)
    _sig(lib, "gss_db_max_var", c_i64, vp)
    _sig(lib, "gss_state_set", c_int, vp, vp, c_i64, c_int, vp, vp, c_int)
    _sig(lib, "gss_check_set_capacity", c_int, vp, c_i64)
    _sig(lib, "gss_state_set_start", c_int, vp, vp, c_int)
    _sig(lib, "gss_check_launch", c_int, vp)
    _sig(lib, "gss_check_wait", c_int, vp, vp)
    _sig(lib, "gss_check_copy_reports", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_check_pass_host", c_int, vp, vp, c_i64, c_int, vp, vp, vp, c_i64, vp)
    _sig(lib, "gss_check_passes_host", c_int, vp, c_int, vp, c_i64, c_int, vp, vp, vp, vp, vp)
    _sig(lib, "gss_check_passes_host_packed", c_int, vp, c_int, vp, c_i64, c_int, vp, vp, vp, vp, vp)
    _sig(lib, "gss_check_passes_host_cells", c_int, vp, c_int, vp, c_i64, c_int, vp, vp, vp, vp, vp)
    _sig(lib, "gss_probe_gather", c_int, c_int, ctypes.c_uint64, c_int, c_int, vp, vp)
    _sig(lib, "gss_db_positions", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_engine_set_length_plan", c_int, vp, c_int, vp, vp)
    _sig(lib, "gss_order_params_default", None, vp)
    _sig(lib, "gss_order_enable", c_int, vp, vp)
    _sig(lib, "gss_order_disable", c_int, vp)
    _sig(lib, "gss_order_set_active", c_int, vp, c_int)
    _sig(lib, "gss_db_set_lbd", c_int, vp, vp, vp, c_i64)
    _sig(lib, "gss_check_wait_head", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_check_copy_tail", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_order_get_stats", c_int, vp, vp)
    _sig(lib, "gss_order_train", c_int, vp)
    _sig(lib, "gss_order_clause_features", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_order_scan_ranks", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_order_get_weights", c_int, vp, vp)
    _sig(lib, "gss_order_set_weights", c_int, vp, vp)
    _sig(lib, "gss_scorer_create", c_int, c_int, ctypes.c_uint64, vp)
    _sig(lib, "gss_scorer_destroy", c_int, vp)
    _sig(lib, "gss_scorer_get_weights", c_int, vp, vp)
    _sig(lib, "gss_scorer_set_weights", c_int, vp, vp)
    _sig(lib, "gss_scorer_infer", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_scorer_gradient", c_int, vp, vp, vp, c_i64, vp, vp)
    _sig(lib, "gss_scorer_train_step", c_int, vp, vp, vp, c_i64, ctypes.c_float, vp)
    _sig(lib, "gss_bench_plant", c_int, vp, vp, c_i64, vp, vp, vp, c_i64, c_int, ctypes.c_uint64, c_i64, c_int, vp)
    _lib = lib
    return lib


def debug_fail_device_alloc(min_bytes, count=1):
    """Testing hook: the next `count` device allocations of at least
    `min_bytes` fail as if the GPU were out of memory (made on the host;
    count=0 turns it off)."""
    _check(load().gss_debug_fail_device_alloc(int(min_bytes), int(count)))


def _check(rc):
    if rc != GSS_OK:
        raise GssError(rc, load().gss_last_error().decode())
    return rc


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Engine:
    """A device-resident clause database checked against assignment bit planes.

    Mirrors the device side of the reference's GpuRunner
    (gpuShareLib/GpuRunner.cu:211-345): load clauses, set the pass's
    assignments, launch the check, read the reports.
    """

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.gss_engine_create(device, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.gss_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        _check(self.lib.gss_engine_set_stream(self.h, _vp(stream_handle)))

    @property
    def launch_count(self):
        return int(self.lib.gss_engine_launch_count(self.h))

    def set_graph(self, on=True):
        _check(self.lib.gss_engine_set_graph(self.h, 1 if on else 0))

    @property
    def graph_captures(self):
        return int(self.lib.gss_engine_graph_captures(self.h))

    def set_timing(self, on=True):
        _check(self.lib.gss_engine_set_timing(self.h, 1 if on else 0))

    def kernel_time(self):
        """(total ms, launches) of the event-bracketed check kernels since the last call."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        _check(self.lib.gss_engine_kernel_time(self.h, ctypes.byref(ms), ctypes.byref(n)))
        return float(ms.value), int(n.value)

    def set_variant(self, kind=-1, lanes_per_clause=0, depth=2, flags=0):
        """kind: KERNEL_*; lanes_per_clause 0 = automatic; flags: VARIANT_* bits."""
        _check(self.lib.gss_engine_set_variant(self.h, kind, lanes_per_clause, depth, int(flags)))

    def set_db(self, lits, offsets):
        lits = np.ascontiguousarray(lits, dtype=np.int32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        _check(self.lib.gss_db_set(self.h, _ptr(lits), _ptr(offsets), offsets.shape[0] - 1))

    def append_db(self, lits, offsets, ids=None):
        lits = np.ascontiguousarray(lits, dtype=np.int32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        _check(self.lib.gss_db_append(self.h, _ptr(lits), _ptr(offsets), offsets.shape[0] - 1, _ptr(ids)))

    def delete(self, ids):
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        _check(self.lib.gss_db_delete(self.h, _ptr(ids), ids.shape[0]))

    def compact(self):
        _check(self.lib.gss_db_compact(self.h))

    def set_locality(self, range_log2=-1):
        """Database order from the next set_db/append_db/compact: -1 automatic
        variable ranges, 0 length order only, 11..31 ranges of 2^range_log2
        variables (see gss_db_set_locality)."""
        _check(self.lib.gss_db_set_locality(self.h, int(range_log2)))

    @property
    def locality_shift(self):
        """log2 of the variables per range of the current order (0: length order)."""
        return int(self.lib.gss_db_locality_shift(self.h))

    @property
    def live_count(self):
        return int(self.lib.gss_db_live_count(self.h))

    @property
    def clause_count(self):
        return int(self.lib.gss_db_clause_count(self.h))

    def set_state(self, state, start, solver_of_word=None):
        state = np.ascontiguousarray(state, dtype=np.uint32)
        start = np.ascontiguousarray(start, dtype=np.uint32)
        sow = None if solver_of_word is None else np.ascontiguousarray(solver_of_word, dtype=np.int32)
        _check(self.lib.gss_state_set(self.h, _ptr(state), state.shape[0], state.shape[1], _ptr(start),
                                      _ptr(sow), 0))

    def set_state_device(self, state_ptr, n_vars, n_words, start_ptr, sow_ptr=None):
        _check(self.lib.gss_state_set(self.h, _vp(state_ptr), n_vars, n_words, _vp(start_ptr),
                                      _vp(sow_ptr) if sow_ptr else None, 1))

    def set_start(self, start):
        start = np.ascontiguousarray(start, dtype=np.uint32)
        _check(self.lib.gss_state_set_start(self.h, _ptr(start), start.shape[0]))

    def set_capacity(self, records):
        _check(self.lib.gss_check_set_capacity(self.h, int(records)))

    def launch(self):
        _check(self.lib.gss_check_launch(self.h))

    def wait(self):
        n = ctypes.c_int64()
        rc = self.lib.gss_check_wait(self.h, ctypes.byref(n))
        if rc == GSS_ERR_OVERFLOW:
            return -1
        _check(rc)
        return int(n.value)

    def reports(self, out=None):
        """Reports of the pass just waited for (no relaunch), into `out` when
        given and large enough."""
        n = self.wait()
        if n < 0:
            raise GssError(GSS_ERR_OVERFLOW, "report queues overflowed")
        if out is None or out.shape[0] < max(n, 1):
            out = np.zeros(max(n, 1), dtype=REPORT_DTYPE)
        got = ctypes.c_int64()
        _check(self.lib.gss_check_copy_reports(self.h, _ptr(out), out.shape[0], ctypes.byref(got)))
        return out[:got.value]

    def check(self):
        """Runs one pass (re-running after an overflow) and returns the reports."""
        for _ in range(4):
            self.launch()
            n = self.wait()
            if n >= 0:
                out = np.zeros(max(n, 1), dtype=REPORT_DTYPE)
                got = ctypes.c_int64()
                _check(self.lib.gss_check_copy_reports(self.h, _ptr(out), out.shape[0], ctypes.byref(got)))
                return out[:got.value]
        raise GssError(GSS_ERR_OVERFLOW, "report queues kept overflowing")

    def set_length_plan(self, max_len=(), layouts=()):
        """Per-length-class lane layouts in one persistent launch (the
        bucketed kernel); empty turns the plan off."""
        ml = np.ascontiguousarray(max_len, dtype=np.int32)
        ly = np.ascontiguousarray(layouts, dtype=np.int32)
        assert ml.shape == ly.shape
        _check(self.lib.gss_engine_set_length_plan(self.h, ml.shape[0], _ptr(ml), _ptr(ly)))

    def positions(self, ids):
        """Position of each clause id in the plain scan order (-1: absent)."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        out = np.zeros(ids.shape[0], dtype=np.int64)
        _check(self.lib.gss_db_positions(self.h, _ptr(ids), ids.shape[0], _ptr(out)))
        return out

    # ---- learned scan order ----

    def order_enable(self, **params):
        """Enables the learned scan order; params: fields of OrderParams."""
        p = OrderParams()
        self.lib.gss_order_params_default(ctypes.byref(p))
        for k, v in params.items():
            if not hasattr(p, k):
                raise KeyError(k)
            setattr(p, k, v)
        _check(self.lib.gss_order_enable(self.h, ctypes.byref(p)))

    def order_disable(self):
        _check(self.lib.gss_order_disable(self.h))

    def order_set_active(self, on=True):
        _check(self.lib.gss_order_set_active(self.h, 1 if on else 0))

    def set_lbd(self, ids, lbd):
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        lbd = np.ascontiguousarray(lbd, dtype=np.uint16)
        _check(self.lib.gss_db_set_lbd(self.h, _ptr(ids), _ptr(lbd), ids.shape[0]))

    def wait_head(self, cap=1 << 20, out=None):
        """Reports of the head of the ordered pass in flight (into `out` when
        given and large enough)."""
        while True:
            if out is None or out.shape[0] < cap:
                out = np.zeros(max(int(cap), 1), dtype=REPORT_DTYPE)
            n = ctypes.c_int64()
            rc = self.lib.gss_check_wait_head(self.h, _ptr(out), out.shape[0], ctypes.byref(n))
            if rc == GSS_ERR_OVERFLOW and n.value > out.shape[0]:
                cap = int(n.value)
                continue
            _check(rc)
            return out[:n.value]

    def copy_tail(self, cap=1 << 20, out=None):
        """After wait_head: the rest of the pass's reports (into `out` when
        given and large enough)."""
        while True:
            if out is None or out.shape[0] < cap:
                out = np.zeros(max(int(cap), 1), dtype=REPORT_DTYPE)
            n = ctypes.c_int64()
            rc = self.lib.gss_check_copy_tail(self.h, _ptr(out), out.shape[0], ctypes.byref(n))
            if rc == GSS_ERR_OVERFLOW and n.value > out.shape[0]:
                cap = int(n.value)
                continue
            _check(rc)
            return out[:n.value]

    def order_stats(self):
        st = OrderStats()
        _check(self.lib.gss_order_get_stats(self.h, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in OrderStats._fields_}

    def order_train(self):
        _check(self.lib.gss_order_train(self.h))

    def order_features(self, ids):
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        x = np.zeros((ids.shape[0], SCORER_FEATURES), dtype=np.float32)
        _check(self.lib.gss_order_clause_features(self.h, _ptr(ids), ids.shape[0], _ptr(x)))
        return x

    def scan_ranks(self, ids):
        """Rank of each clause id in the last ordered pass's scan (-1: absent)."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        out = np.zeros(ids.shape[0], dtype=np.int64)
        _check(self.lib.gss_order_scan_ranks(self.h, _ptr(ids), ids.shape[0], _ptr(out)))
        return out

    def order_weights(self):
        w = np.zeros(SCORER_PARAMS, dtype=np.float32)
        _check(self.lib.gss_order_get_weights(self.h, _ptr(w)))
        return w

    def set_order_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.shape == (SCORER_PARAMS,)
        _check(self.lib.gss_order_set_weights(self.h, _ptr(w)))

    def pass_host(self, state, start, solver_of_word=None, out=None):
        """One pass through host buffers (state H2D, check, reports D2H)."""
        state = np.ascontiguousarray(state, dtype=np.uint32)
        start = np.ascontiguousarray(start, dtype=np.uint32)
        sow = None if solver_of_word is None else np.ascontiguousarray(solver_of_word, dtype=np.int32)
        if out is None:
            out = np.zeros(1 << 20, dtype=REPORT_DTYPE)
        n = ctypes.c_int64()
        while True:
            rc = self.lib.gss_check_pass_host(self.h, _ptr(state), state.shape[0], state.shape[1], _ptr(start),
                                              _ptr(sow), _ptr(out), out.shape[0], ctypes.byref(n))
            if rc == GSS_ERR_OVERFLOW and n.value > out.shape[0]:
                out = np.zeros(int(n.value), dtype=REPORT_DTYPE)
                continue
            _check(rc)
            return out[:n.value]


SCORER_FEATURES = 12
SCORER_HIDDEN = 64
SCORER_PARAMS = 5057


class OrderParams(ctypes.Structure):
    """gss_order_params."""
    _fields_ = [("head_fraction", ctypes.c_double), ("retrain_interval", ctypes.c_int), ("train_epochs", ctypes.c_int),
                ("batch", ctypes.c_int), ("learning_rate", ctypes.c_float), ("log_capacity", ctypes.c_int64),
                ("log_rate", ctypes.c_double), ("seed", ctypes.c_uint64), ("overlap", ctypes.c_int),
                ("rescore_interval", ctypes.c_int)]


class OrderStats(ctypes.Structure):
    """gss_order_stats."""
    _fields_ = [("passes", ctypes.c_int64), ("trainings", ctypes.c_int64), ("last_loss", ctypes.c_double),
                ("head_positions", ctypes.c_int64), ("logged", ctypes.c_int64), ("score_ms", ctypes.c_double),
                ("head_ms", ctypes.c_double), ("tail_ms", ctypes.c_double)]


class Scorer:
    """The learned order's MLP (12-64-64-1) on its own: FP32 weights, BF16
    tensor-core inference, FP32 training kernels. Flat weight layout:
    W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3."""

    def __init__(self, device=0, seed=1):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.gss_scorer_create(device, seed, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.gss_scorer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def weights(self):
        w = np.zeros(SCORER_PARAMS, dtype=np.float32)
        _check(self.lib.gss_scorer_get_weights(self.h, _ptr(w)))
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.shape == (SCORER_PARAMS,)
        _check(self.lib.gss_scorer_set_weights(self.h, _ptr(w)))

    def infer(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, SCORER_FEATURES)
        out = np.zeros(x.shape[0], dtype=np.float32)
        _check(self.lib.gss_scorer_infer(self.h, _ptr(x), x.shape[0], _ptr(out)))
        return out

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, SCORER_FEATURES)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(SCORER_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        _check(self.lib.gss_scorer_gradient(self.h, _ptr(x), _ptr(y), x.shape[0], _ptr(g), ctypes.byref(loss)))
        return g, float(loss.value)

    def train_step(self, x, y, lr=1e-3):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, SCORER_FEATURES)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = ctypes.c_float()
        _check(self.lib.gss_scorer_train_step(self.h, _ptr(x), _ptr(y), x.shape[0], ctypes.c_float(lr),
                                              ctypes.byref(loss)))
        return float(loss.value)


def bench_plant(lits_ptr, offsets_ptr, n_clauses, rate_ptr, state_ptr, base_ptr, n_vars, n_words, seed, pass_no,
                restore, stream=None):
    """gss_bench_plant on device pointers (the learned-order workload)."""
    lib = load()
    _check(lib.gss_bench_plant(_vp(lits_ptr), _vp(offsets_ptr), int(n_clauses), _vp(rate_ptr), _vp(state_ptr),
                               _vp(base_ptr), int(n_vars), int(n_words), int(seed), int(pass_no), int(restore),
                               _vp(stream) if stream else None))


def passes_host(engine, states, start, solver_of_word=None, caps=None, packed=False, records=None):
    """Pipelined passes through host buffers; returns one report array per
    state. records: "full" (gss_check_passes_host, REPORT_DTYPE), "packed"
    (gss_check_passes_host_packed, 12-byte records) or "cells"
    (gss_check_passes_host_cells, 8-byte {clause * n_words + word, mask});
    packed=True is records="packed"."""
    records = records or ("packed" if packed else "full")
    dtype, fn = {"full": (REPORT_DTYPE, engine.lib.gss_check_passes_host),
                 "packed": (PACKED_REPORT_DTYPE, engine.lib.gss_check_passes_host_packed),
                 "cells": (CELL_REPORT_DTYPE, engine.lib.gss_check_passes_host_cells)}[records]
    n = len(states)
    states = [np.ascontiguousarray(s, dtype=np.uint32) for s in states]
    start = np.ascontiguousarray(start, dtype=np.uint32)
    sow = None if solver_of_word is None else np.ascontiguousarray(solver_of_word, dtype=np.int32)
    caps = caps or [1 << 20] * n
    while True:
        outs = [np.zeros(max(int(c), 1), dtype=dtype) for c in caps]
        sp = (ctypes.c_void_p * n)(*[s.ctypes.data for s in states])
        op = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
        cp = np.ascontiguousarray(caps, dtype=np.int64)
        nr = np.zeros(n, dtype=np.int64)
        rc = fn(engine.h, n, sp, states[0].shape[0], states[0].shape[1], _ptr(start), _ptr(sow), op, _ptr(cp),
                _ptr(nr))
        if rc == GSS_ERR_OVERFLOW:
            caps = [max(int(c), int(x)) + 1024 for c, x in zip(caps, nr)]
            continue
        _check(rc)
        return [o[:k] for o, k in zip(outs, nr)]


def probe_gather(buffer_bytes, depth=2, blocks_per_sm=8, device=0):
    """Random 256-byte row gathers over a device buffer (gss_probe_gather):
    returns (rows per second, ms per launch)."""
    lib = load()
    rps = ctypes.c_double()
    ms = ctypes.c_double()
    _check(lib.gss_probe_gather(device, int(buffer_bytes), depth, blocks_per_sm, ctypes.byref(rps), ctypes.byref(ms)))
    return rps.value, ms.value


def cells_to_reports(cells, n_words):
    """8-byte cell records -> PACKED_REPORT_DTYPE {clause, word, mask}."""
    out = np.zeros(len(cells), dtype=PACKED_REPORT_DTYPE)
    out["clause"] = cells["cell"] // np.uint32(n_words)
    out["word"] = cells["cell"] % np.uint32(n_words)
    out["mask"] = cells["mask"]
    return out


def sort_reports(rep):
    """Reports in (clause, word) order, for comparison with the oracle."""
    order = np.lexsort((rep["word"], rep["clause"]))
    return rep[order]


# ---------------------------------------------------------------- sharer ----

class _SharerOptions(ctypes.Structure):
    _fields_ = [("gpu_block_count_guideline", ctypes.c_int),
                ("gpu_threads_per_block_guideline", ctypes.c_int),
                ("min_gpu_latency_micros", ctypes.c_int),
                ("verbosity", ctypes.c_int),
                ("clause_activity_decay", ctypes.c_double),
                ("quick_prof", ctypes.c_int),
                ("init_report_count_per_category", ctypes.c_int),
                ("max_page_locked_memory", ctypes.c_int)]


_LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_char_p, ctypes.c_void_p)

GLOBAL_STATS = ["gpuClauses", "gpuClauseLengthSum", "gpuClausesAdded", "gpuRuns", "clauseTestsOnGroups",
                "clauseTestsOnAssigs", "totalAssigClauseTested", "gpuReduceDbs", "gpuReports",
                "timeSpentTestingClauses", "timeSpentFillingAssigs", "timeSpentFillingReported",
                "timeSpentReduceGpuDb"]
ONE_SOLVER_STATS = ["varUpdatesSentToGpu", "assigsSentToGpu", "failuresToFindAssig", "reportedClauses",
                    "reportedClausesUnit", "reportedClausesBinary"]


def _sharer_sigs(lib):
    if getattr(lib, "_gss_sharer_sigs", False):
        return
    c_int, c_i64, vp = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    ip = ctypes.POINTER(ctypes.c_int)
    _sig(lib, "gss_sharer_options_default", None, vp)
    _sig(lib, "gss_sharer_create", c_int, vp, _LOG_FN, vp, c_int, vp)
    _sig(lib, "gss_sharer_destroy", c_int, vp)
    _sig(lib, "gss_sharer_gpu_run", c_int, vp)
    _sig(lib, "gss_sharer_reduce_db", c_int, vp)
    _sig(lib, "gss_sharer_added_clause_count", c_i64, vp)
    _sig(lib, "gss_sharer_added_clause_count_at_last_reduce_db", c_i64, vp)
    _sig(lib, "gss_sharer_has_run_out_of_gpu_memory_once", c_int, vp)
    _sig(lib, "gss_sharer_gpu_mem_info", c_int, vp, vp, vp)
    _sig(lib, "gss_sharer_global_stat_count", c_int)
    _sig(lib, "gss_sharer_global_stat", c_i64, vp, c_int)
    _sig(lib, "gss_sharer_global_stat_name", ctypes.c_char_p, c_int)
    _sig(lib, "gss_sharer_one_solver_stat_count", c_int)
    _sig(lib, "gss_sharer_one_solver_stat_name", ctypes.c_char_p, c_int)
    _sig(lib, "gss_sharer_one_solver_stat", c_i64, vp, c_int, c_int)
    _sig(lib, "gss_sharer_set_var_count", c_int, vp, c_int)
    _sig(lib, "gss_sharer_add_clause", c_i64, vp, c_int, vp, c_int)
    _sig(lib, "gss_sharer_set_cpu_solver_count", c_int, vp, c_int)
    _sig(lib, "gss_sharer_try_set_solver_values", c_int, vp, c_int, vp, c_int)
    _sig(lib, "gss_sharer_unset_solver_values", c_int, vp, c_int, vp, c_int)
    _sig(lib, "gss_sharer_try_send_assignment", c_i64, vp, c_int)
    _sig(lib, "gss_sharer_pop_reported_clause", c_int, vp, c_int, ctypes.POINTER(ip), ip,
         ctypes.POINTER(ctypes.c_int64))
    _sig(lib, "gss_sharer_last_assig_all_reported", c_i64, vp, c_int)
    _sig(lib, "gss_sharer_current_assignment", c_int, vp, c_int, vp)
    _sig(lib, "gss_sharer_set_max_clause_len", c_int, vp, c_int)
    _sig(lib, "gss_sharer_set_variant", c_int, vp, c_int, c_int, c_int, c_int)
    _sig(lib, "gss_sharer_set_clause_budget", c_int, vp, c_i64)
    _sig(lib, "gss_sharer_set_locality", c_int, vp, c_int)
    _sig(lib, "gss_sharer_evicted_count", c_i64, vp)
    _sig(lib, "gss_sharer_device_compactions", c_i64, vp)
    _sig(lib, "gss_serving_run", c_int, vp, vp)
    _sig(lib, "gss_activity_create", vp, ctypes.c_float)
    _sig(lib, "gss_activity_destroy", None, vp)
    _sig(lib, "gss_activity_add", c_i64, vp, c_int)
    _sig(lib, "gss_activity_bump", c_int, vp, c_i64)
    _sig(lib, "gss_activity_decay", c_int, vp)
    _sig(lib, "gss_activity_get", ctypes.c_float, vp, c_i64)
    _sig(lib, "gss_activity_approx_nth", ctypes.c_float, vp, c_int, c_int, c_i64)
    _sig(lib, "gss_activity_removing_thresholds", c_int, vp, c_int, c_i64, ip, ip, ctypes.POINTER(ctypes.c_float))
    lib._gss_sharer_sigs = True


def _int_array(lits):
    a = np.ascontiguousarray(lits, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.c_void_p)


class ClauseSharer:
    """The reference's GpuClauseSharer (gpuShareLib/GpuClauseSharer.h:74-163)
    through the C ABI, with the same method names. Literals are ints,
    2*var + sign (sign 1 = negative)."""

    def __init__(self, gpuBlockCountGuideline=-1, gpuThreadsPerBlockGuideline=-1, minGpuLatencyMicros=-1,
                 verbosity=0, clauseActivityDecay=-1.0, quickProf=True, initReportCountPerCategory=-1,
                 maxPageLockedMemory=-1, device=0, log=None):
        self.lib = load()
        _sharer_sigs(self.lib)
        o = _SharerOptions(gpuBlockCountGuideline, gpuThreadsPerBlockGuideline, minGpuLatencyMicros, verbosity,
                           clauseActivityDecay, 1 if quickProf else 0, initReportCountPerCategory,
                           maxPageLockedMemory)
        self._log = _LOG_FN(lambda msg, ctx: log(msg.decode())) if log else _LOG_FN()
        h = ctypes.c_void_p()
        _check(self.lib.gss_sharer_create(ctypes.byref(o), self._log, None, device, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.gss_sharer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def gpuRun(self):
        _check(self.lib.gss_sharer_gpu_run(self.h))

    def reduceDb(self):
        _check(self.lib.gss_sharer_reduce_db(self.h))

    def getAddedClauseCount(self):
        return int(self.lib.gss_sharer_added_clause_count(self.h))

    def getAddedClauseCountAtLastReduceDb(self):
        return int(self.lib.gss_sharer_added_clause_count_at_last_reduce_db(self.h))

    def hasRunOutOfGpuMemoryOnce(self):
        return bool(self.lib.gss_sharer_has_run_out_of_gpu_memory_once(self.h))

    def getGpuMemInfo(self):
        f, t = ctypes.c_size_t(), ctypes.c_size_t()
        _check(self.lib.gss_sharer_gpu_mem_info(self.h, ctypes.byref(f), ctypes.byref(t)))
        return int(f.value), int(t.value)

    def getGlobalStatCount(self):
        return int(self.lib.gss_sharer_global_stat_count())

    def getGlobalStat(self, stat):
        if isinstance(stat, str):
            stat = GLOBAL_STATS.index(stat)
        return int(self.lib.gss_sharer_global_stat(self.h, stat))

    def getGlobalStatName(self, stat):
        return self.lib.gss_sharer_global_stat_name(stat).decode()

    def getOneSolverStatCount(self):
        return int(self.lib.gss_sharer_one_solver_stat_count())

    def getOneSolverStatName(self, stat):
        return self.lib.gss_sharer_one_solver_stat_name(stat).decode()

    def getOneSolverStat(self, solver, stat):
        if isinstance(stat, str):
            stat = ONE_SOLVER_STATS.index(stat)
        return int(self.lib.gss_sharer_one_solver_stat(self.h, solver, stat))

    def setVarCount(self, n):
        _check(self.lib.gss_sharer_set_var_count(self.h, n))

    def addClause(self, solverId, lits):
        a, p = _int_array(lits)
        return int(self.lib.gss_sharer_add_clause(self.h, solverId, p, a.shape[0]))

    def setCpuSolverCount(self, n):
        _check(self.lib.gss_sharer_set_cpu_solver_count(self.h, n))

    def trySetSolverValues(self, solver, lits):
        a, p = _int_array(lits)
        return bool(self.lib.gss_sharer_try_set_solver_values(self.h, solver, p, a.shape[0]))

    def unsetSolverValues(self, solver, lits):
        a, p = _int_array(lits)
        _check(self.lib.gss_sharer_unset_solver_values(self.h, solver, p, a.shape[0]))

    def trySendAssignment(self, solver):
        return int(self.lib.gss_sharer_try_send_assignment(self.h, solver))

    def popReportedClause(self, solver):
        """(list of literals, gpu clause id), or None."""
        lp = ctypes.POINTER(ctypes.c_int)()
        n = ctypes.c_int()
        cid = ctypes.c_int64()
        if not self.lib.gss_sharer_pop_reported_clause(self.h, solver, ctypes.byref(lp), ctypes.byref(n),
                                                       ctypes.byref(cid)):
            return None
        return [lp[i] for i in range(n.value)], int(cid.value)

    def popAll(self, solver):
        out = []
        while True:
            r = self.popReportedClause(solver)
            if r is None:
                return out
            out.append(r)

    def getLastAssigAllReported(self, solver):
        return int(self.lib.gss_sharer_last_assig_all_reported(self.h, solver))

    def getCurrentAssignment(self, solver, n_vars):
        buf = np.zeros(n_vars, dtype=np.uint8)
        _check(self.lib.gss_sharer_current_assignment(self.h, solver, buf.ctypes.data_as(ctypes.c_void_p)))
        return buf

    def setMaxClauseLen(self, n):
        _check(self.lib.gss_sharer_set_max_clause_len(self.h, n))

    def setVariant(self, kind=-1, lanes_per_clause=0, depth=2, flags=0):
        _check(self.lib.gss_sharer_set_variant(self.h, kind, lanes_per_clause, depth, flags))

    def setLocality(self, range_log2=-1):
        """Device order of the database (gss_sharer_set_locality): -1
        automatic variable ranges, 0 length order, 11..31 ranges of
        2^range_log2 variables."""
        _check(self.lib.gss_sharer_set_locality(self.h, int(range_log2)))

    def setClauseBudget(self, max_clauses):
        """HBM budget: a pass checks at most max_clauses live clauses; the
        oldest clauses not reported in the last 8 passes are evicted first.
        0 = no budget."""
        _check(self.lib.gss_sharer_set_clause_budget(self.h, int(max_clauses)))

    def evictedCount(self):
        return int(self.lib.gss_sharer_evicted_count(self.h))

    def deviceCompactions(self):
        return int(self.lib.gss_sharer_device_compactions(self.h))


class ServingParams(ctypes.Structure):
    """gss_serving_params: one run of the serving load generator."""
    _fields_ = [("seconds", ctypes.c_double), ("warmup_seconds", ctypes.c_double),
                ("assign_rate", ctypes.c_double), ("n_solvers", ctypes.c_int), ("n_vars", ctypes.c_int),
                ("budget", ctypes.c_int64), ("initial_clauses", ctypes.c_int64),
                ("clause_rate", ctypes.c_double), ("plant_rate", ctypes.c_double),
                ("batch_max", ctypes.c_int), ("trail_fraction", ctypes.c_double),
                ("trail_change", ctypes.c_int), ("seed", ctypes.c_uint64), ("plain_scan", ctypes.c_int)]


class ServingResult(ctypes.Structure):
    _fields_ = [("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("p999_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("assignments", ctypes.c_int64), ("reports_popped", ctypes.c_int64), ("passes", ctypes.c_int64),
                ("checks_per_s", ctypes.c_double), ("assignments_per_s", ctypes.c_double),
                ("elapsed_s", ctypes.c_double), ("evicted", ctypes.c_int64), ("retries", ctypes.c_int64),
                ("clauses_streamed", ctypes.c_int64), ("live_clauses_end", ctypes.c_int64),
                ("device_compactions", ctypes.c_int64), ("run_ms_p50", ctypes.c_double),
                ("run_ms_p99", ctypes.c_double), ("run_ms_max", ctypes.c_double), ("long_runs", ctypes.c_int64),
                ("long_wait_ms", ctypes.c_double), ("long_launch_ms", ctypes.c_double),
                ("long_deliver_ms", ctypes.c_double), ("long_other_ms", ctypes.c_double)]


def serving_run(**params):
    """Runs the serving load generator on the current CUDA device; returns its
    result as a dict. Keys of params: the fields of ServingParams."""
    lib = load()
    _sharer_sigs(lib)
    p = ServingParams(seconds=5.0, warmup_seconds=1.0, assign_rate=5e4, n_solvers=64, n_vars=2 ** 21,
                      budget=0, initial_clauses=1_000_000, clause_rate=2e5, plant_rate=0.01, batch_max=32,
                      trail_fraction=0.5, trail_change=4, seed=1)
    for k, v in params.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    r = ServingResult()
    _check(lib.gss_serving_run(ctypes.byref(p), ctypes.byref(r)))
    return {name: getattr(r, name) for name, _ in ServingResult._fields_}


class ClauseActivity:
    """The reduceDb policy on its own (host code, no GPU): activity with decay,
    bump and rescale, and the removal thresholds."""

    def __init__(self, decay):
        self.lib = load()
        _sharer_sigs(self.lib)
        self.h = ctypes.c_void_p(self.lib.gss_activity_create(ctypes.c_float(decay)))

    def __del__(self):
        try:
            if self.h:
                self.lib.gss_activity_destroy(self.h)
        except Exception:
            pass

    def add(self, lbd):
        return int(self.lib.gss_activity_add(self.h, lbd))

    def bump(self, i):
        _check(self.lib.gss_activity_bump(self.h, i))

    def decay(self):
        _check(self.lib.gss_activity_decay(self.h))

    def get(self, i):
        return float(self.lib.gss_activity_get(self.h, i))

    def approx_nth(self, min_lbd, max_lbd, n):
        return float(self.lib.gss_activity_approx_nth(self.h, min_lbd, max_lbd, n))

    def removing_thresholds(self, act_only, total):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _check(self.lib.gss_activity_removing_thresholds(self.h, 1 if act_only else 0, total, ctypes.byref(a),
                                                         ctypes.byref(b), ctypes.byref(c)))
        return int(a.value), int(b.value), float(c.value)
