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

REPORT_DTYPE = np.dtype([("clause", "<u4"), ("word", "<u4"), ("mask", "<u4"), ("solver", "<u4")])

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
    _sig(lib, "gss_max_clause_len", c_int)
    _sig(lib, "gss_engine_create", c_int, c_int, vp)
    _sig(lib, "gss_engine_destroy", c_int, vp)
    _sig(lib, "gss_engine_set_stream", c_int, vp, vp)
    _sig(lib, "gss_engine_launch_count", c_i64, vp)
    _sig(lib, "gss_engine_set_timing", c_int, vp, c_int)
    _sig(lib, "gss_engine_kernel_time", c_int, vp, vp, vp)
    _sig(lib, "gss_engine_set_variant", c_int, vp, c_int, c_int, c_int, c_int)
    _sig(lib, "gss_db_set", c_int, vp, vp, vp, c_i64)
    _sig(lib, "gss_db_clause_count", c_i64, vp)
    _sig(lib, "gss_db_literal_count", c_i64, vp)
    _sig(lib, "gss_db_max_var", c_i64, vp)
    _sig(lib, "gss_state_set", c_int, vp, vp, c_i64, c_int, vp, vp, c_int)
    _sig(lib, "gss_check_set_capacity", c_int, vp, c_i64)
    _sig(lib, "gss_check_launch", c_int, vp)
    _sig(lib, "gss_check_wait", c_int, vp, vp)
    _sig(lib, "gss_check_copy_reports", c_int, vp, vp, c_i64, vp)
    _sig(lib, "gss_check_pass_host", c_int, vp, vp, c_i64, c_int, vp, vp, vp, c_i64, vp)
    _lib = lib
    return lib


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

    def set_state(self, state, start, solver_of_word=None):
        state = np.ascontiguousarray(state, dtype=np.uint32)
        start = np.ascontiguousarray(start, dtype=np.uint32)
        sow = None if solver_of_word is None else np.ascontiguousarray(solver_of_word, dtype=np.int32)
        _check(self.lib.gss_state_set(self.h, _ptr(state), state.shape[0], state.shape[1], _ptr(start),
                                      _ptr(sow), 0))

    def set_state_device(self, state_ptr, n_vars, n_words, start_ptr, sow_ptr=None):
        _check(self.lib.gss_state_set(self.h, _vp(state_ptr), n_vars, n_words, _vp(start_ptr),
                                      _vp(sow_ptr) if sow_ptr else None, 1))

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


def sort_reports(rep):
    """Reports in (clause, word) order, for comparison with the oracle."""
    order = np.lexsort((rep["word"], rep["clause"]))
    return rep[order]
