"""The C ABI library loads and exports every function the headers declare (CPU only)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        # C declarations of the gss_ ABI: "<type> gss_name(" at line start
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(gss_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_functions():
    assert len(declared_functions()) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_gpu_needed_for_load_and_version(lib):
    assert lib.gss_version().startswith(b"gpusharesat-gb300")
    assert lib.gss_max_clause_len() >= 100


def test_order_params_layout_and_defaults(lib):
    """The Python mirror of gss_order_params has the C field layout: the
    library's defaults land in the right fields, rescore_interval included."""
    import ctypes
    import gpusharesat_gb300 as g
    p = g.OrderParams()
    lib.gss_order_params_default(ctypes.byref(p))
    assert abs(p.head_fraction - 0.1) < 1e-12 and p.retrain_interval == 1000 and p.train_epochs == 2
    assert p.batch == 4096 and p.log_capacity == 1 << 20 and p.overlap == 1 and p.rescore_interval == 1


def test_gather_probe_refuses_bad_arguments(lib):
    """gss_probe_gather checks its arguments before touching a device."""
    import gpusharesat_gb300 as g
    for kw in ({"buffer_bytes": 1 << 20, "depth": 3}, {"buffer_bytes": 100}, {"buffer_bytes": 1 << 20,
                                                                               "blocks_per_sm": 0}):
        with pytest.raises(g.GssError):
            g.probe_gather(**kw)
