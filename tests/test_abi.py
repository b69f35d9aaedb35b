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
