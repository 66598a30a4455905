"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; argument checks fail with a status, not a crash."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(bpl_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "bpl_lbp_forward" in names
    assert len(names) >= 5


def test_library_exports_every_declared_symbol(bpl_lib):
    missing = [n for n in declared_symbols() if not hasattr(bpl_lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_every_symbol(bpl_lib):
    from bpl_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_version_and_status_text(bpl_lib):
    assert bpl_lib.bpl_version() >= 100
    assert bpl_lib.bpl_status_string(0) == b"ok"
    assert bpl_lib.bpl_status_string(1) == b"invalid argument"


def test_invalid_arguments_return_status_without_touching_the_device(bpl_lib):
    # L out of range, null pointers: rejected on the host before any launch
    st = bpl_lib.bpl_lbp_forward(0, None, None, None, None, None, 0, None,
                                 1, 4, 4, 2000, 6, 1, 1, 3, None)
    assert st == 1
    assert b"L=2000" in bpl_lib.bpl_last_error()
    st = bpl_lib.bpl_lbp_forward(7, None, None, None, None, None, 0, None,
                                 1, 4, 4, 8, 6, 1, 1, 3, None)
    assert st == 1


def _declared_arg_counts():
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(bpl_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
            args = m.group(2).strip()
            out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def test_python_signatures_match_header_arity():
    from bpl_gb300 import _lib
    counts = _declared_arg_counts()
    for name, n in counts.items():
        assert len(_lib.SIGNATURES[name]) == n, f"{name}: header has {n} args, binding {len(_lib.SIGNATURES[name])}"
