"""The C ABI surface: the library loads and exports every function that
include/msbg_gpu.h declares, and the Python binding covers each of them.
No GPU calls are made here."""
from __future__ import annotations

import ctypes
import os
import re

from conftest import ROOT

HEADER_DIR = os.path.join(ROOT, "include")


def declared_functions() -> set[str]:
    names = set()
    for fn in os.listdir(HEADER_DIR):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(HEADER_DIR, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(msbg_gpu_[a-z0-9_]+)\s*\(", src))
    return names


def test_header_declares_functions():
    assert len(declared_functions()) >= 30


def test_library_exports_every_declared_symbol(gpulib):
    lib = ctypes.CDLL(gpulib.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_every_declared_symbol(gpulib):
    assert declared_functions() == set(gpulib.SIGNATURES), \
        declared_functions() ^ set(gpulib.SIGNATURES)


def test_missing_library_fails_loudly(gpulib, tmp_path):
    import pytest
    with pytest.raises(OSError):
        gpulib.load_library(str(tmp_path / "nope.so"))
