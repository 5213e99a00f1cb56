"""The C ABI builds, loads and exports every function include/gpurir_gb300.h
declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpurir_gb300.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gpurir_\w+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = _declared()
    for n in ("gpurir_create", "gpurir_destroy", "gpurir_simulate_rir", "gpurir_simulate_rir_device",
              "gpurir_activate_mixed_precision", "gpurir_activate_lut", "gpurir_n_samples"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    from gpurir_gb300 import _lib
    L = _lib.load()
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes table covers the header exactly
    assert sorted(_lib.SIGNATURES) == _declared()


def test_host_only_calls(built):
    from gpurir_gb300 import _lib
    L = _lib.load()
    assert L.gpurir_version().startswith(b"gpurir_gb300")
    assert L.gpurir_n_samples(0.5, 16000.0) == 8000
    assert L.gpurir_n_samples(0.3, 16000.0) == 4800
    # a NULL handle is an argument error, not a crash
    assert L.gpurir_activate_lut(None, 1, None) == -1
    assert b"NULL" in L.gpurir_last_error()
    assert L.gpurir_set_noise(None, 0) == -1


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    """The product path refuses to run when the CUDA library is absent."""
    from gpurir_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.load()
