"""The C ABI library builds for sm_103a, loads, and exports every entry point
declared in include/chromo_gb300.h (no GPU needed: nothing is called)."""
import ctypes
import re
from pathlib import Path

from chromo_gb300 import _native
from chromo_gb300.build import build

HEADER = Path(__file__).resolve().parents[1] / "include" / "chromo_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cg_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib_path = build()
    lib = ctypes.CDLL(str(lib_path))  # fails on unresolved symbols
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_native.EXPORTS), set(names) ^ set(_native.EXPORTS)


def test_error_path_without_gpu_is_reported():
    """With no CUDA device, creating a sim fails with a status, not a crash."""
    import pytest
    lib = _native.lib()
    assert lib.cg_last_error() is not None
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_native.CgError):
        _native.Sim([10], [[2, 2, 2]], 1)
