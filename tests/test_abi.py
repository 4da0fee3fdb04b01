"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
entry point declared in include/*.h (no compute calls here)."""
import ctypes
import os
import re

import pytest

from wolfd2_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            txt = open(os.path.join(inc, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms.update(re.findall(r"\b(wolfd2gpu_\w+)\s*\(", txt))
    return syms


def test_library_exports_declared_symbols():
    path = build.build_library()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_sm103a_code_present():
    path = build.build_library()
    data = open(path, "rb").read()
    assert b"sm_103a" in data or b"sm_103" in data


def test_no_cpu_fallback_without_gpu():
    """Creating a context on a machine without a GPU fails loudly."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from wolfd2_gb300 import deck
    from wolfd2_gb300.gpu import Solver, W2Error
    c = deck.cavity(16, 100.0, 0.01)
    with pytest.raises(W2Error):
        Solver.for_case(c)
