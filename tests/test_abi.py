"""The C ABI library: it loads without a GPU, exports every function that
include/gpuklu.h declares, and refuses to compute without a device (no CPU
fallback)."""
import ctypes as C
import os
import re

import pytest
import torch

from rustspice_gb300 import native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "gpuklu.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    return sorted(set(re.findall(r"\b(gpuklu_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_symbol_list():
    assert _declared() == sorted(N.SYMBOLS)


def test_library_exports_every_declared_symbol():
    L = C.CDLL(N.lib_path()) if os.path.exists(N.lib_path()) else N.lib()
    missing = [s for s in _declared() if not hasattr(L, s)]
    assert not missing, missing


def test_name_and_status_codes():
    L = N.lib()
    assert L.gpuklu_name(None) == b"GpuKLU"
    assert (N.OK, N.INVALID_MATRIX, N.DEVICE_TIMEOUT, N.CUDA_ERROR) == (0, 6, 7, 9)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-device path")
def test_no_device_no_fallback():
    from rustspice_gb300.solver import GpuKluSolver
    with pytest.raises(Exception):
        GpuKluSolver(4)
