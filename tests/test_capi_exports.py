"""The C-ABI library loads on a machine without a GPU and exports every
symbol declared in include/hbi_gpu.h; compute calls fail loudly (no CPU
fallback)."""
import ctypes
import os
import re

import pytest

import hbi_gb300 as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "hbi_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hbi_[a-z0-9_]+)\s*\(", src)))


def test_header_and_python_list_agree():
    assert sorted(H.EXPORTS) == declared_symbols()


def test_every_declared_symbol_is_exported():
    L = H.lib()
    for s in declared_symbols():
        assert hasattr(L, s), s


def test_no_gpu_means_error_not_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(H.HBIError):
        H.Ctl(16)
