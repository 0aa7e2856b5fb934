"""CPU tests of the C ABI boundary: the library loads and exports every entry
point that include/flf.h declares; failures without a GPU are reported as
status codes, not crashes."""

import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "flf.h")).read()
    return sorted(set(re.findall(r"^(?:int|long long)\s+\**\s*(flf_\w+)\s*\(", text, re.M)))


def test_header_matches_binding():
    import _flf
    assert header_functions() == _flf.exported_symbols()


def test_library_exports_all_symbols(built_lib):
    import ctypes
    lib = ctypes.CDLL(built_lib)
    for name in header_functions():
        assert hasattr(lib, name), name


def test_version_string(built_lib):
    import _flf
    assert "sm_103a" in _flf.version()


def test_create_without_gpu_reports_error(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import _flf
    with pytest.raises(_flf.FlfError) as e:
        _flf.Context(15, 11)
    assert e.value.code in (-2, -1)


def test_bad_arguments_rejected_before_cuda(built_lib):
    import _flf
    with pytest.raises(_flf.FlfError) as e:
        _flf.Context(4, 3)
    assert e.value.code == -1 and "odd" in str(e.value)
    with pytest.raises(_flf.FlfError):
        _flf.Context(15, 0)
