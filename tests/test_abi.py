"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/rnng_gpu.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared():
    text = open(os.path.join(ROOT, "include", "rnng_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(rnng_\w+)\s*\(", text, re.M)))


def test_library_builds_and_exports_all_symbols():
    import rnng_gb300
    path = rnng_gb300.build.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    names = declared()
    assert set(names) == set(rnng_gb300.EXPORTS)
    for name in names:
        assert hasattr(lib, name), name


def test_context_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import rnng_gb300
    with pytest.raises(rnng_gb300.RnngError):
        rnng_gb300.Context(0)
