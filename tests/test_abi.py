"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/rnng_gpu.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _have_rnng_sources() -> bool:
    import oracle
    return oracle.ref_source_dir() is not None


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


def test_dropin_harness_builds_against_the_dropin_headers():
    """The harness source that makes RNNG's API calls compiles against include/*.h and
    links to librnng_gpu.so (it runs in the GPU tests)."""
    import subprocess
    import rnng_gb300
    rnng_gb300.build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], check=True)
    assert os.path.exists(os.path.join(ROOT, "oracle", "_build", "dropin_harness"))


@pytest.mark.skipif(not _have_rnng_sources(), reason="needs the RNNG sources ($RNNG_SRC) to build its drivers")
def test_unchanged_reference_drivers_build_against_the_dropin_headers():
    """drivers/systolic.cpp, landmark.cpp and rips.cpp, unmodified, compile against the
    drop-in headers and link to librnng_gpu.so and the single-rank MPI shim."""
    import subprocess
    import rnng_gb300
    rnng_gb300.build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin-drivers"], check=True)
    for d in ("systolic", "landmark", "rips"):
        assert os.path.exists(os.path.join(ROOT, "oracle", "_build", "dropin_" + d))
