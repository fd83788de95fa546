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


def test_dropin_lookup_tables(tmp_path):
    """The open-addressing map behind the drop-in searches' id and row lookups (and
    LocalIndex in both forms) agrees with std::unordered_map on sequential, random,
    negative and extreme keys, with and without reserve."""
    import subprocess
    exe = str(tmp_path / "index_map_check")
    shim = os.path.join(ROOT, "rnng_gb300", "mpi_shim")
    import rnng_gb300
    rnng_gb300.build.build()
    lib = os.path.dirname(rnng_gb300.LIB_PATH)
    subprocess.run(["g++", "-O2", "-std=c++20", "-I" + shim, "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "index_map_check.cpp"), os.path.join(shim, "mpi_shim.cpp"),
                    "-L" + lib, "-lrnng_gpu", "-Wl,-rpath," + lib, "-pthread", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


@pytest.mark.parametrize("m", [1000, 1_500_000])
def test_graph_text_of_the_dropin_writer(tmp_path, m):
    """Graph::write_file (the drivers' collective form) prints each edge as
    "u v w" with w in printf's %.6g, sorted; above 2^20 edges the text is formatted in
    blocks on several host threads and must come out the same."""
    import subprocess
    import numpy as np
    exe = str(tmp_path / "graph_text_check")
    shim = os.path.join(ROOT, "rnng_gb300", "mpi_shim")
    import rnng_gb300
    rnng_gb300.build.build()
    lib = os.path.dirname(rnng_gb300.LIB_PATH)
    subprocess.run(["g++", "-O2", "-std=c++20", "-I" + shim, "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "graph_text_check.cpp"), os.path.join(shim, "mpi_shim.cpp"),
                    "-L" + lib, "-lrnng_gpu", "-Wl,-rpath," + lib, "-pthread", "-o", exe], check=True)
    out = str(tmp_path / "g.mtx")
    subprocess.run([exe, str(m), out], check=True)
    # the same edges in Python, sorted as the writer sorts them
    s = 12345
    mask = (1 << 64) - 1
    rows = []
    for i in range(m):
        s = (s * 6364136223846793005 + 1442695040888963407) & mask
        u, v = i // 7, (s >> 33) % 1000003
        w = np.float32((s >> 40) / (1 << 12) * (1e-3 if i % 5 == 0 else 1.0))
        rows.append((u, v, np.float32(i % 97) if i % 11 == 0 else w))
    rows.sort(key=lambda r: (r[0], r[1], float(r[2])))
    want = "%% %d %d %d\n" % (m // 7 + 1, m // 7 + 1, m) + "".join("%d %d %.6g\n" % (u, v, float(w)) for u, v, w in rows)
    assert open(out).read() == want
