"""The plain-C interface (include/nvtt/nvtt_wrapper.h), driven by a C99 program the way a C user of
NVTT calls it (tests/c/nvtt_wrapper_harness.c), against the bytes the reference's Compressor::process
writes for the same inputs (tests/golden/dds_process.npz).

CPU: the harness compiles as C99 with warnings as errors and links against libntg.so; the global
functions answer; without a GPU nvttCompress returns NVTT_False and the error callback receives
NVTT_Error_CudaError. GPU: whole DDS files are byte-identical to the reference's, through the output
callback and through nvttSetOutputOptionsFileName."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from test_nvtt_api import GOLD, NCASES, case, expected_error, harness_args, header_size, no_gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ERROR_UNSUPPORTED_FEATURE, ERROR_CUDA = 2, 3


@pytest.fixture(scope="session")
def c_harness(ntg_lib, tmp_path_factory):
    import ntg
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(ntg.build())
    exe = str(tmp_path_factory.mktemp("nvtt_c") / "nvtt_wrapper_harness")
    cmd = [cc, "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "nvtt_wrapper_harness.c"), "-L", libdir, "-lntg",
           "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_c(exe, i, tmp_path, **extra):
    inp, out = tmp_path / f"in_{i}.bin", tmp_path / f"out_{i}.bin"
    GOLD[f"input_{i}"].tofile(inp)
    args = [a for a in harness_args(case(i), **extra)]
    r = subprocess.run([exe, str(inp), str(out)] + args, capture_output=True, text=True, timeout=300)
    data = np.fromfile(out, np.uint8) if out.exists() else np.zeros(0, np.uint8)
    return r.returncode, r.stdout + r.stderr, data


# ---- CPU ----

def test_c_harness_compiles_and_links(c_harness):
    assert os.path.getsize(c_harness) > 0


def test_global_functions(ntg_lib):
    ntg_lib.nvttVersion.restype = ctypes.c_uint
    ntg_lib.nvttErrorString.restype = ctypes.c_char_p
    ntg_lib.nvttErrorString.argtypes = [ctypes.c_int]
    assert ntg_lib.nvttVersion() == 20102
    for e in range(7):
        assert ntg_lib.nvttErrorString(e)
    assert b"CUDA" in ntg_lib.nvttErrorString(ERROR_CUDA)


def test_compress_fails_loudly_without_gpu(c_harness, tmp_path):
    if not no_gpu():
        pytest.skip("a GPU is present")
    rc, log, data = run_c(c_harness, 0, tmp_path)
    assert rc == 10 + ERROR_CUDA, log
    assert data.size == 0


# ---- GPU ----

# NVTT's C interface has no setter for the user version word of the DDS header (the C++
# OutputOptions::setUserVersion), so the cases that set one are written by the C++ tests only
C_CASES = [i for i in range(NCASES) if not case(i).get("version")]


@pytest.mark.gpu
@pytest.mark.parametrize("i", C_CASES)
def test_c_compress_matches_reference(c_harness, tmp_path, i):
    rc, log, data = run_c(c_harness, i, tmp_path)
    err = expected_error(i)
    if err is not None:
        assert rc == 10 + err, log
        return
    assert rc == 0, log
    gold = GOLD[f"dds_{i}"]
    np.testing.assert_array_equal(data, gold)
    assert int(log.split("estimate=")[1].split()[0]) == gold.size - header_size(gold)
    assert int(log.split("version=")[1].split()[0]) == 20102


@pytest.mark.gpu
@pytest.mark.parametrize("i", [0, 3])
def test_c_compress_to_file(c_harness, tmp_path, i):
    rc, log, data = run_c(c_harness, i, tmp_path, file=1)
    assert rc == 0, log
    np.testing.assert_array_equal(data, GOLD[f"dds_{i}"])


@pytest.mark.gpu
def test_c_dithering_is_reported(c_harness, tmp_path):
    """Colour dithering belongs to another path: the error callback says so."""
    rc, log, _ = run_c(c_harness, 0, tmp_path, dither=1)
    assert rc == 10 + ERROR_UNSUPPORTED_FEATURE, log
