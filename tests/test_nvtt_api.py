"""The nvtt:: drop-in C++ API (include/nvtt/nvtt.h), driven by a C++ program the way an NVTT user
calls it (tests/cpp/nvtt_harness.cpp), against the bytes the reference's Compressor::process writes
for the same inputs (tests/golden/dds_process.npz, made by tests/golden/make_golden.py).

CPU: the harness compiles and links against libntg.so; the DDS/DX10 headers (Compressor::outputHeader,
no GPU work) equal the reference's; without a GPU, process() reports Error_CudaError instead of
falling back to anything. GPU: whole DDS files are byte-identical, through Compressor::process and
through the Surface loop, and rmsError matches."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "dds_process.npz"))
NCASES = len([k for k in GOLD.files if k.startswith("params_")])
ERROR_CUDA, ERROR_UNSUPPORTED_FEATURE = 3, 2


def case(i):
    return json.loads(str(GOLD[f"params_{i}"]))


def header_size(data):
    if data[:4].tobytes() != b"DDS ":
        return 0
    return 148 if data[84:88].tobytes() == b"DX10" else 128


def harness_args(c, **extra):
    """Harness key=value arguments for a fixture case (the keyword names of Reference.process_ex)."""
    names = dict(w="w", h="h", format="format", quality="quality", mip_filter="filter", alpha_mode="alpha",
                 wrap="wrap", max_level="max_level", container="container", srgb="srgb", version="version",
                 normal_map="normal", normalize_mips="normalize", input_format="input_format", nsrc_levels="nsrc",
                 max_extent="max_extent", round_mode="round_mode", texture_type="type", layers="layers")
    args = {}
    for k, v in c.items():
        if k in names:
            args[names[k]] = int(v)
        elif k == "header":
            args["header"] = int(bool(v))
        elif k == "kaiser":
            args["kw"], args["ka"], args["ks"] = v
        elif k == "gamma":
            args["gin"], args["gout"] = v
        elif k == "cw":
            args["cw_r"], args["cw_g"], args["cw_b"], args["cw_a"] = v
    args.update(extra)
    return [f"{k}={v!r}" if isinstance(v, float) else f"{k}={v}" for k, v in args.items()]


@pytest.fixture(scope="session")
def harness(ntg_lib, tmp_path_factory):
    import ntg
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    libdir = os.path.dirname(ntg.build())
    exe = str(tmp_path_factory.mktemp("nvtt_cpp") / "nvtt_harness")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "nvtt_harness.cpp"), "-L", libdir, "-lntg",
           "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(exe, mode, i, tmp_path, **extra):
    """Runs the harness on fixture case i; returns (exit code, stdout, output bytes)."""
    inp, out = tmp_path / f"in_{i}.bin", tmp_path / f"out_{i}.bin"
    GOLD[f"input_{i}"].tofile(inp)
    r = subprocess.run([exe, mode, str(inp), str(out)] + harness_args(case(i), **extra),
                       capture_output=True, text=True, timeout=300)
    data = np.fromfile(out, np.uint8) if out.exists() else np.zeros(0, np.uint8)
    return r.returncode, r.stdout + r.stderr, data


def expected_error(i):
    g = GOLD[f"dds_{i}"]
    return None if g.dtype == np.uint8 else int(-g[0] - 100)


def no_gpu():
    import torch
    return not torch.cuda.is_available()


# ---- CPU ----

def test_harness_compiles_and_links(harness):
    assert os.path.getsize(harness) > 0


def target_args(i):
    """For a case with the InputOptions resize step or a cube map: the extents the header carries
    (nv::getTargetExtent through ntg_target_extent_ex; the estimate test checks them against the
    reference's file sizes)."""
    import ntg
    c = case(i)
    tt = c.get("texture_type", 0)
    if not c.get("max_extent") and not c.get("round_mode") and tt != 1:
        return {}
    w, h = ntg.target_extent(c["w"], c["h"], c.get("max_extent", 0), c.get("round_mode", 0), tt)
    return dict(w=w, h=h, max_extent=0, round_mode=0)


@pytest.mark.parametrize("i", range(NCASES))
def test_header_matches_reference(harness, tmp_path, i):
    rc, log, data = run(harness, "header", i, tmp_path, **target_args(i))
    err = expected_error(i)
    if err is not None:  # the reference's DDS container rejects the format before writing anything
        assert rc == 10 + err, log
        return
    assert rc == 0, log
    gold = GOLD[f"dds_{i}"]
    n = header_size(gold)
    assert data.size == n
    np.testing.assert_array_equal(data, gold[:n])


@pytest.mark.parametrize("i", [i for i in range(NCASES) if expected_error(i) is None])
def test_estimate_size_matches_reference(harness, tmp_path, i):
    """Compressor::estimateSize(InputOptions) (no GPU work) equals the size of what the reference's process
    writes after the header: the target extent (a cube map's square faces included), the level count and
    the faces or layers."""
    rc, log, _ = run(harness, "estimate", i, tmp_path)
    assert rc == 0, log
    gold = GOLD[f"dds_{i}"]
    assert int(log.split("estimate=")[1].split()[0]) == gold.size - header_size(gold)


def test_process_fails_loudly_without_gpu(harness, tmp_path):
    if not no_gpu():
        pytest.skip("a GPU is present")
    rc, log, data = run(harness, "process", 0, tmp_path)
    assert rc == 10 + ERROR_CUDA, log
    assert data.size == 0


# ---- GPU ----

@pytest.mark.gpu
@pytest.mark.parametrize("i", range(NCASES))
def test_process_matches_reference(harness, tmp_path, i):
    rc, log, data = run(harness, "process", i, tmp_path)
    err = expected_error(i)
    if err is not None:
        assert rc == 10 + err, log
        return
    assert rc == 0, log
    gold = GOLD[f"dds_{i}"]
    assert data.size == gold.size, (data.size, gold.size)
    np.testing.assert_array_equal(data, gold)
    estimate = int(log.split("estimate=")[1].split()[0])
    assert estimate == gold.size - header_size(gold)


@pytest.mark.gpu
@pytest.mark.parametrize("i", [i for i in range(NCASES) if expected_error(i) is None and
                               case(i).get("nsrc_levels", 1) == 1 and case(i).get("texture_type", 0) == 0])
def test_surface_loop_matches_reference(harness, tmp_path, i):
    """The imperative Surface API loop writes the same file as Compressor::process."""
    rc, log, data = run(harness, "surface", i, tmp_path)
    assert rc == 0, log
    gold = GOLD[f"dds_{i}"]
    np.testing.assert_array_equal(data, gold)


@pytest.mark.gpu
@pytest.mark.parametrize("i", sorted(int(k[4:]) for k in GOLD.files if k.startswith("rms_")))
def test_rms_error_matches_reference(harness, tmp_path, i):
    rc, log, _ = run(harness, "rms", i, tmp_path)
    assert rc == 0, log
    got = [float(v) for v in log.split("rms=")[1].split()[:2]]
    np.testing.assert_allclose(got, GOLD[f"rms_{i}"], rtol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("fmt,alpha", [(1, 0), (4, 1), (4, 0)])
def test_srgb_surface_loop_matches_chain(harness, ctx, tmp_path, fmt, alpha):
    """toLinearFromSrgb / toSrgb around the Surface loop equal the fused chain with sRGB transforms."""
    import ntg
    i = 1
    c = case(i)
    w, h = c["w"], c["h"]
    rc, log, data = run(harness, "surface", i, tmp_path, srgb_xform=1, format=fmt, alpha=alpha, quality=1)
    assert rc == 0, log
    opt = ntg.ChainOptions.make(format=fmt, quality=1, filter=c["mip_filter"], wrap=2, alpha_mode=alpha,
                                in_xform=2, out_xform=2)
    chain = ctx.compress_chain_host(GOLD[f"input_{i}"].reshape(h, w, 4), w, h, opt)
    np.testing.assert_array_equal(data[header_size(data):], np.asarray(chain).reshape(-1))


@pytest.mark.gpu
def test_normal_map_renormalisation_is_reported(harness, tmp_path):
    """Renormalising normal-map mipmaps is outside the GPU path: process() says so."""
    i = 10
    rc, log, _ = run(harness, "process", i, tmp_path, normalize=1)
    assert rc == 10 + ERROR_UNSUPPORTED_FEATURE, log
