"""CPU checks of the product boundary: libntg.so builds, loads and exports every entry point of
include/ntg.h, and its host-side tables equal the oracle's (no GPU needed)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if hdr.endswith(".h"):
            text = open(os.path.join(ROOT, "include", hdr)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(ntg_\w+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(ntg_lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(ntg_lib, n)]
    assert not missing, missing


def test_version(ntg_lib):
    assert ntg_lib.ntg_version() == 20102


@pytest.mark.parametrize("filt,width,params", [(0, 0.5, (0, 0)), (0, 1.0, (0, 0)), (1, 1.0, (0, 0)),
                                               (2, 3.0, (4.0, 1.0)), (2, 2.0, (2.0, 0.9))])
def test_host_polyphase_matches_oracle(oracle, filt, width, params):
    import ntg
    for src in [1, 2, 3, 7, 16, 33, 256, 1023, 4096]:
        dst = max(1, src // 2)
        w, left = ntg.host_polyphase(filt, width, params, src, dst)
        ref = oracle.polyphase(filt, width, params[0], params[1], src, dst)
        assert np.array_equal(w.view(np.uint32), ref.view(np.uint32))
        assert [oracle.polyphase_left(width, src, dst, i) for i in range(dst)] == list(left)


@pytest.mark.parametrize("in_x,out_x", [(0, 0), (1, 1), (2, 2), (2, 0), (0, 2)])
def test_host_transform_tables_match_oracle(oracle, in_x, out_x):
    import ntg
    lut_in, comp, lut8, _ = ntg.host_transform_tables(in_x, out_x, 2.2)
    v = np.arange(256, dtype=np.uint8)
    bgra = np.stack([v, v, v, v], axis=1)
    img = oracle.set_image_bgra8(bgra, 256)  # planar r, g, b, a = v / 255
    x = img[:256].copy()
    lin = x if in_x == 0 else (oracle.powf_11_5(x) if in_x == 1 else oracle.from_srgb(x))
    assert np.array_equal(lut_in.view(np.uint32), lin.view(np.uint32))
    enc = lin if out_x == 0 else (oracle.powf_5_11(lin) if out_x == 1 else oracle.to_srgb(lin))
    assert np.array_equal(comp.view(np.uint32), enc.view(np.uint32))
    planar = np.concatenate([enc, enc, enc, img[768:]]).astype(np.float32)
    # ColorBlock quantiser on a 256x1 image, four texels per block
    q = np.concatenate([oracle.colorblock_gather(planar, 256, 1, x0, 0).reshape(16, 4)[:4] for x0 in range(0, 256, 4)])
    assert np.array_equal(lut8[:256], q[:, 2])
    assert np.array_equal(lut8[256:], q[:, 3])


def test_srgb_quantiser_steps_are_exact(oracle):
    """Counting the host-computed steps reproduces toSrgb + quantisation for every float in [0, 1]."""
    import ntg
    steps = ntg.host_transform_tables(2, 2, 2.2)[3]
    assert np.all(np.diff(steps[1:]) > 0)
    assert oracle.count_srgb_step_mismatches(steps, threads=8) == 0
