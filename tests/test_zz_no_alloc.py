"""ntg_encode_noalloc: the allocation-free encode entry point, for callers that cannot call cudaMalloc
(engines that own all GPU memory through their own pools, frame loops that must not synchronise).

Called through the C ABI and checked against the ordinary entry point ntg_encode, bit for bit (the
tolerance every encoder test here uses), on two calls in a row so that the second call runs on
scratch the first one left behind. Collected last on purpose; it also passes alone in a fresh
process (it creates its own context)."""
import ctypes

import numpy as np
import pytest

import ntg

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _encode(entry, ctx, fmt, img, w, h, quality, alpha_mode, out_xform):
    out = torch.full((ntg.BLOCK_BYTES[fmt] * ntg.nblocks(w, h),), 0xCD, dtype=torch.uint8, device="cuda")
    cw = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = entry(ctx.h, fmt, img.data_ptr(), w, h, quality, alpha_mode, out_xform, 2.2, ctypes.cast(cw, ctypes.c_void_p),
               out.data_ptr(), stream)
    assert rc == 0, ntg.lib().ntg_last_error_string().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.fixture(scope="module")
def noalloc_ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = ntg.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("fmt,quality,alpha_mode,out_xform", [
    (ntg.FORMAT_BC1, ntg.QUALITY_NORMAL, ntg.ALPHA_NONE, ntg.XFORM_NONE),
    (ntg.FORMAT_BC1, ntg.QUALITY_NORMAL, ntg.ALPHA_TRANSPARENCY, ntg.XFORM_SRGB),
    (ntg.FORMAT_BC3, ntg.QUALITY_NORMAL, ntg.ALPHA_TRANSPARENCY, ntg.XFORM_SRGB),
    (ntg.FORMAT_BC3, ntg.QUALITY_NORMAL, ntg.ALPHA_NONE, ntg.XFORM_GAMMA),
    (ntg.FORMAT_BC1A, ntg.QUALITY_NORMAL, ntg.ALPHA_TRANSPARENCY, ntg.XFORM_NONE),
    (ntg.FORMAT_BC4, ntg.QUALITY_PRODUCTION, ntg.ALPHA_NONE, ntg.XFORM_NONE),
    (ntg.FORMAT_BC5, ntg.QUALITY_NORMAL, ntg.ALPHA_NONE, ntg.XFORM_NONE),
])
def test_noalloc_matches_encode_on_two_calls(noalloc_ctx, fmt, quality, alpha_mode, out_xform):
    L = ntg.lib()
    rng = np.random.default_rng(fmt * 7 + out_xform)
    for (w, h) in [(96, 40), (61, 33)]:  # second call: other size, over the first call's scratch
        img = torch.from_numpy(rng.random(4 * w * h, dtype=np.float32)).cuda()
        ours = _encode(L.ntg_encode_noalloc, noalloc_ctx, fmt, img, w, h, quality, alpha_mode, out_xform)
        ref = _encode(L.ntg_encode, noalloc_ctx, fmt, img, w, h, quality, alpha_mode, out_xform)
        assert np.array_equal(ours, ref), (fmt, w, h)


def test_noalloc_rejects_levels_above_its_limit(noalloc_ctx):
    w = h = 1025  # 1,050,625 texels > NTG_NOALLOC_MAX_TEXELS (1,048,576)
    img = torch.zeros(4, dtype=torch.float32, device="cuda")  # never read: the size check comes first
    out = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc = ntg.lib().ntg_encode_noalloc(noalloc_ctx.h, ntg.FORMAT_BC3, img.data_ptr(), w, h, 1, 0, 0, 2.2, None,
                                      out.data_ptr(), None)
    assert rc == 1
    assert "scratch limit" in ntg.lib().ntg_last_error_string().decode()


def test_noalloc_runs_on_the_context_device():
    """A caller whose current device is not the context's still gets the context's device (where its
    tables live): the call switches to it, as ntg_encode does."""
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    ctx = ntg.Context(1)
    try:
        L = ntg.lib()
        w, h = 48, 20
        rng = np.random.default_rng(5)
        with torch.cuda.device(1):
            img = torch.from_numpy(rng.random(4 * w * h, dtype=np.float32)).cuda()
            ref = _encode(L.ntg_encode, ctx, ntg.FORMAT_BC3, img, w, h, 1, 1, ntg.XFORM_SRGB)
            out = torch.zeros(16 * ntg.nblocks(w, h), dtype=torch.uint8, device="cuda")
        torch.cuda.set_device(0)
        cw = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
        rc = L.ntg_encode_noalloc(ctx.h, ntg.FORMAT_BC3, img.data_ptr(), w, h, 1, 1, ntg.XFORM_SRGB, 2.2,
                                  ctypes.cast(cw, ctypes.c_void_p), out.data_ptr(), None)
        assert rc == 0, L.ntg_last_error_string().decode()
        torch.cuda.synchronize(1)
        assert np.array_equal(out.cpu().numpy(), ref)
    finally:
        ctx.close()
