"""Python binding of the GB300 texture path (libntg.so, C ABI in include/ntg.h).

ctypes over the C ABI; torch supplies device memory and streams. Every compute call goes to the
CUDA kernels in libntg.so: there is no CPU fallback, and a missing or unbuildable library raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libntg.so")

FORMAT_BC1, FORMAT_BC1A, FORMAT_BC3, FORMAT_BC4, FORMAT_BC5 = 1, 2, 4, 6, 7
QUALITY_FASTEST, QUALITY_NORMAL, QUALITY_PRODUCTION, QUALITY_HIGHEST = 0, 1, 2, 3
WRAP_CLAMP, WRAP_REPEAT, WRAP_MIRROR = 0, 1, 2
FILTER_BOX, FILTER_TRIANGLE, FILTER_KAISER = 0, 1, 2
ALPHA_NONE, ALPHA_TRANSPARENCY = 0, 1
XFORM_NONE, XFORM_GAMMA, XFORM_SRGB = 0, 1, 2
TRANSFORM_TO_LINEAR, TRANSFORM_TO_GAMMA, TRANSFORM_FROM_SRGB, TRANSFORM_TO_SRGB = 0, 1, 2, 3  # ntg_transform kinds
# learned encode: a steepest descent from the proposal instead of a window (radius = DESCENT | moves)
NTG_PROPOSAL_DESCENT = 256
NTG_PROPOSAL_REFIT = 512     # BC1: least-squares endpoint refit after the search
# status codes (nvtt::Error values)
NTG_OK, NTG_ERROR_INVALID_INPUT, NTG_ERROR_UNSUPPORTED_FEATURE, NTG_ERROR_CUDA = 0, 1, 2, 3

BLOCK_BYTES = {FORMAT_BC1: 8, FORMAT_BC1A: 8, FORMAT_BC3: 16, FORMAT_BC4: 8, FORMAT_BC5: 16}

_vp, _i, _f, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t


class NtgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ntg error {code}: {msg}")
        self.code = code


class ChainOptions(ctypes.Structure):
    """Mirror of ntg_chain_options."""
    _fields_ = [("format", _i), ("quality", _i), ("filter", _i), ("filter_width", _f), ("params", _f * 2),
                ("wrap", _i), ("alpha_mode", _i), ("in_xform", _i), ("out_xform", _i), ("gamma", _f),
                ("max_levels", _i), ("weighted", _i), ("cw", _f * 3)]

    @classmethod
    def make(cls, format=FORMAT_BC1, quality=QUALITY_NORMAL, filter=FILTER_BOX, filter_width=0.0, params=(0.0, 0.0),
             wrap=WRAP_MIRROR, alpha_mode=ALPHA_NONE, in_xform=XFORM_NONE, out_xform=XFORM_NONE, gamma=2.2,
             max_levels=0, weighted=0, cw=(1.0, 1.0, 1.0)):
        o = cls()
        o.format, o.quality, o.filter, o.filter_width = format, quality, filter, filter_width
        o.params[0], o.params[1] = params
        o.wrap, o.alpha_mode, o.in_xform, o.out_xform, o.gamma = wrap, alpha_mode, in_xform, out_xform, gamma
        o.max_levels, o.weighted = max_levels, weighted
        o.cw[0], o.cw[1], o.cw[2] = cw
        return o


_lib = None


class BatchTexture(ctypes.Structure):
    """Mirror of ntg_batch_texture."""
    _fields_ = [("d_bgra", _vp), ("w", _i), ("h", _i), ("opt", ChainOptions), ("d_blocks", _vp)]


def build(force: bool = False) -> str:
    import importlib.util
    spec = importlib.util.spec_from_file_location("ntg_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    """Loads libntg.so (building it first when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "ntg_version": (_i, []),
        "ntg_launch_count": (ctypes.c_ulonglong, []),
        "ntg_last_error_string": (ctypes.c_char_p, []),
        "ntg_create": (_i, [_i, ctypes.POINTER(_vp)]),
        "ntg_destroy": (_i, [_vp]),
        "ntg_set_image_bgra8": (_i, [_vp, _vp, _i, _i, _i, _f, _vp, _vp]),
        "ntg_mip_level": (_i, [_vp, _vp, _i, _i, _vp, _i, _f, _vp, _i, _i, _i, _vp]),
        "ntg_resize": (_i, [_vp, _vp, _i, _i, _vp, _i, _i, _i, _f, _vp, _i, _i, _vp]),
        "ntg_target_extent": (_i, [_i, _i, _i, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
        "ntg_target_extent_ex": (_i, [_i, _i, _i, _i, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
        "ntg_selftest_srgb_quantizer": (_i, [_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
        "ntg_mip_set_wait_limit": (_i, [_vp, _i]),
        "ntg_mip_status": (_i, [_vp, ctypes.POINTER(ctypes.c_int)]),
        "ntg_encode": (_i, [_vp, _i, _vp, _i, _i, _i, _i, _i, _f, _vp, _vp, _vp]),
        "ntg_encode_noalloc": (_i, [_vp, _i, _vp, _i, _i, _i, _i, _i, _f, _vp, _vp, _vp]),
        "ntg_chain_levels": (_i, [_i, _i, _i]),
        "ntg_chain_bytes": (_sz, [_i, _i, ctypes.POINTER(ChainOptions)]),
        "ntg_compress_chain": (_i, [_vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _vp, _vp]),
        "ntg_compress_chain_host": (_i, [_vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _vp, _vp]),
        "ntg_batch_bind_alternate": (_i, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
        "ntg_batch_launch_alternate": (_i, [_vp, _vp]),
        "ntg_batch_process_host": (_i, [_vp, _i, _vp, _vp, _vp]),
        "ntg_compress_chains_host": (_i, [_vp, _i, ctypes.POINTER(_vp), _i, _i, ctypes.POINTER(ChainOptions),
                                          ctypes.POINTER(_vp), _vp]),
        "ntg_mip_chain": (_i, [_vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _vp, _vp]),
        "ntg_decode": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp]),
        "ntg_profile_enable": (_i, [_vp, _i]),
        "ntg_transform": (_i, [_vp, _vp, _i, _i, _i, _f, _vp]),
        "ntg_profile_read": (_i, [_vp, ctypes.POINTER(_f), ctypes.POINTER(_f)]),
        "ntg_error_sums": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp]),
        "ntg_host_polyphase": (_i, [_i, _f, _vp, _i, _i, _vp, _vp, _i]),
        "ntg_host_transform_tables": (_i, [_i, _i, _f, _vp, _vp, _vp, _vp]),
        "ntg_batch_build": (_i, [_vp, ctypes.POINTER(BatchTexture), _i, ctypes.POINTER(_vp)]),
        "ntg_batch_launch": (_i, [_vp, _vp]),
        "ntg_batch_autotune": (_i, [_vp, _vp]),
        "ntg_batch_info": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                ctypes.POINTER(_i), ctypes.POINTER(_i)]),
        "ntg_batch_destroy": (_i, [_vp]),
        "ntg_batch_time_phases": (_i, [_vp, _vp, ctypes.POINTER(_f), ctypes.POINTER(ctypes.c_longlong)]),
        "ntg_batch_count_work": (_i, [_vp, _vp, ctypes.POINTER(ctypes.c_ulonglong)]),
        "ntg_batch_set_proposal": (_i, [_vp, _vp, _i, _f]),
        "ntg_batch_proposal_stats": (_i, [_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
        "ntg_batch_set_proposal_format": (_i, [_vp, _i, _vp, _i, _f]),
        "ntg_batch_proposal_stats_format": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_ulonglong)]),
        "ntg_mlp_create": (_i, [_i, ctypes.c_ulonglong, ctypes.POINTER(_vp)]),
        "ntg_mlp_destroy": (_i, [_vp]),
        "ntg_mlp_param_count": (_i, []),
        "ntg_mlp_get_params": (_i, [_vp, _vp]),
        "ntg_mlp_set_params": (_i, [_vp, _vp]),
        "ntg_mlp_infer": (_i, [_vp, _vp, _i, _vp, _vp]),
        "ntg_mlp_infer_unfused": (_i, [_vp, _vp, _i, _vp, _vp]),
        "ntg_mlp_gradients": (_i, [_vp, _vp, _vp, _i, _vp, ctypes.POINTER(_f), _vp]),
        "ntg_mlp_train_step": (_i, [_vp, _vp, _vp, _i, _f, _vp, _vp]),
        "ntg_mlp_status": (_i, [_vp]),
        "ntg_mlp_set_wait_limit": (_i, [_vp, _i]),
        "ntg_gemm_bf16": (_i, [_vp, _vp, _i, _i, _i, _vp, _vp]),
        "ntg_compress_chain_learned": (_i, [_vp, _vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _i, _f, _vp,
                                            ctypes.POINTER(ctypes.c_ulonglong), _vp]),
        "ntg_chain_features": (_i, [_vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _vp, _vp]),
        "ntg_compress_chain_proposed": (_i, [_vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _vp, _i, _f, _vp,
                                             ctypes.POINTER(ctypes.c_ulonglong), _vp]),
        "ntg_chain_targets": (_i, [_vp, _vp, _i, _i, ctypes.POINTER(ChainOptions), _vp, _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _lib = L
    return L


def _check(code: int):
    if code != 0:
        raise NtgError(code, lib().ntg_last_error_string().decode())


def _stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def target_extent(w: int, h: int, max_extent: int, round_mode: int, texture_type: int = 0):
    """nv::getTargetExtent (ntg_target_extent_ex): texture_type 0 2D, 1 cube map (square faces), 3 array."""
    ow, oh = _i(), _i()
    _check(lib().ntg_target_extent_ex(w, h, max_extent, round_mode, texture_type, ctypes.byref(ow), ctypes.byref(oh)))
    return ow.value, oh.value


def launch_count() -> int:
    """Kernel launches issued through the library by this process so far (ntg_launch_count)."""
    return int(lib().ntg_launch_count())


def chain_levels(w: int, h: int, max_levels: int = 0):
    out = []
    while True:
        out.append((w, h))
        if (max_levels > 0 and len(out) >= max_levels) or (w == 1 and h == 1):
            break
        w, h = max(1, w // 2), max(1, h // 2)
    return out


def chain_bytes(w: int, h: int, opt: ChainOptions) -> int:
    return int(lib().ntg_chain_bytes(w, h, ctypes.byref(opt)))


def nblocks(w: int, h: int) -> int:
    return ((w + 3) // 4) * ((h + 3) // 4)


class Context:
    """One device's tables and workspace (ntg_context)."""

    def __init__(self, device: int = 0):
        self.h = ctypes.c_void_p()
        _check(lib().ntg_create(device, ctypes.byref(self.h)))
        self.device = device

    def close(self):
        if self.h:
            lib().ntg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- device-buffer calls (torch tensors on this device) --
    def set_image(self, bgra, w, h, in_xform=XFORM_NONE, gamma=2.2, out=None, stream=None):
        import torch
        out = out if out is not None else torch.empty(4 * w * h, dtype=torch.float32, device=bgra.device)
        _check(lib().ntg_set_image_bgra8(self.h, bgra.data_ptr(), w, h, in_xform, gamma, out.data_ptr(), _stream_ptr(stream)))
        return out

    def mip_level(self, src, w, h, filter=FILTER_BOX, width=0.0, params=(0.0, 0.0), wrap=WRAP_MIRROR,
                  alpha_mode=ALPHA_NONE, weighted=0, out=None, stream=None):
        import torch
        dw, dh = max(1, w // 2), max(1, h // 2)
        out = out if out is not None else torch.empty(4 * dw * dh, dtype=torch.float32, device=src.device)
        p = (ctypes.c_float * 2)(*params)
        _check(lib().ntg_mip_level(self.h, src.data_ptr(), w, h, out.data_ptr(), filter, width, ctypes.cast(p, _vp),
                                   wrap, alpha_mode, weighted, _stream_ptr(stream)))
        return out

    def selftest_srgb_quantizer(self) -> int:
        """Disagreements of the mip kernels' sRGB quantiser with the step search over all floats."""
        n = ctypes.c_ulonglong()
        _check(lib().ntg_selftest_srgb_quantizer(self.h, ctypes.byref(n)))
        return n.value

    def set_mip_wait_limit(self, polls: int = -1):
        """Polls of each mbarrier wait of the TMA-staged mip kernels before it gives up (-1: the default)."""
        _check(lib().ntg_mip_set_wait_limit(self.h, polls))

    def mip_status(self) -> int:
        """1 when a mip wait gave up since the previous call (which clears the record), else 0."""
        v = ctypes.c_int()
        _check(lib().ntg_mip_status(self.h, ctypes.byref(v)))
        return v.value

    def resize(self, src, w, h, dw, dh, filter=FILTER_BOX, width=0.0, params=(0.0, 0.0), wrap=WRAP_MIRROR,
               alpha_mode=ALPHA_NONE, out=None, stream=None):
        """Surface::resize of a planar FP32 image to dw x dh (ntg_resize)."""
        import torch
        out = out if out is not None else torch.empty(4 * dw * dh, dtype=torch.float32, device=src.device)
        p = (ctypes.c_float * 2)(*params)
        _check(lib().ntg_resize(self.h, src.data_ptr(), w, h, out.data_ptr(), dw, dh, filter, width, ctypes.cast(p, _vp),
                                wrap, alpha_mode, _stream_ptr(stream)))
        return out

    def encode(self, fmt, rgba, w, h, quality=QUALITY_NORMAL, alpha_mode=ALPHA_NONE, out_xform=XFORM_NONE, gamma=2.2,
               cw=(1.0, 1.0, 1.0), out=None, stream=None):
        import torch
        out = out if out is not None else torch.empty(BLOCK_BYTES[fmt] * nblocks(w, h), dtype=torch.uint8, device=rgba.device)
        c = (ctypes.c_float * 3)(*cw)
        _check(lib().ntg_encode(self.h, fmt, rgba.data_ptr(), w, h, quality, alpha_mode, out_xform, gamma,
                                ctypes.cast(c, _vp), out.data_ptr(), _stream_ptr(stream)))
        return out

    def compress_chain(self, bgra, w, h, opt: ChainOptions, out=None, stream=None):
        import torch
        out = out if out is not None else torch.empty(chain_bytes(w, h, opt), dtype=torch.uint8, device=bgra.device)
        _check(lib().ntg_compress_chain(self.h, bgra.data_ptr(), w, h, ctypes.byref(opt), out.data_ptr(), _stream_ptr(stream)))
        return out

    def compress_chains_host(self, images, w, h, opt: ChainOptions, outs=None, stream=None):
        """Same-shaped host images through the chain with overlapped copies (ntg_compress_chains_host);
        returns the list of output arrays."""
        n = len(images)
        ins = [np.ascontiguousarray(im) for im in images]
        if outs is None:
            outs = [np.empty(chain_bytes(w, h, opt), np.uint8) for _ in range(n)]
        a = (_vp * max(n, 1))(*[im.ctypes.data for im in ins])
        b = (_vp * max(n, 1))(*[o.ctypes.data for o in outs])
        _check(lib().ntg_compress_chains_host(self.h, n, a, w, h, ctypes.byref(opt), b, _stream_ptr(stream)))
        return outs

    def compress_chain_host(self, bgra: np.ndarray, w, h, opt: ChainOptions, out: np.ndarray | None = None, stream=None):
        out = out if out is not None else np.empty(chain_bytes(w, h, opt), np.uint8)
        _check(lib().ntg_compress_chain_host(self.h, bgra.ctypes.data, w, h, ctypes.byref(opt), out.ctypes.data,
                                             _stream_ptr(stream)))
        return out

    def mip_chain(self, bgra, w, h, opt: ChainOptions, out=None, stream=None):
        import torch
        total = sum(4 * lw * lh for lw, lh in chain_levels(w, h, opt.max_levels))
        out = out if out is not None else torch.empty(total, dtype=torch.float32, device=bgra.device)
        _check(lib().ntg_mip_chain(self.h, bgra.data_ptr(), w, h, ctypes.byref(opt), out.data_ptr(), _stream_ptr(stream)))
        return out

    def compress_chain_learned(self, mlp, bgra, w, h, opt: ChainOptions, radius=2, margin=0.01, out=None, stats=True,
                               stream=None):
        """Learned BC1 chain encode; returns (blocks, {kept, full_fit, orderings}) (stats synchronise)."""
        import torch
        out = out if out is not None else torch.empty(chain_bytes(w, h, opt), dtype=torch.uint8, device=bgra.device)
        st = (ctypes.c_ulonglong * 3)()
        _check(lib().ntg_compress_chain_learned(self.h, mlp.h, bgra.data_ptr(), w, h, ctypes.byref(opt), radius, margin,
                                                out.data_ptr(), st if stats else None, _stream_ptr(stream)))
        return out, ({"kept": st[0], "full_fit": st[1], "orderings": st[2]} if stats else None)

    def compress_chain_proposed(self, proposals, bgra, w, h, opt: ChainOptions, radius=2, margin=0.01, out=None,
                                stream=None):
        """The pruned search seeded by caller-supplied proposals ([blocks x 16] float32 device tensor)."""
        import torch
        out = out if out is not None else torch.empty(chain_bytes(w, h, opt), dtype=torch.uint8, device=bgra.device)
        st = (ctypes.c_ulonglong * 3)()
        _check(lib().ntg_compress_chain_proposed(self.h, bgra.data_ptr(), w, h, ctypes.byref(opt), proposals.data_ptr(),
                                                 radius, margin, out.data_ptr(), st, _stream_ptr(stream)))
        return out, {"kept": st[0], "full_fit": st[1], "orderings": st[2]}

    def chain_features(self, bgra, w, h, opt: ChainOptions, stream=None):
        import torch
        n = sum(nblocks(lw, lh) for lw, lh in chain_levels(w, h, opt.max_levels))
        x = torch.empty((n, 48), dtype=torch.float32, device=bgra.device)
        _check(lib().ntg_chain_features(self.h, bgra.data_ptr(), w, h, ctypes.byref(opt), x.data_ptr(), _stream_ptr(stream)))
        return x

    def chain_targets(self, bgra, w, h, opt: ChainOptions, blocks, stream=None):
        import torch
        n = sum(nblocks(lw, lh) for lw, lh in chain_levels(w, h, opt.max_levels))
        t = torch.empty((n, 8), dtype=torch.float32, device=bgra.device)
        _check(lib().ntg_chain_targets(self.h, bgra.data_ptr(), w, h, ctypes.byref(opt), blocks.data_ptr(), t.data_ptr(),
                                       _stream_ptr(stream)))
        return t

    def profile(self, enable: bool = True):
        _check(lib().ntg_profile_enable(self.h, int(enable)))

    def profile_read(self):
        """(mips_ms, encode_ms) of the last chain call, from events on its stream."""
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(lib().ntg_profile_read(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def decode(self, fmt, blocks, w, h, out=None, stream=None):
        import torch
        out = out if out is not None else torch.empty(4 * w * h, dtype=torch.float32, device=blocks.device)
        _check(lib().ntg_decode(self.h, fmt, blocks.data_ptr(), w, h, out.data_ptr(), _stream_ptr(stream)))
        return out

    def error_sums(self, ref, img, w, h, alpha_mode=ALPHA_NONE, out=None, stream=None):
        import torch
        out = out if out is not None else torch.empty(2, dtype=torch.float64, device=ref.device)
        _check(lib().ntg_error_sums(self.h, ref.data_ptr(), img.data_ptr(), w, h, alpha_mode, out.data_ptr(),
                                    _stream_ptr(stream)))
        return out


def split_levels(flat, w, h, max_levels=0):
    """Splits back-to-back planar levels into a list of (4, h_l, w_l) arrays/tensors."""
    out, off = [], 0
    for lw, lh in chain_levels(w, h, max_levels):
        out.append(flat[off: off + 4 * lw * lh].reshape(4, lh, lw))
        off += 4 * lw * lh
    return out


def split_blocks(flat, w, h, fmt, max_levels=0):
    out, off = [], 0
    for lw, lh in chain_levels(w, h, max_levels):
        n = BLOCK_BYTES[fmt] * nblocks(lw, lh)
        out.append(flat[off: off + n])
        off += n
    return out


def host_polyphase(filter, width, params, src, dst):
    ws = lib().ntg_host_polyphase(filter, width, None, src, dst, None, None, 0)
    w = np.zeros(ws * dst, np.float32)
    left = np.zeros(dst, np.int32)
    p = (ctypes.c_float * 2)(*params)
    lib().ntg_host_polyphase(filter, width, ctypes.cast(p, _vp), src, dst, w.ctypes.data, left.ctypes.data, w.size)
    return w.reshape(dst, ws), left


def host_transform_tables(in_xform, out_xform, gamma=2.2):
    lut_in = np.zeros(256, np.float32)
    comp = np.zeros(256, np.float32)
    lut8 = np.zeros(512, np.uint8)
    steps = np.zeros(256, np.float32)
    lib().ntg_host_transform_tables(in_xform, out_xform, gamma, lut_in.ctypes.data, comp.ctypes.data, lut8.ctypes.data,
                                    steps.ctypes.data)
    return lut_in, comp, lut8, steps


class Batch:
    """Many textures' chains as one CUDA graph (ntg_batch). `textures` is a list of
    (bgra device tensor, w, h, ChainOptions, output device tensor); the tensors must outlive the batch."""

    def __init__(self, ctx: "Context", textures):
        self.ctx = ctx
        self._keep = [(t[0], t[4]) for t in textures]
        arr = (BatchTexture * len(textures))()
        for i, (bgra, w, h, opt, out) in enumerate(textures):
            arr[i].d_bgra, arr[i].w, arr[i].h, arr[i].opt, arr[i].d_blocks = bgra.data_ptr(), w, h, opt, out.data_ptr()
        self.h = ctypes.c_void_p()
        _check(lib().ntg_batch_build(ctx.h, arr, len(textures), ctypes.byref(self.h)))

    def launch(self, stream=None, alternate=False):
        fn = lib().ntg_batch_launch_alternate if alternate else lib().ntg_batch_launch
        _check(fn(self.h, _stream_ptr(stream)))

    def bind_alternate(self, inputs, outputs):
        """A second set of device inputs and outputs (one per texture, same sizes) with its own graph,
        replayed by launch(alternate=True); the tensors must outlive the batch."""
        n = len(self._keep)
        assert len(inputs) == n and len(outputs) == n
        self._keep_alt = list(zip(inputs, outputs))
        a = (_vp * n)(*[x.data_ptr() for x in inputs])
        b = (_vp * n)(*[y.data_ptr() for y in outputs])
        _check(lib().ntg_batch_bind_alternate(self.h, a, b))

    def process_host(self, sets, stream=None):
        """The batch over host buffers (ntg_batch_process_host): sets = [(inputs, outputs), ...], one
        host buffer per texture each (numpy arrays or CPU tensors; page-locked ones overlap the copies
        with the neighbouring sets' graphs when an alternate binding is bound). Returns when the last
        set's blocks are on the host."""
        n = len(self._keep)

        def ptr(x):
            return x.data_ptr() if hasattr(x, "data_ptr") else x.ctypes.data

        inner = []
        for ins, outs in sets:
            assert len(ins) == n and len(outs) == n
            inner.append(((_vp * n)(*[ptr(x) for x in ins]), (_vp * n)(*[ptr(y) for y in outs])))
        a = (_vp * len(sets))(*[ctypes.cast(i[0], _vp).value for i in inner])
        b = (_vp * len(sets))(*[ctypes.cast(i[1], _vp).value for i in inner])
        _check(lib().ntg_batch_process_host(self.h, len(sets), ctypes.cast(a, _vp), ctypes.cast(b, _vp),
                                            _stream_ptr(stream)))

    def autotune(self, stream=None):
        _check(lib().ntg_batch_autotune(self.h, _stream_ptr(stream)))

    def info(self):
        tex, blk, n = ctypes.c_longlong(), ctypes.c_longlong(), _i()
        shape = (_i * 6)()
        _check(lib().ntg_batch_info(self.h, ctypes.byref(tex), ctypes.byref(blk), ctypes.byref(n), shape))
        keys = ("strip", "threads", "tail_texels", "bc1_blocks_per_cta", "bc3_blocks_per_cta", "bc5_blocks_per_cta")
        return {"texels": tex.value, "blocks": blk.value, "launches": n.value, "shape": dict(zip(keys, list(shape)))}

    def set_proposal(self, mlp, radius=1, margin=0.5, format=FORMAT_BC1):
        """Learned endpoint proposal for the batch's BC1 (or BC3) Normal blocks (mlp None: the full fit)."""
        if not hasattr(self, "_mlps"):
            self._mlps = {}
        self._mlps[format] = mlp
        _check(lib().ntg_batch_set_proposal_format(self.h, format, mlp.h if mlp is not None else None, radius, margin))

    def proposal_stats(self, format=FORMAT_BC1):
        st = (ctypes.c_ulonglong * 3)()
        _check(lib().ntg_batch_proposal_stats_format(self.h, format, st))
        return {"kept": st[0], "full_fit": st[1], "orderings": st[2]}

    def time_phases(self, stream=None):
        """{mips, bc1, bc3, bc5} ms of one run of each phase outside the graph, and blocks per format."""
        ms = (_f * 4)()
        blocks = (ctypes.c_longlong * 3)()
        _check(lib().ntg_batch_time_phases(self.h, _stream_ptr(stream), ms, blocks))
        return ({"mips": ms[0], "bc1": ms[1], "bc3": ms[2], "bc5": ms[3]},
                {"bc1": blocks[0], "bc3": blocks[1], "bc5": blocks[2]})

    def count_work(self, stream=None):
        """(four-cluster, three-cluster) orderings the BC1 Level8 fit evaluates over the batch."""
        n = (ctypes.c_ulonglong * 2)()
        _check(lib().ntg_batch_count_work(self.h, _stream_ptr(stream), n))
        return int(n[0]), int(n[1])

    def close(self):
        if self.h:
            lib().ntg_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """The learned endpoint proposal's network (ntg_mlp): 48 -> 256 -> 256 -> 8 on the tensor cores."""
    IN, OUT, OUTP = 48, 8, 16

    def __init__(self, device: int = 0, seed: int = 0x4E4554):
        self.h = ctypes.c_void_p()
        _check(lib().ntg_mlp_create(device, seed, ctypes.byref(self.h)))

    @staticmethod
    def param_count() -> int:
        return int(lib().ntg_mlp_param_count())

    def get_params(self) -> np.ndarray:
        p = np.empty(self.param_count(), np.float32)
        _check(lib().ntg_mlp_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.param_count()
        _check(lib().ntg_mlp_set_params(self.h, p.ctypes.data))

    def infer(self, x, out=None, stream=None):
        import torch
        b = x.shape[0]
        out = out if out is not None else torch.empty((b, self.OUTP), dtype=torch.float32, device=x.device)
        _check(lib().ntg_mlp_infer(self.h, x.data_ptr(), b, out.data_ptr(), _stream_ptr(stream)))
        return out

    def infer_unfused(self, x, out=None, stream=None):
        import torch
        b = x.shape[0]
        out = out if out is not None else torch.empty((b, self.OUTP), dtype=torch.float32, device=x.device)
        _check(lib().ntg_mlp_infer_unfused(self.h, x.data_ptr(), b, out.data_ptr(), _stream_ptr(stream)))
        return out

    def gradients(self, x, t, stream=None):
        import torch
        g = torch.empty(self.param_count(), dtype=torch.float32, device=x.device)
        loss = _f()
        _check(lib().ntg_mlp_gradients(self.h, x.data_ptr(), t.data_ptr(), x.shape[0], g.data_ptr(), ctypes.byref(loss),
                                       _stream_ptr(stream)))
        return g, loss.value

    def train_step(self, x, t, lr=1e-3, loss_out=None, stream=None):
        _check(lib().ntg_mlp_train_step(self.h, x.data_ptr(), t.data_ptr(), x.shape[0], lr,
                                        loss_out.data_ptr() if loss_out is not None else None, _stream_ptr(stream)))

    def status(self):
        _check(lib().ntg_mlp_status(self.h))

    def set_wait_limit(self, polls: int = -1):
        """Polls of each tensor-core wait before it gives up (-1: the default); clears the status."""
        _check(lib().ntg_mlp_set_wait_limit(self.h, polls))

    def close(self):
        if self.h:
            lib().ntg_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gemm_bf16(a, b, stream=None):
    """C = A @ B^T with A [M x K], B [N x K] torch bf16 CUDA tensors, through the tensor-core kernel."""
    import torch
    m, k = a.shape
    n = b.shape[0]
    c = torch.empty((m, n), dtype=torch.float32, device=a.device)
    _check(lib().ntg_gemm_bf16(a.data_ptr(), b.data_ptr(), m, n, k, c.data_ptr(), _stream_ptr(stream)))
    return c
