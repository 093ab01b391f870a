"""ctypes bindings for the oracle libraries.

TEST INFRASTRUCTURE ONLY. Imported by tests/, by the smoke check in __graft_entry__.py and by
bench.py's CPU-baseline leg; the product never imports this module.

Two libraries are bound, both built from sources under oracle/:
  * ``Oracle``    -- oracle/_build/libntg_oracle.so, the C restatement of the reference path
                     (oracle/ntg_oracle.c). Builds anywhere gcc runs, the GPU host included.
  * ``Reference`` -- oracle/_ref/libnvtt_ref.so, the reference library compiled from its own
                     sources (oracle/ref/Makefile). Only exists where the reference tree does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libntg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnvtt_ref.so")
# Where the reference's source tree is: $NTG_REFERENCE_ROOT, else the default of the build recipe
# oracle/ref/Makefile (asked with `make print-ref`).
REF_ENV = "NTG_REFERENCE_ROOT"

_vp = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_ll = ctypes.c_longlong


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


def reference_root() -> str:
    """The reference source tree this machine builds from ($NTG_REFERENCE_ROOT or the recipe's default)."""
    root = os.environ.get(REF_ENV)
    if root:
        return root
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", os.path.join(HERE, "ref"), "print-ref"],
                       capture_output=True, text=True)
    return r.stdout.strip()


def build_reference(ref_root: str | None = None) -> str | None:
    """Compile the reference library when its source tree is present; None otherwise."""
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src", "nvtt")):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"), f"REF={ref_root}"], check=True)
    return REF_SO


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _bind(lib, name, res, args):
    fn = getattr(lib, name)
    fn.restype = res
    fn.argtypes = args
    return fn


class Oracle:
    """The C restatement (oracle/ntg_oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        self.lib = lib = ctypes.CDLL(path)
        self._bc1_block = _bind(lib, "ora_bc1_block", _f, [_i, _vp, _vp, _vp, _i, _i, _vp])
        self._bc1_image = _bind(lib, "ora_bc1_image", None, [_vp, _i, _i, _i, _i, _vp, _vp, _i])
        self._bc3_image = _bind(lib, "ora_bc3_image", None, [_vp, _i, _i, _i, _i, _vp, _vp, _i])
        self._bc3_image_u8 = _bind(lib, "ora_bc3_image_u8", None, [_vp, _i, _i, _i, _i, _vp, _vp, _i])
        self._bc5_image = _bind(lib, "ora_bc5_image", None, [_vp, _i, _i, _i, _vp, _i])
        self._bc3_block = _bind(lib, "ora_bc3_block", None, [_vp, _i, _i, _vp, _vp])
        self._bc5_block = _bind(lib, "ora_bc5_block", None, [_vp, _i, _vp])
        self._bc1a_block = _bind(lib, "ora_bc1a_block", None, [_vp, _i, _vp, _vp])
        self._bc4_block = _bind(lib, "ora_bc4_block", None, [_vp, _i, _vp])
        self._bc1a_image = _bind(lib, "ora_bc1a_image", None, [_vp, _i, _i, _i, _vp, _vp, _i])
        self._bc4_image = _bind(lib, "ora_bc4_image", None, [_vp, _i, _i, _i, _vp, _i])
        self._dxt1a_single = _bind(lib, "ora_dxt1a_single_color", None, [_i, _i, _i, ctypes.c_uint32, _vp])
        self._target_extent = _bind(lib, "ora_target_extent", None, [_i, _i, _i, _i, _vp, _vp])
        self._dxt5a_quick = _bind(lib, "ora_dxt5a_quick", None, [_vp, _vp])
        self._dxt5a_optimal = _bind(lib, "ora_dxt5a_optimal", None, [_vp, _vp])
        self._dxt1_single = _bind(lib, "ora_dxt1_single_color", None, [_i, _i, _i, _vp])
        self._quick_dxt1 = _bind(lib, "ora_quick_dxt1", None, [_vp, _vp])
        self._gather = _bind(lib, "ora_colorblock_gather", None, [_vp, _i, _i, _i, _i, _vp])
        self._filter_eval = _bind(lib, "ora_filter_evaluate", _f, [_i, _f, _f, _f, _f])
        self._poly = _bind(lib, "ora_polyphase", _i, [_i, _f, _f, _f, _i, _i, _vp, _i])
        self._poly_left = _bind(lib, "ora_polyphase_left", _i, [_f, _i, _i, _i])
        self._fast_down = _bind(lib, "ora_fast_downsample", None, [_vp, _i, _i, _i, _vp])
        self._resize = _bind(lib, "ora_resize", None, [_vp, _i, _i, _i, _i, _i, _i, _f, _f, _f, _i, _vp])
        self._resize_w = _bind(lib, "ora_resize_weighted", None, [_vp, _i, _i, _i, _i, _i, _f, _f, _f, _i, _vp])
        self._mip_chain = _bind(lib, "ora_mip_chain", _i, [_vp, _i, _i, _i, _f, _f, _f, _i, _i, _i, _i, _f, _i, _vp, _vp])
        self._set_image = _bind(lib, "ora_set_image_bgra8", None, [_vp, _i, _vp])
        self._p115 = _bind(lib, "ora_powf_11_5", None, [_vp, _vp, _i])
        self._p511 = _bind(lib, "ora_powf_5_11", None, [_vp, _vp, _i])
        self._to_srgb = _bind(lib, "ora_to_srgb", None, [_vp, _vp, _i])
        self._from_srgb = _bind(lib, "ora_from_srgb", None, [_vp, _vp, _i])
        self._decode = _bind(lib, "ora_decode", _i, [_i, _vp, _i, _i, _vp])
        self._rms = _bind(lib, "ora_rms", _i, [_i, _vp, _vp, _i, _i, _i, _vp, _vp])
        self._srgb_check = _bind(lib, "ora_count_srgb_step_mismatches", _ll, [_vp, _i])

    def count_srgb_step_mismatches(self, steps, threads=8):
        s = np.ascontiguousarray(steps, np.float32)
        return self._srgb_check(_ptr(s), threads)

    # -- blocks --
    def bc1_block(self, level, colors, weights, cw=(1, 1, 1), three=1, black=1):
        c = np.ascontiguousarray(colors, np.float32).reshape(64)
        w = np.ascontiguousarray(weights, np.float32).reshape(16)
        cwa = np.asarray(cw, np.float32)
        out = np.zeros(8, np.uint8)
        err = self._bc1_block(level, _ptr(c), _ptr(w), _ptr(cwa), three, black, _ptr(out))
        return out, err

    def bc3_block(self, bgra64, alpha_mode=0, quality=1, cw=(1, 1, 1)):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(16, np.uint8)
        self._bc3_block(_ptr(b), alpha_mode, quality, _ptr(np.asarray(cw, np.float32)), _ptr(out))
        return out

    def bc5_block(self, bgra64, quality=1):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(16, np.uint8)
        self._bc5_block(_ptr(b), quality, _ptr(out))
        return out

    def bc1a_block(self, bgra64, alpha_mode=0, cw=(1, 1, 1)):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(8, np.uint8)
        self._bc1a_block(_ptr(b), alpha_mode, _ptr(np.asarray(cw, np.float32)), _ptr(out))
        return out

    def bc4_block(self, bgra64, quality=1):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(8, np.uint8)
        self._bc4_block(_ptr(b), quality, _ptr(out))
        return out

    def target_extent(self, w, h, max_extent, round_mode):
        ow, oh = _i(), _i()
        self._target_extent(w, h, max_extent, round_mode, ctypes.byref(ow), ctypes.byref(oh))
        return ow.value, oh.value

    def dxt1a_single_color(self, r, g, b, alpha_mask):
        out = np.zeros(8, np.uint8)
        self._dxt1a_single(r, g, b, alpha_mask, _ptr(out))
        return out

    def dxt5a_quick(self, a16):
        a = np.ascontiguousarray(a16, np.uint8)
        out = np.zeros(8, np.uint8)
        self._dxt5a_quick(_ptr(a), _ptr(out))
        return out

    def dxt5a_optimal(self, a16):
        a = np.ascontiguousarray(a16, np.uint8)
        out = np.zeros(8, np.uint8)
        self._dxt5a_optimal(_ptr(a), _ptr(out))
        return out

    def dxt1_single_color(self, r, g, b):
        out = np.zeros(8, np.uint8)
        self._dxt1_single(r, g, b, _ptr(out))
        return out

    def quick_dxt1(self, bgra64):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(8, np.uint8)
        self._quick_dxt1(_ptr(b), _ptr(out))
        return out

    def colorblock_gather(self, rgba, w, h, x, y):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(64, np.uint8)
        self._gather(_ptr(r), w, h, x, y, _ptr(out))
        return out

    # -- images --
    def bc1a_image(self, rgba, w, h, alpha_mode=0, cw=(1, 1, 1), threads=1):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(8 * self.nblocks(w, h), np.uint8)
        self._bc1a_image(_ptr(r), w, h, alpha_mode, _ptr(np.asarray(cw, np.float32)), _ptr(out), threads)
        return out

    def bc4_image(self, rgba, w, h, quality=1, threads=1):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(8 * self.nblocks(w, h), np.uint8)
        self._bc4_image(_ptr(r), w, h, quality, _ptr(out), threads)
        return out

    @staticmethod
    def nblocks(w, h):
        return ((w + 3) // 4) * ((h + 3) // 4)

    def bc1_image(self, rgba, w, h, alpha_mode=0, quality=1, cw=(1, 1, 1), threads=1):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(8 * self.nblocks(w, h), np.uint8)
        self._bc1_image(_ptr(r), w, h, alpha_mode, quality, _ptr(np.asarray(cw, np.float32)), _ptr(out), threads)
        return out

    def bc3_image(self, rgba, w, h, alpha_mode=0, quality=1, cw=(1, 1, 1), threads=1):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(16 * self.nblocks(w, h), np.uint8)
        self._bc3_image(_ptr(r), w, h, alpha_mode, quality, _ptr(np.asarray(cw, np.float32)), _ptr(out), threads)
        return out

    def bc3_image_u8(self, bgra, w, h, alpha_mode=0, quality=1, cw=(1, 1, 1), threads=1):
        b = np.ascontiguousarray(bgra, np.uint8)
        out = np.zeros(16 * self.nblocks(w, h), np.uint8)
        self._bc3_image_u8(_ptr(b), w, h, alpha_mode, quality, _ptr(np.asarray(cw, np.float32)), _ptr(out), threads)
        return out

    def bc5_image(self, rgba, w, h, quality=1, threads=1):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(16 * self.nblocks(w, h), np.uint8)
        self._bc5_image(_ptr(r), w, h, quality, _ptr(out), threads)
        return out

    # -- filters / mips --
    def filter_evaluate(self, filt, width, p0, p1, x):
        return self._filter_eval(filt, width, p0, p1, x)

    def polyphase(self, filt, width, p0, p1, src, dst):
        ws = self._poly(filt, width, p0, p1, src, dst, None, 0)
        out = np.zeros(ws * dst, np.float32)
        self._poly(filt, width, p0, p1, src, dst, _ptr(out), out.size)
        return out.reshape(dst, ws)

    def polyphase_left(self, width, src, dst, i):
        return self._poly_left(width, src, dst, i)

    def fast_downsample(self, rgba, w, h, channels=4):
        s = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(channels * max(1, w // 2) * max(1, h // 2), np.float32)
        self._fast_down(_ptr(s), w, h, channels, _ptr(out))
        return out

    def resize(self, rgba, w, h, dw, dh, filt, width, p0=0.0, p1=0.0, wrap=2, channels=4):
        s = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(channels * dw * dh, np.float32)
        self._resize(_ptr(s), w, h, channels, dw, dh, filt, width, p0, p1, wrap, _ptr(out))
        return out

    def resize_weighted(self, rgba, w, h, dw, dh, filt, width, p0=0.0, p1=0.0, wrap=2):
        s = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(4 * dw * dh, np.float32)
        self._resize_w(_ptr(s), w, h, dw, dh, filt, width, p0, p1, wrap, _ptr(out))
        return out

    def mip_chain(self, bgra, w, h, filt, width, p0=0.0, p1=0.0, wrap=2, alpha_mode=0, in_xform=0,
                  out_xform=0, gamma=2.2, max_levels=64):
        b = np.ascontiguousarray(bgra, np.uint8)
        total = sum(4 * lw * lh for lw, lh in level_sizes(w, h, max_levels))
        lin = np.zeros(total, np.float32)
        enc = np.zeros(total, np.float32)
        n = self._mip_chain(_ptr(b), w, h, filt, width, p0, p1, wrap, alpha_mode, in_xform, out_xform, gamma,
                            max_levels, _ptr(lin), _ptr(enc))
        return split_levels(lin, w, h, n), split_levels(enc, w, h, n)

    # -- transforms --
    def set_image_bgra8(self, bgra, n):
        b = np.ascontiguousarray(bgra, np.uint8)
        out = np.zeros(4 * n, np.float32)
        self._set_image(_ptr(b), n, _ptr(out))
        return out

    def _map(self, fn, x):
        s = np.ascontiguousarray(x, np.float32)
        out = np.zeros_like(s)
        fn(_ptr(s), _ptr(out), s.size)
        return out

    def powf_11_5(self, x):
        return self._map(self._p115, x)

    def powf_5_11(self, x):
        return self._map(self._p511, x)

    def to_srgb(self, x):
        return self._map(self._to_srgb, x)

    def from_srgb(self, x):
        return self._map(self._from_srgb, x)

    # -- decode / rms --
    def decode(self, fmt, blocks, w, h):
        b = np.ascontiguousarray(blocks, np.uint8)
        out = np.zeros(4 * w * h, np.float32)
        assert self._decode(fmt, _ptr(b), w, h, _ptr(out)) == 0
        return out

    def rms(self, fmt, rgba, blocks, w, h, alpha_mode=0):
        r = np.ascontiguousarray(rgba, np.float32)
        b = np.ascontiguousarray(blocks, np.uint8)
        c, a = _f(), _f()
        assert self._rms(fmt, _ptr(r), _ptr(b), w, h, alpha_mode, ctypes.byref(c), ctypes.byref(a)) == 0
        return c.value, a.value


class Reference:
    """The reference library compiled from its own sources (oracle/_ref/libnvtt_ref.so)."""

    def __init__(self, path: str = REF_SO):
        self.lib = lib = ctypes.CDLL(path)
        self._icbc = _bind(lib, "ref_icbc_compress_dxt1", _f, [_i, _vp, _vp, _vp, _i, _i, _vp])
        self._compress = _bind(lib, "ref_compress_planar", _ll, [_vp, _i, _i, _i, _i, _i, _vp, _vp, _ll])
        self._bc3_block = _bind(lib, "ref_bc3_block", None, [_vp, _i, _i, _vp, _vp])
        self._bc5_block = _bind(lib, "ref_bc5_block", None, [_vp, _i, _vp])
        self._bc1a_block = _bind(lib, "ref_bc1a_block", None, [_vp, _i, _vp, _vp])
        self._bc4_block = _bind(lib, "ref_bc4_block", None, [_vp, _i, _vp])
        self._dxt5a_quick = _bind(lib, "ref_dxt5a_quick", None, [_vp, _vp])
        self._surface_resize = _bind(lib, "ref_surface_resize", None, [_vp, _i, _i, _i, _i, _i, _f, _f, _f, _i, _i, _vp])
        self._target_extent = _bind(lib, "ref_target_extent", None, [_i, _i, _i, _i, _vp, _vp])
        self._target_extent_type = _bind(lib, "ref_target_extent_type", None, [_i, _i, _i, _i, _i, _vp, _vp])
        self._dxt5a_optimal = _bind(lib, "ref_dxt5a_optimal", None, [_vp, _vp])
        self._dxt1_single = _bind(lib, "ref_dxt1_single_color", None, [_i, _i, _i, _vp])
        self._quick_dxt1 = _bind(lib, "ref_quick_dxt1", None, [_vp, _vp])
        self._gather = _bind(lib, "ref_colorblock_init", None, [_vp, _i, _i, _i, _i, _vp])
        self._poly = _bind(lib, "ref_polyphase", _i, [_i, _f, _f, _f, _i, _i, _vp, _i])
        self._filter_eval = _bind(lib, "ref_filter_evaluate", _f, [_i, _f, _f, _f, _f])
        self._p115 = _bind(lib, "ref_powf_11_5", None, [_vp, _vp, _i])
        self._p511 = _bind(lib, "ref_powf_5_11", None, [_vp, _vp, _i])
        self._mip_chain = _bind(lib, "ref_mip_chain", _i, [_vp, _i, _i, _i, _f, _f, _f, _i, _i, _i, _i, _f, _i, _vp, _vp])
        self._resize_w = _bind(lib, "ref_resize_weighted", None, [_vp, _i, _i, _i, _i, _i, _f, _f, _f, _i, _vp])
        self._decode = _bind(lib, "ref_decode", _i, [_i, _vp, _i, _i, _vp])
        self._rms = _bind(lib, "ref_rms", _i, [_i, _vp, _vp, _i, _i, _i, _vp, _vp])
        self._process = _bind(lib, "ref_process", _ll, [_vp, _i, _i, _i, _i, _i, _i, _i, _f, _f, _i, _i, _vp, _ll])
        self._process_ex = _bind(lib, "ref_process_ex", _ll,
                                 [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _ll])

    def bc1_block(self, level, colors, weights, cw=(1, 1, 1), three=1, black=1):
        c = np.ascontiguousarray(colors, np.float32).reshape(64)
        w = np.ascontiguousarray(weights, np.float32).reshape(16)
        out = np.zeros(8, np.uint8)
        err = self._icbc(level, _ptr(c), _ptr(w), _ptr(np.asarray(cw, np.float32)), three, black, _ptr(out))
        return out, err

    def surface_resize(self, rgba, w, h, dw, dh, filt, width, p0=0.0, p1=0.0, wrap=2, alpha_mode=0):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(4 * dw * dh, np.float32)
        self._surface_resize(_ptr(r), w, h, dw, dh, filt, width, p0, p1, wrap, alpha_mode, _ptr(out))
        return out

    def target_extent(self, w, h, max_extent, round_mode, texture_type=None):
        """nv::getTargetExtent; texture_type (nvtt::TextureType) None keeps the 2D entry point."""
        ow, oh = _i(), _i()
        if texture_type is None:
            self._target_extent(w, h, max_extent, round_mode, ctypes.byref(ow), ctypes.byref(oh))
        else:
            self._target_extent_type(w, h, max_extent, round_mode, texture_type, ctypes.byref(ow), ctypes.byref(oh))
        return ow.value, oh.value

    def compress(self, rgba, w, h, fmt, quality=1, alpha_mode=0, cw=(1, 1, 1, 1)):
        r = np.ascontiguousarray(rgba, np.float32)
        bs = 8 if fmt in (1, 2, 6) else 16
        out = np.zeros(bs * Oracle.nblocks(w, h), np.uint8)
        n = self._compress(_ptr(r), w, h, alpha_mode, fmt, quality, _ptr(np.asarray(cw, np.float32)), _ptr(out), out.size)
        assert n == out.size, n
        return out

    def bc3_block(self, bgra64, alpha_mode=0, quality=1, cw=(1, 1, 1, 1)):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(16, np.uint8)
        self._bc3_block(_ptr(b), alpha_mode, quality, _ptr(np.asarray(cw, np.float32)), _ptr(out))
        return out

    def bc5_block(self, bgra64, quality=1):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(16, np.uint8)
        self._bc5_block(_ptr(b), quality, _ptr(out))
        return out

    def bc1a_block(self, bgra64, alpha_mode=0, cw=(1, 1, 1, 1)):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(8, np.uint8)
        self._bc1a_block(_ptr(b), alpha_mode, _ptr(np.asarray(cw, np.float32)), _ptr(out))
        return out

    def bc4_block(self, bgra64, quality=1):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(8, np.uint8)
        self._bc4_block(_ptr(b), quality, _ptr(out))
        return out

    def dxt5a_quick(self, a16):
        a = np.ascontiguousarray(a16, np.uint8)
        out = np.zeros(8, np.uint8)
        self._dxt5a_quick(_ptr(a), _ptr(out))
        return out

    def dxt5a_optimal(self, a16):
        a = np.ascontiguousarray(a16, np.uint8)
        out = np.zeros(8, np.uint8)
        self._dxt5a_optimal(_ptr(a), _ptr(out))
        return out

    def dxt1_single_color(self, r, g, b):
        out = np.zeros(8, np.uint8)
        self._dxt1_single(r, g, b, _ptr(out))
        return out

    def quick_dxt1(self, bgra64):
        b = np.ascontiguousarray(bgra64, np.uint8).reshape(64)
        out = np.zeros(8, np.uint8)
        self._quick_dxt1(_ptr(b), _ptr(out))
        return out

    def colorblock_gather(self, rgba, w, h, x, y):
        r = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(64, np.uint8)
        self._gather(_ptr(r), w, h, x, y, _ptr(out))
        return out

    def polyphase(self, filt, width, p0, p1, src, dst):
        ws = self._poly(filt, width, p0, p1, src, dst, None, 0)
        out = np.zeros(ws * dst, np.float32)
        self._poly(filt, width, p0, p1, src, dst, _ptr(out), out.size)
        return out.reshape(dst, ws)

    def filter_evaluate(self, filt, width, p0, p1, x):
        return self._filter_eval(filt, width, p0, p1, x)

    def powf_11_5(self, x):
        s = np.ascontiguousarray(x, np.float32)
        out = np.zeros_like(s)
        self._p115(_ptr(s), _ptr(out), s.size)
        return out

    def powf_5_11(self, x):
        s = np.ascontiguousarray(x, np.float32)
        out = np.zeros_like(s)
        self._p511(_ptr(s), _ptr(out), s.size)
        return out

    def mip_chain(self, bgra, w, h, filt, width, p0=0.0, p1=0.0, wrap=2, alpha_mode=0, in_xform=0,
                  out_xform=0, gamma=2.2, max_levels=64):
        b = np.ascontiguousarray(bgra, np.uint8)
        total = sum(4 * lw * lh for lw, lh in level_sizes(w, h, max_levels))
        lin = np.zeros(total, np.float32)
        enc = np.zeros(total, np.float32)
        n = self._mip_chain(_ptr(b), w, h, filt, width, p0, p1, wrap, alpha_mode, in_xform, out_xform, gamma,
                            max_levels, _ptr(lin), _ptr(enc))
        return split_levels(lin, w, h, n), split_levels(enc, w, h, n)

    def resize_weighted(self, rgba, w, h, dw, dh, filt, width, p0=0.0, p1=0.0, wrap=2):
        s = np.ascontiguousarray(rgba, np.float32)
        out = np.zeros(4 * dw * dh, np.float32)
        self._resize_w(_ptr(s), w, h, dw, dh, filt, width, p0, p1, wrap, _ptr(out))
        return out

    def decode(self, fmt, blocks, w, h):
        b = np.ascontiguousarray(blocks, np.uint8)
        out = np.zeros(4 * w * h, np.float32)
        assert self._decode(fmt, _ptr(b), w, h, _ptr(out)) == 0
        return out

    def rms(self, fmt, rgba, blocks, w, h, alpha_mode=0):
        r = np.ascontiguousarray(rgba, np.float32)
        b = np.ascontiguousarray(blocks, np.uint8)
        c, a = _f(), _f()
        assert self._rms(fmt, _ptr(r), _ptr(b), w, h, alpha_mode, ctypes.byref(c), ctypes.byref(a)) == 0
        return c.value, a.value

    def process(self, bgra, w, h, fmt, quality=1, mip_filter=0, alpha_mode=0, wrap=2, in_gamma=2.2,
                out_gamma=2.2, max_level=-1, header=True, cap=None):
        b = np.ascontiguousarray(bgra, np.uint8)
        cap = cap or (16 * Oracle.nblocks(w, h) * 2 + 4096)
        out = np.zeros(cap, np.uint8)
        n = self._process(_ptr(b), w, h, fmt, quality, mip_filter, alpha_mode, wrap, in_gamma, out_gamma,
                          max_level, int(header), _ptr(out), cap)
        assert n >= 0, n
        return out[:n]

    def process_ex(self, data, w, h, fmt, input_format=0, nsrc_levels=1, quality=1, mip_filter=0, alpha_mode=0,
                   wrap=2, max_level=-1, header=True, kaiser=(3.0, 4.0, 1.0), gamma=(2.2, 2.2), cw=(1, 1, 1, 1),
                   container=0, srgb=0, version=0, normal_map=0, normalize_mips=1, max_extent=0, round_mode=0,
                   texture_type=0, layers=1):
        """Compressor::process with containers, flags, Kaiser parameters, source mipmaps, float
        input, cube maps (texture_type 1) and arrays (3, `layers` images); returns the bytes, or the
        negative nvtt::Error - 100 on failure."""
        b = np.ascontiguousarray(data).view(np.uint8)
        opts = np.array(list(kaiser) + list(gamma) + list(cw), np.float32)
        flags = np.array([container, srgb, version, normal_map, normalize_mips, max_extent, round_mode, texture_type,
                          layers], np.int32)
        side = 1 << (max(w, h) - 1).bit_length()  # rounding modes may grow the extents up to the next power of two
        faces = 6 if texture_type == 1 else (layers if texture_type == 3 else 1)
        cap = faces * 16 * Oracle.nblocks(side, side) * 2 + 4096
        out = np.zeros(cap, np.uint8)
        n = self._process_ex(_ptr(b), w, h, input_format, nsrc_levels, fmt, quality, mip_filter, alpha_mode, wrap,
                             max_level, int(header), _ptr(opts), _ptr(flags), _ptr(out), cap)
        return out[:n] if n >= 0 else n


def level_sizes(w, h, max_levels=64):
    out = []
    while True:
        out.append((w, h))
        if len(out) >= max_levels or (w == 1 and h == 1):
            break
        w, h = max(1, w // 2), max(1, h // 2)
    return out


def split_levels(flat, w, h, n):
    out, off = [], 0
    for lw, lh in level_sizes(w, h, n):
        out.append(flat[off: off + 4 * lw * lh].reshape(4, lh, lw))
        off += 4 * lw * lh
    return out
