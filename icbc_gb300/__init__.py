"""icbc_gb300 -- GB300 (sm_103a) BC1 encoder, a drop-in for icbc's compress path.

Python mirror of the icbc.h surface (``init``, ``compress_bc1``,
``decode_bc1``, ``evaluate_bc1_error`` with the same enum values and argument
meanings) plus the batched forms, all calling the CUDA kernels through the C
ABI of ``include/icbc_gpu.h`` (``icbc_gb300/_lib/libicbc_gpu.so``).  There is
no CPU fallback: without the built library and a CUDA device every call
raises.  PyTorch is used only to hold device buffers and streams.
"""
from __future__ import annotations

import ctypes
import os
import threading
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _build

# icbc::Decoder (icbc.h:12-17)
Decoder_D3D10, Decoder_NVIDIA, Decoder_AMD, Decoder_Intel = 0, 1, 2, 3
DECODER_DEFAULT = -1
# icbc::Quality (icbc.h:21-36)
(Quality_Level0, Quality_Level1, Quality_Level2, Quality_Level3, Quality_Level4, Quality_Level5,
 Quality_Level6, Quality_Level7, Quality_Level8, Quality_Level9) = range(10)
Quality_Fast, Quality_Default, Quality_Max = 1, 8, 9
# weight sources of RGBA8 images
WEIGHTS_UNIFORM, WEIGHTS_ALPHA, WEIGHTS_PLANE = 0, 1, 2
# largest batch of icbc_gpu_compress_bc1_images_noalloc (ICBC_GPU_NOALLOC_MAX_IMAGES)
NOALLOC_MAX_IMAGES = 256
# SIMD builds of the reference whose output the *_simd entry points reproduce.
SIMD_SCALAR, SIMD_SSE2, SIMD_SSE41, SIMD_AVX, SIMD_AVX2, SIMD_AVX512 = 0, 1, 2, 3, 4, 5
SIMD_NEON = -1  # ICBC_SIMD's value for NEON (icbc.h:65)

STATUS = {0: "ok", 1: "invalid argument", 2: "not initialized", 3: "CUDA error", 4: "out of memory",
          5: "misaligned", 6: "over budget", 7: "not ready", 8: "cancelled", 9: "not found"}


class IcbcGpuError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        super().__init__("%s failed: %s%s" % (what, STATUS.get(status, status), (" (%s)" % detail) if detail else ""))


class ImageDesc(ctypes.Structure):
    """struct icbc_gpu_image (include/icbc_gpu.h)."""
    _fields_ = [("rgba", ctypes.c_void_p), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("pitch", ctypes.c_int64), ("weight_mode", ctypes.c_int32), ("weight_plane", ctypes.c_void_p),
                ("weight_pitch", ctypes.c_int64), ("level", ctypes.c_int32), ("decoder", ctypes.c_int32),
                ("three_color_mode", ctypes.c_int32), ("three_color_black", ctypes.c_int32),
                ("color_weights", ctypes.c_float * 3), ("out", ctypes.c_void_p), ("errors", ctypes.c_void_p)]


class LaunchConfig(ctypes.Structure):
    """struct icbc_gpu_launch_config."""
    _fields_ = [("groups_per_warp", ctypes.c_int32), ("persistent", ctypes.c_int32), ("cta_warps", ctypes.c_int32),
                ("batch_cta_warps", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    """struct icbc_gpu_server_config."""
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_inflight", ctypes.c_int32),
                ("max_batch_images", ctypes.c_int32)]


class RequestDesc(ctypes.Structure):
    """struct icbc_gpu_request."""
    _fields_ = [("rgba", ctypes.c_void_p), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("pitch", ctypes.c_int64), ("weight_mode", ctypes.c_int32), ("level", ctypes.c_int32),
                ("decoder", ctypes.c_int32), ("three_color_mode", ctypes.c_int32),
                ("three_color_black", ctypes.c_int32), ("color_weights", ctypes.c_float * 3),
                ("out", ctypes.c_void_p), ("errors", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    """struct icbc_gpu_server_stats."""
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "rejected", "cancelled", "failed",
                                              "pending", "in_flight", "batches", "arena_bytes", "arena_used",
                                              "arena_peak")] + \
               [(n, ctypes.c_double) for n in ("pixels_completed", "latency_mean_ms", "latency_p50_ms",
                                               "latency_p99_ms", "latency_max_ms")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Loads libicbc_gpu.so (building it first if asked).  Raises if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError("icbc_gb300: %s is missing; run icbc_gb300._build.build()" % path)
        L = ctypes.CDLL(path)
        i32, i64, vp, f32p = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)
        sig = {
            "icbc_gpu_init": (i32, [i32]),
            "icbc_gpu_get_decoder": (i32, []),
            "icbc_gpu_status_string": (ctypes.c_char_p, [i32]),
            "icbc_gpu_last_error": (ctypes.c_char_p, []),
            "icbc_gpu_sm_count": (i32, []),
            "icbc_gpu_compress_bc1_blocks": (i32, [i32, vp, vp, f32p, i32, i32, i32, vp, vp, i64, vp]),
            "icbc_gpu_compress_bc1_image": (i32, [ctypes.POINTER(ImageDesc), vp]),
            "icbc_gpu_compress_bc1_blocks_simd": (i32, [i32, i32, vp, vp, f32p, i32, i32, i32, vp, vp, i64, vp]),
            "icbc_gpu_compress_bc1_image_simd": (i32, [i32, ctypes.POINTER(ImageDesc), vp]),
            "icbc_gpu_batch_create": (i32, [ctypes.POINTER(ImageDesc), i32, ctypes.POINTER(vp)]),
            "icbc_gpu_batch_launch": (i32, [vp, vp]),
            "icbc_gpu_batch_destroy": (i32, [vp]),
            "icbc_gpu_compress_bc1_images": (i32, [ctypes.POINTER(ImageDesc), i32, vp]),
            "icbc_gpu_compress_bc1_images_each": (i32, [ctypes.POINTER(ImageDesc), i32, vp]),
            "icbc_gpu_decode_bc1": (i32, [vp, vp, i64, i32, vp]),
            "icbc_gpu_evaluate_bc1_error": (i32, [vp, vp, vp, i64, i32, vp]),
            "icbc_gpu_decode_bc3": (i32, [vp, vp, i64, i32, vp]),
            "icbc_gpu_evaluate_bc3_error": (i32, [vp, vp, vp, i64, i32, i32, vp]),
            "icbc_gpu_compress_bc1_image_host": (i32, [vp, i32, i32, i64, i32, vp, i32, i32, i32, i32, f32p, vp, vp]),
            "icbc_gpu_debug_tables": (i32, [i32, vp, vp, vp, vp, vp, vp, vp]),
            "icbc_gpu_server_create": (i32, [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]),
            "icbc_gpu_server_submit": (i32, [vp, ctypes.POINTER(RequestDesc), ctypes.POINTER(ctypes.c_uint64)]),
            "icbc_gpu_server_poll": (i32, [vp, ctypes.c_uint64]),
            "icbc_gpu_server_wait": (i32, [vp, ctypes.c_uint64, ctypes.c_int32]),
            "icbc_gpu_server_cancel": (i32, [vp, ctypes.c_uint64]),
            "icbc_gpu_server_get_stats": (i32, [vp, ctypes.POINTER(ServerStats)]),
            "icbc_gpu_server_destroy": (i32, [vp]),
            "icbc_gpu_write_dds": (i32, [ctypes.c_char_p, i32, i32, vp]),
            "icbc_gpu_write_dds_mips": (i32, [ctypes.c_char_p, i32, i32, i32, vp]),
            "icbc_gpu_expand_rgba8": (i32, [vp, i32, i32, i32, i64, vp, i64, vp]),
            "icbc_gpu_mip_levels": (i32, [i32, i32]),
            "icbc_gpu_mip_layout": (i32, [i32, i32, i32, vp, vp, vp]),
            "icbc_gpu_build_mips": (i32, [vp, i32, i32, i64, i32, vp, vp]),
            "icbc_gpu_compress_bc1_mips": (i32, [ctypes.POINTER(ImageDesc), i32, vp]),
            "icbc_gpu_set_launch_config": (i32, [i32, ctypes.POINTER(LaunchConfig)]),
            "icbc_gpu_get_launch_config": (i32, [i32, ctypes.POINTER(LaunchConfig)]),
            "icbc_gpu_write_ktx": (i32, [ctypes.c_char_p, i32, i32, vp]),
            "icbc_gpu_compare_dds": (i32, [ctypes.c_char_p, i32, i32, vp]),
            "icbc_gpu_compress_bc1_images_noalloc": (i32, [ctypes.POINTER(ImageDesc), i32, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int, what: str):
    if status != 0:
        detail = ""
        if status == 3 and _lib is not None:
            detail = (_lib.icbc_gpu_last_error() or b"").decode()
        raise IcbcGpuError(status, what, detail)


def _cw(color_weights):
    arr = (ctypes.c_float * 3)(*[float(x) for x in color_weights])
    return arr


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("icbc_gb300 needs a CUDA device (no CPU fallback)")
    return torch


def _on(stream):
    """Stream context for the staging a call does before its launch (copies,
    zeroed outputs), so it is ordered before the launch on `stream`."""
    import contextlib
    return _torch().cuda.stream(stream) if stream is not None else contextlib.nullcontext()


def _stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


# ------------------------------------------------------------ icbc.h mirror

def init(decoder: int = Decoder_D3D10) -> None:
    """icbc::init (icbc.h:19): uploads the tables and sets the default decoder."""
    _check(load().icbc_gpu_init(int(decoder)), "init")


def get_decoder() -> int:
    return load().icbc_gpu_get_decoder()


def compress_bc1(level: int, input_colors, input_weights, color_weights, three_color_mode: bool,
                 three_color_black: bool, output=None) -> float:
    """icbc::compress_bc1 (icbc.h:48) for one block: 16x4 floats in, 8 bytes out.

    Returns the block's weighted error; writes the block into ``output``
    (a writable 8-byte buffer) when given and returns (error, bytes) otherwise.
    One synchronous device round trip: a correctness path, not a fast one.
    """
    cols = np.ascontiguousarray(input_colors, np.float32).reshape(1, 16, 4)
    w = np.ascontiguousarray(input_weights, np.float32).reshape(1, 16)
    prev = None
    if output is not None:
        prev = np.frombuffer(output, dtype=np.uint8, count=8).reshape(1, 8).copy()
    blocks, errors = compress_blocks(cols, w, level, color_weights=color_weights,
                                     three_color_mode=three_color_mode, three_color_black=three_color_black,
                                     decoder=DECODER_DEFAULT, initial=prev)
    blocks = blocks.cpu().numpy() if hasattr(blocks, "cpu") else blocks
    errors = errors.cpu().numpy() if hasattr(errors, "cpu") else errors
    if output is not None:
        np.frombuffer(output, dtype=np.uint8, count=8)[:] = blocks[0]
        return float(errors[0])
    return float(errors[0]), bytes(blocks[0])


def decode_bc1(block, decoder: int = Decoder_D3D10) -> np.ndarray:
    """icbc::decode_bc1 (icbc.h:38) for one block -> 64 RGBA8 bytes."""
    torch = _torch()
    b = torch.as_tensor(np.frombuffer(bytes(block), np.uint8).reshape(1, 8)).cuda()
    return decode_blocks(b, decoder).cpu().numpy().reshape(64)


def evaluate_bc1_error(rgba_block, block, decoder: int = Decoder_D3D10) -> float:
    """icbc::evaluate_bc1_error (icbc.h:43) for one block."""
    torch = _torch()
    t = torch.as_tensor(np.ascontiguousarray(rgba_block, np.uint8).reshape(1, 64)).cuda()
    b = torch.as_tensor(np.frombuffer(bytes(block), np.uint8).reshape(1, 8)).cuda()
    return float(evaluate_errors(t, b, decoder).cpu()[0])


def debug_tables(decoder: int) -> dict:
    """The init-time tables the library builds (host only, no GPU needed)."""
    L = load()
    t = {"match5": np.zeros(512, np.uint8), "match6": np.zeros(512, np.uint8), "weights": np.zeros(5, np.float32),
         "four": np.zeros(968, np.uint32), "four_total": np.zeros(16, np.int32), "three": np.zeros(152, np.uint32),
         "three_total": np.zeros(16, np.int32)}
    _check(L.icbc_gpu_debug_tables(int(decoder), *[t[k].ctypes.data for k in
                                                   ("match5", "match6", "weights", "four", "four_total", "three",
                                                    "three_total")]), "debug_tables")
    return t


# ---------------------------------------------------------- batched forms

def compress_blocks(colors, weights, level: int, decoder: int = DECODER_DEFAULT, color_weights=(1.0, 1.0, 1.0),
                    three_color_mode: bool = True, three_color_black: bool = True, initial=None, stream=None,
                    out=None, errors=None, simd_profile: int = 0):
    """Encodes n blocks given as compress_bc1 inputs.

    colors: (n,16,4) float32, weights: (n,16) float32 or None (1.0f).  numpy
    arrays are copied to the device and results come back as numpy; CUDA
    tensors stay on the device and (blocks uint8 (n,8), errors float32 (n,))
    tensors are returned.  ``initial`` seeds the output bytes (kept by levels
    4..9 when no candidate has a finite error, as the reference does).
    ``simd_profile`` (SIMD_*) reproduces a SIMD build of the reference.
    """
    torch = _torch()
    L = load()
    with _on(stream):
        return _compress_blocks(torch, L, colors, weights, level, decoder, color_weights, three_color_mode,
                                three_color_black, initial, stream, out, errors, simd_profile)


def _compress_blocks(torch, L, colors, weights, level, decoder, color_weights, three_color_mode, three_color_black,
                     initial, stream, out, errors, simd_profile):
    on_host = not (hasattr(colors, "is_cuda") and colors.is_cuda)
    dev = torch.device("cuda")
    c = torch.as_tensor(np.ascontiguousarray(colors, np.float32) if on_host else colors).to(dev)
    c = c.reshape(-1, 64).contiguous()
    n = c.shape[0]
    w = None
    if weights is not None:
        w = torch.as_tensor(np.ascontiguousarray(weights, np.float32) if on_host else weights).to(dev)
        w = w.reshape(n, 16).contiguous()
    if out is None:
        out = torch.zeros((n, 8), dtype=torch.uint8, device=dev)
        if initial is not None:
            out.copy_(torch.as_tensor(np.ascontiguousarray(initial, np.uint8)).reshape(n, 8))
    if errors is None:
        errors = torch.empty(n, dtype=torch.float32, device=dev)
    cw = _cw(color_weights)
    args = (int(level), c.data_ptr(), None if w is None else w.data_ptr(), cw, int(bool(three_color_mode)),
            int(bool(three_color_black)), int(decoder), out.data_ptr(), errors.data_ptr(), n, _stream_ptr(stream))
    if simd_profile:
        st = L.icbc_gpu_compress_bc1_blocks_simd(int(simd_profile), *args)
    else:
        st = L.icbc_gpu_compress_bc1_blocks(*args)
    _check(st, "compress_bc1_blocks")
    if on_host:
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
        return out.cpu().numpy(), errors.cpu().numpy()
    return out, errors


def image_desc(rgba, level: int, out, errors=None, decoder: int = DECODER_DEFAULT, color_weights=(1.0, 1.0, 1.0),
               weight_mode: int = WEIGHTS_UNIFORM, weight_plane=None, three_color_mode: bool = True,
               three_color_black: bool = True, width: int | None = None, height: int | None = None,
               pitch: int | None = None) -> ImageDesc:
    """Builds an icbc_gpu_image for a CUDA uint8 tensor of shape (h, w, 4)
    (or a flat buffer with explicit width/height/pitch)."""
    d = ImageDesc()
    if width is None:
        height, width = int(rgba.shape[0]), int(rgba.shape[1])
        pitch = int(rgba.stride(0))
    d.rgba = rgba.data_ptr()
    d.width, d.height, d.pitch = int(width), int(height), int(pitch)
    d.weight_mode = int(weight_mode)
    d.weight_plane = weight_plane.data_ptr() if weight_plane is not None else None
    d.weight_pitch = int(weight_plane.stride(0)) if weight_plane is not None else 0
    d.level, d.decoder = int(level), int(decoder)
    d.three_color_mode, d.three_color_black = int(bool(three_color_mode)), int(bool(three_color_black))
    d.color_weights = (ctypes.c_float * 3)(*[float(x) for x in color_weights])
    d.out = out.data_ptr()
    d.errors = errors.data_ptr() if errors is not None else None
    return d


def blocks_of(width: int, height: int) -> int:
    return ((width + 3) // 4) * ((height + 3) // 4)


def compress_image(rgba, level: int, decoder: int = DECODER_DEFAULT, color_weights=(1.0, 1.0, 1.0),
                   weight_mode: int = WEIGHTS_UNIFORM, weight_plane=None, three_color_mode: bool = True,
                   three_color_black: bool = True, out=None, errors=None, with_errors: bool = False, stream=None,
                   simd_profile: int = 0):
    """Plain form: one launch for one RGBA8 image (CUDA uint8 tensor (h,w,4)).
    ``simd_profile`` (SIMD_*) reproduces a SIMD build of the reference."""
    torch = _torch()
    L = load()
    h, w = int(rgba.shape[0]), int(rgba.shape[1])
    nb = blocks_of(w, h)
    with _on(stream):  # the zeroed output is ordered before the launch
        if out is None:
            out = torch.zeros((nb, 8), dtype=torch.uint8, device=rgba.device)
        if errors is None and with_errors:
            errors = torch.empty(nb, dtype=torch.float32, device=rgba.device)
    d = image_desc(rgba, level, out, errors, decoder, color_weights, weight_mode, weight_plane, three_color_mode,
                   three_color_black)
    if simd_profile:
        st = L.icbc_gpu_compress_bc1_image_simd(int(simd_profile), ctypes.byref(d), _stream_ptr(stream))
    else:
        st = L.icbc_gpu_compress_bc1_image(ctypes.byref(d), _stream_ptr(stream))
    _check(st, "compress_bc1_image")
    return (out, errors) if with_errors else out


class Batch:
    """A planned batched launch over many images (icbc_gpu_batch_*)."""

    def __init__(self, descs: Sequence[ImageDesc], keepalive=()):
        L = load()
        arr = (ImageDesc * len(descs))(*descs)
        h = ctypes.c_void_p()
        _check(L.icbc_gpu_batch_create(arr, len(descs), ctypes.byref(h)), "batch_create")
        self._h = h
        self._keep = list(keepalive)

    def launch(self, stream=None):
        _check(load().icbc_gpu_batch_launch(self._h, _stream_ptr(stream)), "batch_launch")

    def close(self):
        if self._h:
            load().icbc_gpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def compress_images_each(descs: Sequence[ImageDesc], stream=None):
    """Plain form over many images: one launch per image, looped in native code."""
    arr = (ImageDesc * len(descs))(*descs)
    _check(load().icbc_gpu_compress_bc1_images_each(arr, len(descs), _stream_ptr(stream)), "compress_bc1_images_each")


def decode_blocks(blocks, decoder: int = Decoder_D3D10, stream=None):
    """decode_bc1 over a CUDA uint8 tensor (n,8) -> (n,64) RGBA8."""
    torch = _torch()
    n = blocks.shape[0]
    with _on(stream):  # a contiguous copy, if any, is ordered before the launch
        b = blocks.contiguous()
        out = torch.empty((n, 64), dtype=torch.uint8, device=blocks.device)
        _check(load().icbc_gpu_decode_bc1(b.data_ptr(), out.data_ptr(), n, int(decoder), _stream_ptr(stream)),
               "decode_bc1")
    return out


def evaluate_errors(rgba_blocks, blocks, decoder: int = Decoder_D3D10, stream=None):
    """evaluate_bc1_error over CUDA tensors (n,64) uint8 and (n,8) uint8 -> (n,) float32."""
    torch = _torch()
    n = blocks.shape[0]
    with _on(stream):  # contiguous copies, if any, are ordered before the launch
        r, b = rgba_blocks.contiguous(), blocks.contiguous()
        out = torch.empty(n, dtype=torch.float32, device=blocks.device)
        _check(load().icbc_gpu_evaluate_bc1_error(r.data_ptr(), b.data_ptr(), out.data_ptr(), n, int(decoder),
                                                  _stream_ptr(stream)), "evaluate_bc1_error")
    return out


def decode_bc3_blocks(blocks, decoder: int = Decoder_D3D10, stream=None):
    """decode_bc3 (as the reference implements it) over a CUDA uint8 tensor
    (n,16) -> (n,64) RGBA8."""
    torch = _torch()
    n = blocks.shape[0]
    with _on(stream):
        b = blocks.contiguous()
        out = torch.empty((n, 64), dtype=torch.uint8, device=blocks.device)
        _check(load().icbc_gpu_decode_bc3(b.data_ptr(), out.data_ptr(), n, int(decoder), _stream_ptr(stream)),
               "decode_bc3")
    return out


def evaluate_bc3_errors(rgba_blocks, blocks, alpha_blend: bool, decoder: int = Decoder_D3D10, stream=None):
    """evaluate_bc3_error over CUDA tensors (n,64) uint8 and (n,16) uint8 -> (n,) float32."""
    torch = _torch()
    n = blocks.shape[0]
    with _on(stream):
        r, b = rgba_blocks.contiguous(), blocks.contiguous()
        out = torch.empty(n, dtype=torch.float32, device=blocks.device)
        _check(load().icbc_gpu_evaluate_bc3_error(r.data_ptr(), b.data_ptr(), out.data_ptr(), n,
                                                  int(bool(alpha_blend)), int(decoder), _stream_ptr(stream)),
               "evaluate_bc3_error")
    return out


def compress_image_host(rgba: np.ndarray, level: int, decoder: int = DECODER_DEFAULT,
                        color_weights=(1.0, 1.0, 1.0), weight_mode: int = WEIGHTS_UNIFORM, weight_plane=None,
                        three_color_mode: bool = True, three_color_black: bool = True, out=None, errors=None):
    """End-to-end call on host buffers: H2D, encode, D2H (synchronous).
    rgba: (h,w,4) uint8 (pinned memory gives the fastest copies)."""
    L = load()
    h, w = int(rgba.shape[0]), int(rgba.shape[1])
    nb = blocks_of(w, h)
    if out is None:
        out = np.zeros((nb, 8), np.uint8)
    plane_ptr = None
    if weight_mode == WEIGHTS_PLANE:
        weight_plane = np.ascontiguousarray(weight_plane, np.float32)
        plane_ptr = weight_plane.ctypes.data
    pitch = rgba.strides[0] if isinstance(rgba, np.ndarray) else 4 * w
    ptr = rgba.ctypes.data if isinstance(rgba, np.ndarray) else rgba.data_ptr()
    optr = out.ctypes.data if isinstance(out, np.ndarray) else out.data_ptr()
    eptr = None
    if errors is not None:
        eptr = errors.ctypes.data if isinstance(errors, np.ndarray) else errors.data_ptr()
    st = L.icbc_gpu_compress_bc1_image_host(ptr, w, h, pitch, int(weight_mode), plane_ptr, int(level), int(decoder),
                                            int(bool(three_color_mode)), int(bool(three_color_black)),
                                            _cw(color_weights), optr, eptr)
    _check(st, "compress_bc1_image_host")
    return out


def _blocks_ptr(blocks):
    return blocks.data_ptr() if hasattr(blocks, "data_ptr") else np.ascontiguousarray(blocks, np.uint8).ctypes.data


def write_dds(path: str, width: int, height: int, blocks) -> None:
    """DDS file (DXT1, one mip) of host (numpy) or device (torch) blocks."""
    b = blocks if hasattr(blocks, "data_ptr") else np.ascontiguousarray(blocks, np.uint8)
    _check(load().icbc_gpu_write_dds(os.fsencode(path), int(width), int(height), _blocks_ptr(b)), "write_dds")


def write_dds_mips(path: str, width: int, height: int, levels: int, blocks) -> None:
    """DDS file of a whole mip chain (blocks of every level, mip_layout order)."""
    b = blocks if hasattr(blocks, "data_ptr") else np.ascontiguousarray(blocks, np.uint8)
    _check(load().icbc_gpu_write_dds_mips(os.fsencode(path), int(width), int(height), int(levels), _blocks_ptr(b)),
           "write_dds_mips")


def expand_rgba8(pixels, stream=None):
    """stbi_load(..., 4)-style expansion on the device: a CUDA uint8 tensor
    (h, w, c) with c in 1..4 (or (h, w) grey) -> (h, w, 4) RGBA8."""
    torch = _torch()
    src = pixels if pixels.dim() == 3 else pixels.unsqueeze(-1)
    h, w, c = (int(x) for x in src.shape)
    src = src.contiguous()
    out = torch.empty((h, w, 4), dtype=torch.uint8, device=src.device)
    _check(load().icbc_gpu_expand_rgba8(src.data_ptr(), c, w, h, w * c, out.data_ptr(), 4 * w, _stream_ptr(stream)),
           "expand_rgba8")
    return out


def mip_levels(width: int, height: int) -> int:
    return int(load().icbc_gpu_mip_levels(int(width), int(height)))


def mip_layout(width: int, height: int, levels: int | None = None):
    """(widths, heights, block_offsets) of a chain (offsets has levels + 1 entries)."""
    levels = mip_levels(width, height) if levels is None else int(levels)
    ws, hs = (ctypes.c_int32 * levels)(), (ctypes.c_int32 * levels)()
    off = (ctypes.c_int64 * (levels + 1))()
    _check(load().icbc_gpu_mip_layout(int(width), int(height), levels, ws, hs, off), "mip_layout")
    return list(ws), list(hs), list(off)


def build_mips(rgba, levels: int | None = None, stream=None):
    """Mip chain of a CUDA RGBA8 tensor (h, w, 4): a list of (h_k, w_k, 4)
    tensors, level 0 being `rgba` itself."""
    torch = _torch()
    h, w = int(rgba.shape[0]), int(rgba.shape[1])
    ws, hs, _ = mip_layout(w, h, levels)
    total = sum(4 * ws[k] * hs[k] for k in range(1, len(ws)))
    chain = torch.empty(max(total, 4), dtype=torch.uint8, device=rgba.device)
    _check(load().icbc_gpu_build_mips(rgba.data_ptr(), w, h, int(rgba.stride(0)), len(ws), chain.data_ptr(),
                                      _stream_ptr(stream)), "build_mips")
    out, pos = [rgba], 0
    for k in range(1, len(ws)):
        n = 4 * ws[k] * hs[k]
        out.append(chain[pos:pos + n].view(hs[k], ws[k], 4))
        pos += n
    return out


def compress_mips(rgba, level: int, levels: int | None = None, decoder: int = DECODER_DEFAULT,
                  color_weights=(1.0, 1.0, 1.0), weight_mode: int = WEIGHTS_UNIFORM, three_color_mode: bool = True,
                  three_color_black: bool = True, with_errors: bool = False, stream=None):
    """Builds the mip chain of a CUDA RGBA8 tensor (h, w, 4) and encodes every
    level in one batch.  Returns (blocks (total, 8)[, errors], block_offsets)."""
    torch = _torch()
    h, w = int(rgba.shape[0]), int(rgba.shape[1])
    ws, hs, off = mip_layout(w, h, levels)
    with _on(stream):  # the zeroed output is ordered before the launches
        out = torch.zeros((off[-1], 8), dtype=torch.uint8, device=rgba.device)
        errors = torch.empty(off[-1], dtype=torch.float32, device=rgba.device) if with_errors else None
    d = image_desc(rgba, level, out, errors, decoder, color_weights, weight_mode, None, three_color_mode,
                   three_color_black)
    _check(load().icbc_gpu_compress_bc1_mips(ctypes.byref(d), len(ws), _stream_ptr(stream)), "compress_bc1_mips")
    return (out, errors, off) if with_errors else (out, off)


def write_ktx(path: str, width: int, height: int, blocks) -> None:
    """KTX 1.1 file (GL_COMPRESSED_RGB_S3TC_DXT1_EXT) of host or device blocks."""
    b = blocks if hasattr(blocks, "data_ptr") else np.ascontiguousarray(blocks, np.uint8)
    _check(load().icbc_gpu_write_ktx(os.fsencode(path), int(width), int(height), _blocks_ptr(b)), "write_ktx")


def compare_dds(path: str, width: int, height: int, blocks) -> bool:
    """Golden-file check: True when the DDS file holds exactly these blocks."""
    b = blocks if hasattr(blocks, "data_ptr") else np.ascontiguousarray(blocks, np.uint8)
    r = load().icbc_gpu_compare_dds(os.fsencode(path), int(width), int(height), _blocks_ptr(b))
    if r < 0:
        raise IcbcGpuError(-r, "compare_dds")
    return r == 1


class Server:
    """The serving form (icbc_gpu_server_*): submit host RGBA8 images as they
    arrive; they are admitted under the HBM budget and batched onto the GPU.
    Host arrays are kept alive here until their request finishes."""

    def __init__(self, hbm_budget_bytes: int, max_inflight: int = 2, max_batch_images: int = 512):
        L = load()
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_inflight), int(max_batch_images))
        h = ctypes.c_void_p()
        _check(L.icbc_gpu_server_create(ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self._h = h
        self._keep = {}

    def submit(self, rgba: np.ndarray, level: int, decoder: int = Decoder_D3D10, color_weights=(1.0, 1.0, 1.0),
               weight_mode: int = WEIGHTS_UNIFORM, three_color_mode: bool = True, three_color_black: bool = True,
               out: np.ndarray | None = None, errors: np.ndarray | None = None) -> int:
        """Queues one image; returns the request id.  Raises IcbcGpuError
        (status ICBC_GPU_ERR_BUDGET etc.) when the request is refused."""
        h, w = int(rgba.shape[0]), int(rgba.shape[1])
        if out is None:
            out = np.zeros((blocks_of(w, h), 8), np.uint8)
        r = RequestDesc()
        r.rgba = rgba.ctypes.data
        r.width, r.height, r.pitch = w, h, int(rgba.strides[0])
        r.weight_mode, r.level, r.decoder = int(weight_mode), int(level), int(decoder)
        r.three_color_mode, r.three_color_black = int(bool(three_color_mode)), int(bool(three_color_black))
        r.color_weights = (ctypes.c_float * 3)(*[float(x) for x in color_weights])
        r.out = out.ctypes.data
        r.errors = errors.ctypes.data if errors is not None else None
        rid = ctypes.c_uint64()
        _check(load().icbc_gpu_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)), "server_submit")
        self._keep[rid.value] = (rgba, out, errors)
        return rid.value

    def result(self, rid: int):
        """(blocks, errors) of a finished request."""
        return self._keep[rid][1], self._keep[rid][2]

    def poll(self, rid: int) -> int:
        return load().icbc_gpu_server_poll(self._h, int(rid))

    def wait(self, rid: int, timeout_ms: int = -1) -> int:
        return load().icbc_gpu_server_wait(self._h, int(rid), int(timeout_ms))

    def cancel(self, rid: int) -> int:
        return load().icbc_gpu_server_cancel(self._h, int(rid))

    def stats(self) -> dict:
        st = ServerStats()
        _check(load().icbc_gpu_server_get_stats(self._h, ctypes.byref(st)), "server_get_stats")
        return st.as_dict()

    def close(self):
        if self._h:
            load().icbc_gpu_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- autotuner

# Launch shapes the autotuner tries: (groups_per_warp, persistent) for the
# kernels that take one block per lane (levels 0-1, the first pass of levels
# 2-9), and the CTA size of the pass that encodes the listed blocks of
# levels 2-9 (4: warp-wide searches; 8, 16: CTA-wide).
TUNE_CANDIDATES = [(g, p) for p in (0, 1) for g in (1, 2, 4, 8)]
TUNE_CTA_WARPS = (4, 8, 16)


def get_launch_config(level: int) -> tuple[int, int, int]:
    """(groups_per_warp, persistent, cta_warps) of a level (cta_warps 0: the level's default)."""
    c = LaunchConfig()
    _check(load().icbc_gpu_get_launch_config(int(level), ctypes.byref(c)), "get_launch_config")
    return c.groups_per_warp, c.persistent, c.cta_warps


def set_launch_config(level: int, groups_per_warp: int, persistent: int, cta_warps: int | None = None) -> None:
    """Sets a level's launch shape; cta_warps None keeps the current one (the
    batched form's CTA size is kept either way)."""
    c = LaunchConfig()
    _check(load().icbc_gpu_get_launch_config(int(level), ctypes.byref(c)), "get_launch_config")
    c.groups_per_warp, c.persistent = int(groups_per_warp), int(persistent)
    if cta_warps is not None:
        c.cta_warps = int(cta_warps)
    _check(load().icbc_gpu_set_launch_config(int(level), ctypes.byref(c)), "set_launch_config")


def get_batch_cta_warps(level: int) -> int:
    """The batched form's CTA size at a level (0: the default, 4)."""
    c = LaunchConfig()
    _check(load().icbc_gpu_get_launch_config(int(level), ctypes.byref(c)), "get_launch_config")
    return c.batch_cta_warps


def set_batch_cta_warps(level: int, cta_warps: int) -> None:
    """Sets the batched form's CTA size at a level (read when a batch is created)."""
    c = LaunchConfig()
    _check(load().icbc_gpu_get_launch_config(int(level), ctypes.byref(c)), "get_launch_config")
    c.batch_cta_warps = int(cta_warps)
    _check(load().icbc_gpu_set_launch_config(int(level), ctypes.byref(c)), "set_launch_config")


def autotune_batch(descs: Sequence[ImageDesc], candidates=TUNE_CTA_WARPS, repeats: int = 3, stream=None,
                   apply: bool = True) -> dict:
    """Times the batched form of `descs` (the same batch planned once per
    candidate) with each CTA size for the per-level kernels of levels 2-9,
    keeps the fastest (applied when `apply`) and returns {"batch_cta_warps",
    "ms", "candidates": {cta: ms}}.  The images' outputs are overwritten."""
    torch = _torch()
    before = {lv: get_batch_cta_warps(lv) for lv in range(2, 10)}
    times = {}
    for c in candidates:
        for lv in range(2, 10):
            set_batch_cta_warps(lv, c)
        b = Batch(descs)
        b.launch(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s = stream if stream is not None else torch.cuda.current_stream()
        e0.record(s)
        for _ in range(repeats):
            b.launch(stream)
        e1.record(s)
        torch.cuda.synchronize()
        b.close()
        times[c] = e0.elapsed_time(e1) / repeats
    best = min(times, key=times.get)
    for lv in range(2, 10):
        set_batch_cta_warps(lv, best if apply else before[lv])
    return {"batch_cta_warps": best, "ms": times[best], "candidates": times}


def autotune(image, levels=range(10), candidates=TUNE_CANDIDATES, cta_candidates=TUNE_CTA_WARPS, repeats: int = 3,
             decoder: int = Decoder_D3D10, color_weights=(1.0, 1.0, 1.0), weight_mode: int = WEIGHTS_UNIFORM,
             apply: bool = True, path: str | None = None) -> dict:
    """Times launch shapes of the plain image kernels on `image` (a CUDA
    uint8 tensor (h, w, 4)) for each level with CUDA events and keeps the
    fastest (applied to the library when `apply`): first (groups_per_warp,
    persistent) over `candidates`, then, at levels 2-9, the listed pass's CTA
    size over `cta_candidates`.  Returns {level: {"groups_per_warp",
    "persistent", "cta_warps", "ms", "candidates": {...}}}.  With `path` the
    table is also written as JSON (load_tuning reads it)."""
    import json
    torch = _torch()
    nb = blocks_of(int(image.shape[1]), int(image.shape[0]))
    stream = torch.cuda.Stream(device=image.device)
    stream.wait_stream(torch.cuda.current_stream())  # the image is ready
    with torch.cuda.stream(stream):
        out = torch.zeros((nb, 8), dtype=torch.uint8, device=image.device)

    def timed():
        with torch.cuda.stream(stream):
            compress_image(image, lv, decoder, color_weights, weight_mode, out=out, stream=stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(repeats):
                compress_image(image, lv, decoder, color_weights, weight_mode, out=out, stream=stream)
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / repeats

    table = {}
    for lv in levels:
        before = get_launch_config(lv)
        times = {}
        for g, p in candidates:
            set_launch_config(lv, g, p, before[2])
            times["%d/%d" % (g, p)] = timed()
        best = min(times, key=times.get)
        g, p = (int(x) for x in best.split("/"))
        cta = before[2]
        if lv >= 2 and cta_candidates:
            ctimes = {}
            for c in cta_candidates:
                set_launch_config(lv, g, p, c)
                ctimes[c] = timed()
                times["%d/%d/cta%d" % (g, p, c)] = ctimes[c]
            cta = min(ctimes, key=ctimes.get)
            best = "%d/%d/cta%d" % (g, p, cta)
        set_launch_config(lv, *((g, p, cta) if apply else before))
        table[int(lv)] = {"groups_per_warp": g, "persistent": p, "cta_warps": cta, "ms": times[best],
                          "candidates": times}
    if path:
        with open(path, "w") as f:
            json.dump({str(k): v for k, v in table.items()}, f, indent=1)
    return table


def load_tuning(path: str) -> None:
    """Applies a table written by autotune(path=...)."""
    import json
    with open(path) as f:
        table = json.load(f)
    for lv, cfg in table.items():
        set_launch_config(int(lv), cfg["groups_per_warp"], cfg["persistent"], cfg.get("cta_warps", 0))
