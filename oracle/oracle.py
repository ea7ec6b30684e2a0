"""ctypes access to the CPU oracle and to the compiled reference.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, as the checker -- never by the product
package ``icbc_gb300``.

* ``liboracle.so`` is the C restatement in ``icbc_oracle.c`` (built here with
  gcc, on any host).
* ``_ref/libicbc_ref.so`` is the reference's own icbc.h in its scalar profile,
  built by ``build_ref.sh`` only where the reference checkout exists;
  ``_ref/libicbc_ref_simd<N>.so`` are its x86 SIMD builds (N = ICBC_SIMD 1..5).

SIMD profiles: every ``decoder`` below may be combined with ``profile``
(0 scalar, 1 SSE2, 2 SSE4.1, 3 AVX, 4 AVX2, 5 AVX-512, 6 NEON); the oracle
then reproduces that build's cluster-fit loops.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libicbc_ref.so")

_lock = threading.Lock()
_lib = None
_ref = {}

PROFILE_SHIFT = 8
PROFILES = {"scalar": 0, "sse2": 1, "sse41": 2, "avx": 3, "avx2": 4, "avx512": 5, "neon": 6}
# ORACLE_VECTOR_LOOPS: the cluster loops of a 4-lane profile as 4-lane vector
# code (same results; a vectorised CPU encoder to time).
VECTOR_LOOPS = 1 << 11


def _decoder_word(decoder, profile, vector):
    return int(decoder) | (int(profile) << PROFILE_SHIFT) | (VECTOR_LOOPS if vector else 0)


def ref_path(profile: int = 0) -> str:
    return REF_PATH if profile == 0 else os.path.join(HERE, "_ref", "libicbc_ref_simd%d.so" % profile)

CFLAGS = ["-O2", "-std=c99", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "blocks", "zero_blocks", "single_blocks", "reduce_pairs", "reduce_merges",
        "sat_builds", "sat_points", "cf4_combos", "cf3_combos", "out4_blocks",
        "out3_blocks", "box_fits", "box_points", "lsq_fits", "refine_steps")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


def build(force: bool = False) -> str:
    """Compiles icbc_oracle.c into liboracle.so (when stale or missing)."""
    src = os.path.join(HERE, "icbc_oracle.c")
    hdr = os.path.join(HERE, "icbc_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    tmp = LIB_PATH + ".%d.tmp" % os.getpid()
    cmd = [os.environ.get("CC", "gcc")] + CFLAGS + [src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_dir() -> str | None:
    """Where build_ref.sh finds the reference checkout (it holds the default;
    ICBC_REFERENCE_DIR overrides it), or None where there is none."""
    r = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True, text=True)
    path = r.stdout.strip()
    return path if r.returncode == 0 and path and os.path.exists(os.path.join(path, "icbc.h")) else None


def build_ref() -> str | None:
    """Builds oracle/_ref/libicbc_ref.so when the reference checkout exists."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.run(["sh", script], check=True, stdout=subprocess.DEVNULL)
    return REF_PATH if os.path.exists(REF_PATH) else None


def _P(dtype):
    return np.ctypeslib.ndpointer(dtype=dtype, flags="C_CONTIGUOUS")


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            f32p = ctypes.POINTER(ctypes.c_float)
            L.oracle_init.restype = None
            L.oracle_compress_bc1.restype = ctypes.c_float
            L.oracle_compress_bc1.argtypes = [ctypes.c_int, ctypes.c_int, f32p, f32p, f32p,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.POINTER(Stats)]
            L.oracle_compress_blocks.restype = ctypes.c_int
            L.oracle_compress_blocks.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                 f32p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                                 ctypes.POINTER(Stats)]
            L.oracle_encode_image.restype = ctypes.c_int
            L.oracle_encode_image.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                              ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              f32p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Stats)]
            L.oracle_decode_bc1.restype = None
            L.oracle_decode_bc1.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            L.oracle_evaluate_bc1_error.restype = ctypes.c_float
            L.oracle_evaluate_bc1_error.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            L.oracle_decode_bc3.restype = None
            L.oracle_decode_bc3.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            L.oracle_evaluate_bc3_error.restype = ctypes.c_float
            L.oracle_evaluate_bc3_error.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
            L.oracle_image_sse.restype = ctypes.c_double
            L.oracle_image_sse.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                           ctypes.c_void_p, ctypes.c_int]
            L.oracle_tables.restype = None
            L.oracle_tables.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            L.oracle_cluster_tables.restype = ctypes.c_int
            L.oracle_cluster_tables.argtypes = [ctypes.c_void_p] * 4
            L.oracle_init()
            _lib = L
    return _lib


def ref(profile: int = 0):
    """The compiled reference (scalar build, or the x86 SIMD build `profile`),
    or None where it cannot be built."""
    with _lock:
        if profile not in _ref:
            path = ref_path(profile)
            if not os.path.exists(path):
                try:
                    build_ref()
                except Exception:
                    return None
            if not os.path.exists(path):
                return None
            R = ctypes.CDLL(path)
            R.ref_init.restype = None
            R.ref_init.argtypes = [ctypes.c_int]
            R.ref_compress_blocks.restype = None
            R.ref_compress_blocks.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int64]
            R.ref_decode_bc1.restype = None
            R.ref_decode_bc1.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            R.ref_evaluate_bc1_error.restype = ctypes.c_float
            R.ref_evaluate_bc1_error.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            if profile == 0:
                R.ref_decode_bc3.restype = None
                R.ref_decode_bc3.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
                R.ref_evaluate_bc3_error.restype = ctypes.c_float
                R.ref_evaluate_bc3_error.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
            _ref[profile] = R
    return _ref[profile]


def _aligned_f32(a, align: int = 64):
    """A float32 copy of `a` whose data starts on an `align`-byte boundary
    (the SIMD builds load input colours with aligned vector loads)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    buf = np.empty(a.size + align // 4, np.float32)
    off = (-buf.ctypes.data % align) // 4
    out = buf[off:off + a.size].reshape(a.shape)
    out[...] = a
    return out


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _cw(color_weights):
    cw = _f32(color_weights).reshape(3)
    return cw, cw.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def compress_blocks(colors, weights, level, decoder=0, color_weights=(1, 1, 1), three_color_mode=True,
                    three_color_black=True, nthreads=1, out=None, with_stats=False, profile=0, vector=False):
    """Oracle encode of n blocks.  colors: (n,16,4) float32; weights: (n,16) or None.
    Returns (blocks uint8 (n,8), errors float32 (n,)[, stats dict]).  vector:
    run a 4-lane profile's cluster loops as vector code."""
    L = lib()
    colors = _f32(colors).reshape(-1, 64)
    n = colors.shape[0]
    w = None if weights is None else _f32(weights).reshape(n, 16)
    out = np.zeros((n, 8), np.uint8) if out is None else np.ascontiguousarray(out, dtype=np.uint8).copy()
    err = np.zeros(n, np.float32)
    cw, cwp = _cw(color_weights)
    st = Stats()
    L.oracle_compress_blocks(_decoder_word(decoder, profile, vector), int(level), colors.ctypes.data,
                             None if w is None else w.ctypes.data,
                             cwp, int(bool(three_color_mode)), int(bool(three_color_black)), out.ctypes.data,
                             err.ctypes.data, n, int(nthreads), ctypes.byref(st))
    return (out, err, st.as_dict()) if with_stats else (out, err)


def encode_image(rgba, level, decoder=0, color_weights=(1, 1, 1), weight_mode=0, weight_plane=None,
                 three_color_mode=True, three_color_black=True, nthreads=1, with_stats=False, profile=0,
                 vector=False):
    """Oracle encode of an RGBA8 image (h, w, 4) uint8 -> (blocks (nb,8), errors (nb,)).
    vector: run a 4-lane profile's cluster loops as vector code."""
    L = lib()
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    nb = ((w + 3) // 4) * ((h + 3) // 4)
    out = np.zeros((nb, 8), np.uint8)
    err = np.zeros(nb, np.float32)
    cw, cwp = _cw(color_weights)
    plane = None if weight_plane is None else _f32(weight_plane).reshape(h, w)
    st = Stats()
    L.oracle_encode_image(rgba.ctypes.data, w, h, w * 4, int(weight_mode),
                          None if plane is None else plane.ctypes.data, _decoder_word(decoder, profile, vector),
                          int(level), cwp,
                          int(bool(three_color_mode)), int(bool(three_color_black)), out.ctypes.data,
                          err.ctypes.data, int(nthreads), ctypes.byref(st))
    return (out, err, st.as_dict()) if with_stats else (out, err)


def image_blocks(rgba, weight_mode=0, weight_plane=None):
    """Edge-replicated block gather of an image into the float form compress_bc1
    takes: colors (nb,16,4) = u8/255.0f with alpha 1.0f, weights (nb,16)."""
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    bw, bh = (w + 3) // 4, (h + 3) // 4
    ys = np.minimum(np.arange(bh * 4), h - 1)
    xs = np.minimum(np.arange(bw * 4), w - 1)
    pad = rgba[ys][:, xs]                                         # (bh*4, bw*4, 4)
    tex = pad.reshape(bh, 4, bw, 4, 4).transpose(0, 2, 1, 3, 4).reshape(bh * bw, 16, 4)
    lut = (np.arange(256, dtype=np.float32) / np.float32(255.0)).astype(np.float32)
    colors = lut[tex].astype(np.float32)
    colors[:, :, 3] = 1.0
    if weight_mode == 1:
        weights = lut[tex[:, :, 3]]
    elif weight_mode == 2:
        pl = np.asarray(weight_plane, np.float32)[ys][:, xs]
        weights = pl.reshape(bh, 4, bw, 4).transpose(0, 2, 1, 3).reshape(bh * bw, 16)
    else:
        weights = np.ones((bh * bw, 16), np.float32)
    return np.ascontiguousarray(colors), np.ascontiguousarray(weights, dtype=np.float32), tex


def decode_bc1(blocks, decoder=0):
    L = lib()
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 8)
    out = np.zeros((b.shape[0], 64), np.uint8)
    for i in range(b.shape[0]):
        L.oracle_decode_bc1(b[i].ctypes.data, out[i].ctypes.data, int(decoder))
    return out


def evaluate_bc1_error(rgba_blocks, blocks, decoder=0):
    L = lib()
    t = np.ascontiguousarray(rgba_blocks, dtype=np.uint8).reshape(-1, 64)
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 8)
    return np.array([L.oracle_evaluate_bc1_error(t[i].ctypes.data, b[i].ctypes.data, int(decoder))
                     for i in range(b.shape[0])], np.float32)


def decode_bc3(blocks, decoder=0):
    """icbc::decode_bc3 of 16-byte blocks -> (n, 64) RGBA8."""
    L = lib()
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 16)
    out = np.zeros((b.shape[0], 64), np.uint8)
    for i in range(b.shape[0]):
        L.oracle_decode_bc3(b[i].ctypes.data, out[i].ctypes.data, int(decoder))
    return out


def evaluate_bc3_error(rgba_blocks, blocks, alpha_blend, decoder=0):
    L = lib()
    t = np.ascontiguousarray(rgba_blocks, dtype=np.uint8).reshape(-1, 64)
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 16)
    return np.array([L.oracle_evaluate_bc3_error(t[i].ctypes.data, b[i].ctypes.data, int(bool(alpha_blend)),
                                                 int(decoder)) for i in range(b.shape[0])], np.float32)


def image_sse(rgba, blocks, decoder=0):
    L = lib()
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    b = np.ascontiguousarray(blocks, dtype=np.uint8)
    return float(L.oracle_image_sse(rgba.ctypes.data, w, h, w * 4, b.ctypes.data, int(decoder)))


def tables(decoder):
    L = lib()
    m5 = np.zeros(512, np.uint8)
    m6 = np.zeros(512, np.uint8)
    w = np.zeros(5, np.float32)
    L.oracle_tables(int(decoder), m5.ctypes.data, m6.ctypes.data, w.ctypes.data)
    return m5, m6, w


def cluster_tables():
    L = lib()
    four = np.zeros(968, np.uint32)
    ft = np.zeros(16, np.int32)
    three = np.zeros(152, np.uint32)
    tt = np.zeros(16, np.int32)
    L.oracle_cluster_tables(four.ctypes.data, ft.ctypes.data, three.ctypes.data, tt.ctypes.data)
    return four, ft, three, tt


def ref_compress_blocks(colors, weights, level, decoder=0, color_weights=(1, 1, 1), three_color_mode=True,
                        three_color_black=True, out=None, profile=0):
    """The compiled reference (single thread) on the same inputs.  None if unavailable."""
    R = ref(profile)
    if R is None:
        return None
    colors = _aligned_f32(_f32(colors).reshape(-1, 64))
    n = colors.shape[0]
    w = np.ones((n, 16), np.float32) if weights is None else _f32(weights).reshape(n, 16)
    out = np.zeros((n, 8), np.uint8) if out is None else np.ascontiguousarray(out, dtype=np.uint8).copy()
    err = np.zeros(n, np.float32)
    cw = _f32(color_weights).reshape(3)
    with _lock:  # icbc::init mutates the reference's globals
        R.ref_init(int(decoder))
        R.ref_compress_blocks(int(level), colors.ctypes.data, w.ctypes.data, cw.ctypes.data,
                              int(bool(three_color_mode)), int(bool(three_color_black)), out.ctypes.data,
                              err.ctypes.data, n)
    return out, err


def ref_decode_bc1(blocks, decoder=0):
    R = ref()
    if R is None:
        return None
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 8)
    out = np.zeros((b.shape[0], 64), np.uint8)
    for i in range(b.shape[0]):
        R.ref_decode_bc1(b[i].ctypes.data, out[i].ctypes.data, int(decoder))
    return out


def ref_evaluate_bc1_error(rgba_blocks, blocks, decoder=0):
    R = ref()
    if R is None:
        return None
    t = np.ascontiguousarray(rgba_blocks, dtype=np.uint8).reshape(-1, 64)
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 8)
    return np.array([R.ref_evaluate_bc1_error(t[i].ctypes.data, b[i].ctypes.data, int(decoder))
                     for i in range(b.shape[0])], np.float32)


def ref_decode_bc3(blocks, decoder=0):
    R = ref()
    if R is None:
        return None
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 16)
    out = np.zeros((b.shape[0], 64), np.uint8)
    for i in range(b.shape[0]):
        R.ref_decode_bc3(b[i].ctypes.data, out[i].ctypes.data, int(decoder))
    return out


def ref_evaluate_bc3_error(rgba_blocks, blocks, alpha_blend, decoder=0):
    R = ref()
    if R is None:
        return None
    t = np.ascontiguousarray(rgba_blocks, dtype=np.uint8).reshape(-1, 64)
    b = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 16)
    return np.array([R.ref_evaluate_bc3_error(t[i].ctypes.data, b[i].ctypes.data, int(bool(alpha_blend)),
                                              int(decoder)) for i in range(b.shape[0])], np.float32)


def expand_rgba8(pixels):
    """stbi_load(..., 4) channel expansion (icbc_test.cpp:345) of an (h, w, c)
    or (h, w) uint8 array: grey -> (g, g, g, 255), grey + alpha -> (g, g, g, a),
    RGB -> (r, g, b, 255), RGBA unchanged."""
    p = np.asarray(pixels, np.uint8)
    if p.ndim == 2:
        p = p[:, :, None]
    h, w, c = p.shape
    out = np.empty((h, w, 4), np.uint8)
    if c in (1, 2):
        out[..., 0] = out[..., 1] = out[..., 2] = p[..., 0]
    else:
        out[..., :3] = p[..., :3]
    out[..., 3] = p[..., c - 1] if c in (2, 4) else 255
    return out


def mip_down(rgba):
    """One 2x2 box-filter mip step of an (h, w, 4) uint8 image: size
    max(1, w >> 1) x max(1, h >> 1), each channel (a + b + c + d + 2) >> 2 over
    texels (2x, 2y) .. (2x + 1, 2y + 1), coordinates clamped to the source."""
    src = np.asarray(rgba, np.uint8).astype(np.int32)
    h, w = src.shape[:2]
    dh, dw = max(1, h >> 1), max(1, w >> 1)
    xs0 = np.minimum(2 * np.arange(dw), w - 1)
    xs1 = np.minimum(2 * np.arange(dw) + 1, w - 1)
    ys0 = np.minimum(2 * np.arange(dh), h - 1)
    ys1 = np.minimum(2 * np.arange(dh) + 1, h - 1)
    s = (src[ys0][:, xs0] + src[ys0][:, xs1] + src[ys1][:, xs0] + src[ys1][:, xs1] + 2) >> 2
    return s.astype(np.uint8)


def mip_chain(rgba, levels=None):
    """[level 0, level 1, ...] down to 1 x 1 (or `levels` levels)."""
    out = [np.asarray(rgba, np.uint8)]
    while (levels is None or len(out) < levels) and (out[-1].shape[0] > 1 or out[-1].shape[1] > 1):
        out.append(mip_down(out[-1]))
    return out
