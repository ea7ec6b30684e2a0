"""Seeded synthetic RGBA8 workloads for the BC1 encoder.

The reference measures on the Kodak set, which is not shipped with it; these
generators stand in for it with the shapes and value distributions of the
benchmark configurations:

* ``gradient_noise_rects`` -- smooth bilinear gradients + 4-octave value noise
  (amplitude 0.3) + 20 hard-edged rectangles of uniform colour, clamped.
* ``quality_sweep_image`` -- the same at 4096x4096, plus 5% single-colour
  blocks, 5% near-black blocks (0..12) and alpha from a second noise field
  (weights = alpha / 255).
* ``batch_specs`` -- 2,000 images, sides log-uniform in 64..2048 (multiples
  of 4, 10% not), random level 0..9 and decoder D3D10/NVIDIA/AMD.
* ``serving_requests`` -- Poisson arrivals with the side/level mixture of the
  serving workload.
* ``hard_mixture_image`` -- per-block mixture of noise, two-colour dither,
  single colour, near-black and gradient+noise blocks, 25% zero-weight texels.

Every random number comes from a splitmix64 hash of (seed, stream, index) and
every float step is an elementwise IEEE operation, so the images are the
same bytes on every platform and numpy version.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def hash_u64(seed: int, stream: int, index) -> np.ndarray:
    idx = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = _mix(np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * np.uint64(0x100000001B3) + np.uint64(stream))
        return _mix(idx ^ key)


def uniform(seed: int, stream: int, shape) -> np.ndarray:
    """Uniform float64 in [0, 1) of the given shape."""
    n = int(np.prod(shape)) if shape else 1
    h = hash_u64(seed, stream, np.arange(n, dtype=np.uint64))
    return ((h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)).reshape(shape)


def randint(seed: int, stream: int, shape, lo: int, hi: int) -> np.ndarray:
    """Integers in [lo, hi)."""
    return (lo + np.floor(uniform(seed, stream, shape) * (hi - lo))).astype(np.int64)


def _smooth(t):
    return t * t * (3.0 - 2.0 * t)


def value_noise(w: int, h: int, seed: int, stream: int, octaves: int = 4, base_cells: int | None = None) -> np.ndarray:
    """Sum of value-noise octaves in [0, 1) as (h, w) float64.  Octave k has
    base_cells * 2^k lattice cells across the larger side (default: the finest
    octave has cells of about 2 pixels) and amplitude 2^-k; the sum is
    normalised.  Interpolation is smoothstep-bilinear, done separably."""
    side = max(w, h)
    if base_cells is None:
        base_cells = max(2, side // (2 << octaves))
    out = np.zeros((h, w), np.float64)
    total = 0.0
    for k in range(octaves):
        cells = base_cells << k
        amp = 1.0 / (1 << k)
        lat = uniform(seed, stream * 16 + k, (cells + 1, cells + 1))
        fy = (np.arange(h, dtype=np.float64) + 0.5) * (cells / side)
        fx = (np.arange(w, dtype=np.float64) + 0.5) * (cells / side)
        iy = np.minimum(fy.astype(np.int64), cells - 1)
        ix = np.minimum(fx.astype(np.int64), cells - 1)
        ty, tx = _smooth(fy - iy), _smooth(fx - ix)
        rows = lat[:, ix] + (lat[:, ix + 1] - lat[:, ix]) * tx[None, :]      # (cells+1, w)
        top, bot = rows[iy], rows[iy + 1]                                      # (h, w)
        out += amp * (top + (bot - top) * ty[:, None])
        total += amp
    return out / total


def gradient_noise_rects(w: int, h: int, seed: int, rects: int = 20, noise_amp: float = 0.3) -> np.ndarray:
    """(h, w, 4) uint8: bilinear gradients + value noise + hard rectangles, alpha 255."""
    img = np.zeros((h, w, 4), np.uint8)
    v = (np.arange(h, dtype=np.float64) / max(h - 1, 1))[:, None]
    u = (np.arange(w, dtype=np.float64) / max(w - 1, 1))[None, :]
    corners = uniform(seed, 1, (2, 4, 3))  # two bilinear gradients, four corner colours each
    for c in range(3):
        acc = np.zeros((h, w), np.float64)
        for g in range(2):
            c00, c10, c01, c11 = corners[g, :, c]
            acc += 0.5 * ((c00 * (1 - u) + c10 * u) * (1 - v) + (c01 * (1 - u) + c11 * u) * v)
        n = value_noise(w, h, seed, 2 + c)
        val = (acc + noise_amp * (n - 0.5)) * 255.0
        img[:, :, c] = np.clip(np.floor(val + 0.5), 0, 255).astype(np.uint8)
    img[:, :, 3] = 255
    r = uniform(seed, 7, (rects, 7))
    for k in range(rects):
        x0, y0 = int(r[k, 0] * w), int(r[k, 1] * h)
        rw, rh = 1 + int(r[k, 2] * w / 4), 1 + int(r[k, 3] * h / 4)
        col = np.floor(r[k, 4:7] * 256).clip(0, 255).astype(np.uint8)
        img[y0:y0 + rh, x0:x0 + rw, :3] = col
    return img


def quality_sweep_image(w: int = 4096, h: int = 4096, seed: int = 1) -> np.ndarray:
    """The quality-sweep image: gradient/noise/rects, 5% single-colour blocks,
    5% near-black blocks (0..12), alpha = a second value-noise field."""
    img = gradient_noise_rects(w, h, seed)
    bw, bh = w // 4, h // 4
    kind = uniform(seed, 20, (bh, bw))
    view = img[: bh * 4, : bw * 4, :3].reshape(bh, 4, bw, 4, 3)
    by, bx = np.nonzero(kind < 0.05)
    fc = np.floor(uniform(seed, 21, (len(by), 3)) * 256).clip(0, 255).astype(np.uint8)
    view[by, :, bx, :, :] = fc[:, None, None, :]
    by, bx = np.nonzero((kind >= 0.05) & (kind < 0.10))
    view[by, :, bx, :, :] = randint(seed, 22, (len(by), 4, 4, 3), 0, 13).astype(np.uint8)
    alpha = value_noise(w, h, seed, 30)
    img[:, :, 3] = np.clip(np.floor(alpha * 255.0 + 0.5), 0, 255).astype(np.uint8)
    return img


def hard_mixture_image(w: int, h: int, seed: int) -> np.ndarray:
    """(h, w, 4) uint8 of independent 4x4 blocks: 30% i.i.d. noise, 20% two-colour
    dither, 15% single colour, 15% near-black (some texels 0..8), 20% gradient
    + value noise.  Alpha is 0 on 25% of texels (zero weight), else 255."""
    bw, bh = (w + 3) // 4, (h + 3) // 4
    kind = uniform(seed, 40, (bh, bw))
    out = np.zeros((bh, 4, bw, 4, 4), np.uint8)
    noise = randint(seed, 41, (bh, 4, bw, 4, 3), 0, 256)
    ca = randint(seed, 42, (bh, 1, bw, 1, 3), 0, 256)
    cb = randint(seed, 43, (bh, 1, bw, 1, 3), 0, 256)
    pick = uniform(seed, 44, (bh, 4, bw, 4, 1)) < 0.5
    dither = np.where(pick, ca, cb)
    single = np.broadcast_to(ca, (bh, 4, bw, 4, 3))
    dark = np.where(uniform(seed, 45, (bh, 4, bw, 4, 1)) < 0.5, randint(seed, 46, (bh, 4, bw, 4, 3), 0, 9),
                    randint(seed, 47, (bh, 4, bw, 4, 3), 0, 32))
    g = (np.arange(4, dtype=np.float64) / 3.0)
    gx = g[None, None, None, :, None]
    gy = g[None, :, None, None, None]
    tgt = cb.astype(np.float64)
    grad = ca + (tgt - ca) * (0.5 * gx + 0.5 * gy) + 24.0 * (uniform(seed, 48, (bh, 4, bw, 4, 3)) - 0.5)
    grad = np.clip(np.floor(grad + 0.5), 0, 255).astype(np.int64)
    k = kind[:, None, :, None, None]
    rgb = np.where(k < 0.30, noise,
          np.where(k < 0.50, dither,
          np.where(k < 0.65, single,
          np.where(k < 0.80, dark, grad))))
    out[..., :3] = rgb.astype(np.uint8)
    out[..., 3] = np.where(uniform(seed, 49, (bh, 4, bw, 4)) < 0.25, 0, 255).astype(np.uint8)
    img = out.reshape(bh * 4, bw * 4, 4)
    return np.ascontiguousarray(img[:h, :w])


@dataclass
class ImageSpec:
    width: int
    height: int
    level: int
    decoder: int
    seed: int


def extreme_weight_blocks(n: int, seed: int, levels: int = 8) -> tuple[np.ndarray, np.ndarray]:
    """Blocks of dark colours (channels 0..levels-1) with per-texel weights
    spread log-uniformly over 1e-30 .. 1e30: the weighted sums overflow and
    degenerate cluster splits divide zero by zero, the inputs where the
    reference's NEON build (whose vsaturate keeps a NaN) and its x86 builds
    part ways.  Returns compress_bc1 inputs (n,16,4) and (n,16)."""
    tex = randint(seed, 90, (n, 16, 3), 0, levels)
    lut = (np.arange(256, dtype=np.float32) / np.float32(255.0)).astype(np.float32)
    cols = np.ones((n, 16, 4), np.float32)
    cols[:, :, :3] = lut[tex]
    w = (10.0 ** (uniform(seed, 91, (n, 16)) * 60.0 - 30.0)).astype(np.float32)
    return cols, w


def batch_specs(n: int = 2000, seed: int = 7, lo: int = 64, hi: int = 2048) -> list[ImageSpec]:
    """Sizes log-uniform in [lo, hi] per side, rounded to multiples of 4 except
    10% left as is; level uniform 0..9; decoder uniform over D3D10/NVIDIA/AMD."""
    r = uniform(seed, 60, (n, 6))
    specs = []
    span = math.log(hi / lo)
    for i in range(n):
        sides = []
        for j in range(2):
            s = lo * math.exp(r[i, j] * span)
            s = int(min(hi, max(lo, round(s))))
            if r[i, 2] >= 0.10:
                s = max(lo, (s // 4) * 4)
            sides.append(s)
        specs.append(ImageSpec(sides[0], sides[1], int(r[i, 3] * 10), int(r[i, 4] * 3), seed * 100003 + i))
    return specs


SERVING_SIDES = (64, 128, 256, 512, 1024, 2048)
SERVING_PROBS = (0.30, 0.25, 0.20, 0.15, 0.07, 0.03)


@dataclass
class Request:
    arrival_s: float
    side: int
    level: int
    seed: int


def serving_requests(n: int, rate_per_s: float, seed: int = 11) -> list[Request]:
    """Poisson arrivals at rate_per_s; side from SERVING_SIDES with
    SERVING_PROBS, level uniform 0..9."""
    r = uniform(seed, 70, (n, 3))
    cum = np.cumsum(SERVING_PROBS)
    t = 0.0
    out = []
    for i in range(n):
        t += -math.log(1.0 - r[i, 0]) / rate_per_s
        side = SERVING_SIDES[int(np.searchsorted(cum, r[i, 1], side="right"))] if r[i, 1] < cum[-1] else SERVING_SIDES[-1]
        out.append(Request(t, side, int(r[i, 2] * 10), seed * 1000003 + i))
    return out


def mixed_blocks(n: int, seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """n blocks in compress_bc1 form from the hard mixture (colors (n,16,4),
    weights (n,16) = alpha/255 with 25% zeros)."""
    side = int(math.ceil(math.sqrt(n))) * 4
    img = hard_mixture_image(side, side, seed)
    tex = img.reshape(side // 4, 4, side // 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)[:n]
    lut = (np.arange(256, dtype=np.float32) / np.float32(255.0)).astype(np.float32)
    colors = lut[tex].astype(np.float32)
    colors[:, :, 3] = 1.0
    return np.ascontiguousarray(colors), np.ascontiguousarray(lut[tex[:, :, 3]])


def hard_mixture_torch(w: int, h: int, seed: int, device="cuda"):
    """The hard block mixture of ``hard_mixture_image`` generated on the GPU
    with torch's seeded generator (for the 64 x 8192^2 workload, where host
    generation would dominate).  Same mixture and weights; different random
    stream, so compare results only against the same tensor's contents.
    w and h must be multiples of 4."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    bw, bh = w // 4, h // 4

    def rnd(*shape):
        return torch.rand(shape, generator=g, device=device)

    def rint(lo, hi, *shape):
        return torch.randint(lo, hi, shape, generator=g, device=device, dtype=torch.int16)

    kind = rnd(bh, 1, bw, 1, 1)
    ca, cb = rint(0, 256, bh, 1, bw, 1, 3), rint(0, 256, bh, 1, bw, 1, 3)
    out = rint(0, 256, bh, 4, bw, 4, 3)                                       # i.i.d. noise
    dither = torch.where(rnd(bh, 4, bw, 4, 1) < 0.5, ca, cb)
    out = torch.where((kind >= 0.30) & (kind < 0.50), dither, out)
    del dither
    out = torch.where((kind >= 0.50) & (kind < 0.65), ca.expand(bh, 4, bw, 4, 3), out)
    dark = torch.where(rnd(bh, 4, bw, 4, 1) < 0.5, rint(0, 9, bh, 4, bw, 4, 3), rint(0, 32, bh, 4, bw, 4, 3))
    out = torch.where((kind >= 0.65) & (kind < 0.80), dark, out)
    del dark
    gr = torch.arange(4, device=device, dtype=torch.float32) / 3.0
    t = 0.5 * gr.view(1, 1, 1, 4, 1) + 0.5 * gr.view(1, 4, 1, 1, 1)
    grad = ca.float() + (cb.float() - ca.float()) * t + 24.0 * (rnd(bh, 4, bw, 4, 3) - 0.5)
    grad = torch.floor(grad + 0.5).clamp(0, 255).to(torch.int16)
    out = torch.where(kind >= 0.80, grad, out)
    del grad
    alpha = torch.where(rnd(bh, 4, bw, 4, 1) < 0.25, 0, 255).to(torch.int16)
    img = torch.cat([out, alpha], dim=-1).to(torch.uint8)
    return img.reshape(bh * 4, bw * 4, 4).contiguous()
