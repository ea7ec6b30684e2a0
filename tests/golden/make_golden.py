"""Generates the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own icbc.h, compiled unmodified in its scalar profile by
oracle/build_ref.sh (needs the reference checkout), on seeded inputs and
stores inputs and outputs:

  blocks.npz   mixed blocks (noise, dither, single colour, near black,
               gradients, exact and near duplicates, zero weights) and the
               reference's blocks + returned errors for every level 0..9 x
               decoder x (three_color_mode, three_color_black) x weight set
  image512.npz the 512x512 gradient/noise/rectangle image (seed 0) encoded at
               Quality_Default, D3D10, uniform weights, cw {1,1,1}, both
               three-colour flags on; plus the SHA-256 of the generated image
  decode.npz   decode_bc1 and evaluate_bc1_error of the reference for every
               decoder on encoded blocks, including 3-colour blocks
  bc3.npz      decode_bc3 and evaluate_bc3_error (alpha_blend off and on)
               of the reference for every decoder on 16-byte blocks whose
               colour halves are encoded blocks (both endpoint orders) and
               whose alpha halves are random bytes
  simd.npz     the reference's x86 SIMD builds (ICBC_SIMD 1..5, compiled
               without FP contraction by the same script) on two sets of 128
               image blocks -- the blocks of two 512x512 images where some
               SIMD build differs from the scalar one, topped up with the
               first others -- at levels 2, 4, 8, 9 x decoder x
               (three_color_mode, three_color_black) in {(1, 1), (0, 0)}

Usage: python tests/golden/make_golden.py [simd|bc3]   (only simd.npz / bc3.npz)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from icbc_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

FLAGS = ((1, 1), (1, 0), (0, 0))
CWS = ((1.0, 1.0, 1.0), (0.299, 0.587, 0.114))


def golden_blocks(n_mixed: int = 224) -> tuple[np.ndarray, np.ndarray]:
    """Mixed blocks plus hand-made edge cases, as compress_bc1 inputs."""
    cols, w = synth.mixed_blocks(n_mixed, seed=5)
    extra_c, extra_w = [], []
    lut = (np.arange(256, dtype=np.float32) / np.float32(255.0)).astype(np.float32)

    def add(tex, wt):
        c = np.ones((16, 4), np.float32)
        c[:, :3] = lut[np.asarray(tex, np.int64).reshape(16, 3)]
        extra_c.append(c)
        extra_w.append(np.asarray(wt, np.float32).reshape(16))

    r = synth.uniform(99, 0, (64, 16, 3))
    add(np.zeros((16, 3)), np.zeros(16))                        # every weight zero -> zero block
    add(np.full((16, 3), 200), np.ones(16))                     # single colour
    add(np.tile([[255, 255, 255]], (16, 1)), np.ones(16))       # white
    add(np.zeros((16, 3)), np.ones(16))                         # black
    add(np.tile([[10, 20, 30], [200, 100, 50]], (8, 1)), np.ones(16))          # two colours
    add(np.tile([[0, 0, 0], [0, 0, 0], [255, 255, 255], [8, 8, 8]], (4, 1)), np.ones(16))  # black + white
    add((r[0] * 256).astype(int).clip(0, 255), np.full(16, 1e-3))                 # tiny weights
    add((r[1] * 256).astype(int).clip(0, 255), np.where(np.arange(16) < 15, 0.0, 1.0))  # one live texel
    add(np.tile([[128, 128, 128]], (16, 1)) + (np.arange(16)[:, None] % 2), np.ones(16))  # near duplicates
    base = (r[2] * 200).astype(int)
    add(np.clip(base + (r[3] * 4).astype(int), 0, 255), np.ones(16))            # within-threshold jitter
    add(np.tile([[31, 0, 0]], (16, 1)) + np.arange(16)[:, None] * np.array([[14, 15, 16]]), np.ones(16))  # ramp
    for k in range(21):
        add((r[4 + k] * 256).astype(int).clip(0, 255), (r[30 + k, :, 0] * 2.0).astype(np.float32))
    return (np.concatenate([cols, np.stack(extra_c)]), np.concatenate([w, np.stack(extra_w)]))


SIMD_LEVELS = (2, 4, 8, 9)
SIMD_FLAGS = ((1, 1), (0, 0))


def simd_sets(per_set: int = 128):
    """Two block sets (colors, weights, cw) where the SIMD builds matter."""
    sets = []
    for img, wm, cw in ((synth.gradient_noise_rects(512, 512, 1), 0, (1.0, 1.0, 1.0)),
                        (synth.quality_sweep_image(512, 512, seed=4), 1, (0.299, 0.587, 0.114))):
        cols, w, _ = O.image_blocks(img, weight_mode=wm)
        differ = np.zeros(cols.shape[0], bool)
        for lvl in (4, 8):
            base, _ = O.compress_blocks(cols, w, lvl, 0, cw, True, True, nthreads=os.cpu_count() or 1)
            for prof in range(1, 6):
                b, _ = O.compress_blocks(cols, w, lvl, 0, cw, True, True, nthreads=os.cpu_count() or 1,
                                         profile=prof)
                differ |= (b != base).any(1)
        pick = list(np.flatnonzero(differ)[:per_set])
        pick += [i for i in range(cols.shape[0]) if not differ[i]][:per_set - len(pick)]
        pick = np.array(sorted(pick))
        wt = np.ones((len(pick), 16), np.float32) if w is None else w[pick]
        sets.append((np.ascontiguousarray(cols[pick]), np.ascontiguousarray(wt), cw))
    return sets


def golden_simd():
    out = {}
    for si, (cols, wt, cw) in enumerate(simd_sets()):
        out["set%d_colors" % si] = cols
        out["set%d_weights" % si] = wt
        out["set%d_cw" % si] = np.array(cw, np.float32)
        for prof in range(1, 6):
            if O.ref(prof) is None:
                raise SystemExit("the x86 SIMD builds of the reference are needed for simd.npz")
            for lvl in SIMD_LEVELS:
                for dec in range(4):
                    for tc, tcb in SIMD_FLAGS:
                        b, e = O.ref_compress_blocks(cols, wt, lvl, dec, cw, tc, tcb, profile=prof)
                        key = "set%d_P%d_L%d_D%d_tc%d_tcb%d" % (si, prof, lvl, dec, tc, tcb)
                        out[key + "_blocks"] = b
                        out[key + "_errors"] = e
    np.savez_compressed(os.path.join(HERE, "simd.npz"), **out)
    print("simd.npz", os.path.getsize(os.path.join(HERE, "simd.npz")))


def golden_bc3(blocks, rgba):
    """BC3 decode/evaluate of the reference on `blocks` (n, 8) colour halves
    with random alpha halves, against `rgba` (n, 64) with random alpha."""
    n = blocks.shape[0]
    r = synth.randint(77, 0, (n, 8), 0, 256).astype(np.uint8)
    bc3 = np.concatenate([r, blocks], axis=1)
    tex = rgba.copy().reshape(n, 16, 4)
    tex[:, :, 3] = synth.randint(77, 1, (n, 16), 0, 256).astype(np.uint8)
    tex = tex.reshape(n, 64)
    out = {"blocks": bc3, "rgba": tex}
    for d in range(4):
        out["decoded_D%d" % d] = O.ref_decode_bc3(bc3, d)
        for ab in (0, 1):
            out["error_D%d_blend%d" % (d, ab)] = O.ref_evaluate_bc3_error(tex, bc3, ab, d)
    np.savez_compressed(os.path.join(HERE, "bc3.npz"), **out)
    print("bc3.npz", os.path.getsize(os.path.join(HERE, "bc3.npz")))


def main():
    if O.ref() is None:
        raise SystemExit("the reference checkout is needed to generate golden vectors")
    if sys.argv[1:] == ["simd"]:
        golden_simd()
        return
    if sys.argv[1:] == ["bc3"]:
        g = np.load(os.path.join(HERE, "decode.npz"))
        golden_bc3(g["blocks"], g["rgba"])
        return
    colors, wr = golden_blocks()
    n = colors.shape[0]
    wu = np.ones((n, 16), np.float32)
    out = {"colors": colors, "weights_rand": wr}
    for lvl in range(10):
        for dec in range(4):
            for tc, tcb in FLAGS:
                for wn, wt in (("u", wu), ("r", wr)):
                    cw = CWS[(dec + (wn == "r")) % 2]
                    b, e = O.ref_compress_blocks(colors, wt, lvl, dec, cw, tc, tcb)
                    key = "L%d_D%d_tc%d_tcb%d_w%s" % (lvl, dec, tc, tcb, wn)
                    out[key + "_blocks"] = b
                    out[key + "_errors"] = e
    np.savez_compressed(os.path.join(HERE, "blocks.npz"), **out)

    img = synth.gradient_noise_rects(512, 512, 0)
    cols, w, _ = O.image_blocks(img)
    b, e = O.ref_compress_blocks(cols, w, 8, 0, (1, 1, 1), True, True)
    np.savez_compressed(os.path.join(HERE, "image512.npz"), blocks=b, errors=e,
                        sha256=np.frombuffer(hashlib.sha256(img.tobytes()).digest(), np.uint8))

    dec_out = {}
    tex = (colors[:, :, :3] * 255.0 + 0.5).astype(np.uint8)
    rgba = np.concatenate([tex, np.full((n, 16, 1), 255, np.uint8)], axis=2).reshape(n, 64)
    b4, _ = O.ref_compress_blocks(colors, wu, 8, 0, (1, 1, 1), True, True)
    bsw = b4.copy()
    bsw[:, [0, 1, 2, 3]] = b4[:, [2, 3, 0, 1]]  # swapped endpoints flip 4- and 3-colour modes
    blocks = np.concatenate([b4, bsw])
    rgba2 = np.concatenate([rgba, rgba])
    dec_out["blocks"] = blocks
    dec_out["rgba"] = rgba2
    for d in range(4):
        dec_out["decoded_D%d" % d] = O.ref_decode_bc1(blocks, d)
        dec_out["error_D%d" % d] = O.ref_evaluate_bc1_error(rgba2, blocks, d)
    np.savez_compressed(os.path.join(HERE, "decode.npz"), **dec_out)
    for f in ("blocks.npz", "image512.npz", "decode.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))
    golden_bc3(blocks, rgba2)
    golden_simd()


if __name__ == "__main__":
    main()
