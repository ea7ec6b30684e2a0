"""GPU: the SIMD-profile entry points against the golden vectors of the
reference's SIMD builds and against the oracle's profiles."""
import os

import numpy as np
import pytest

from icbc_gb300 import synth
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("profile", range(1, 6))
def test_simd_blocks_match_golden(gpu_lib, profile):
    ig = gpu_lib
    g = np.load(os.path.join(GOLDEN, "simd.npz"))
    for si in range(2):
        cols, wt, cw = g["set%d_colors" % si], g["set%d_weights" % si], tuple(g["set%d_cw" % si])
        for lvl in (2, 4, 8, 9):
            for dec in range(4):
                for tc, tcb in ((1, 1), (0, 0)):
                    key = "set%d_P%d_L%d_D%d_tc%d_tcb%d" % (si, profile, lvl, dec, tc, tcb)
                    b, e = ig.compress_blocks(cols, wt, lvl, dec, cw, tc, tcb, simd_profile=profile)
                    assert np.array_equal(b, g[key + "_blocks"]), key
                    assert same_bits(e, g[key + "_errors"]), key


def test_neon_profile(gpu_lib):
    """ICBC_GPU_SIMD_NEON: the SSE4.1 build's golden output on ordinary blocks
    (the two builds share every operation but vsaturate's NaN handling), and
    the oracle's NEON profile -- not its SSE4.1 one -- on blocks with extreme
    weights, where NaN combinations decide the winner."""
    ig = gpu_lib
    g = np.load(os.path.join(GOLDEN, "simd.npz"))
    for si in range(2):
        cols, wt, cw = g["set%d_colors" % si], g["set%d_weights" % si], tuple(g["set%d_cw" % si])
        for lvl in (2, 4, 8, 9):
            for dec in range(4):
                for tc, tcb in ((1, 1), (0, 0)):
                    key = "set%d_P2_L%d_D%d_tc%d_tcb%d" % (si, lvl, dec, tc, tcb)
                    b, e = ig.compress_blocks(cols, wt, lvl, dec, cw, tc, tcb, simd_profile=ig.SIMD_NEON)
                    assert np.array_equal(b, g[key + "_blocks"]), key
                    assert same_bits(e, g[key + "_errors"]), key
    cols, w = synth.extreme_weight_blocks(6000, seed=8)
    for lvl in (2, 8, 9):
        for dec in (0, 3):
            b, e = ig.compress_blocks(cols, w, lvl, dec, (1, 1, 1), True, True, simd_profile=ig.SIMD_NEON)
            ob, oe = O.compress_blocks(cols, w, lvl, dec, (1, 1, 1), True, True, nthreads=8,
                                       profile=O.PROFILES["neon"])
            assert np.array_equal(b, ob), (lvl, dec)
            assert same_bits(e, oe), (lvl, dec)
    s4, _ = ig.compress_blocks(cols, w, 8, 0, (1, 1, 1), True, True, simd_profile=ig.SIMD_SSE41)
    nb, _ = ig.compress_blocks(cols, w, 8, 0, (1, 1, 1), True, True, simd_profile=ig.SIMD_NEON)
    assert (s4 != nb).any(1).sum() > 0


@pytest.mark.parametrize("profile", [-1, 0, 1, 2, 3, 4, 5])
def test_simd_image_matches_oracle(gpu_lib, profile):
    import torch
    ig = gpu_lib
    img = synth.quality_sweep_image(200, 136, seed=12)
    dev = torch.from_numpy(img).cuda()
    for lvl in (1, 3, 5, 8, 9):
        for dec in (0, 2):
            out, err = ig.compress_image(dev, lvl, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA, with_errors=True,
                                         simd_profile=profile)
            ob, oe = O.encode_image(img, lvl, dec, (0.299, 0.587, 0.114), 1, None, True, True, nthreads=8,
                                    profile=profile if profile >= 0 else O.PROFILES["neon"])
            assert np.array_equal(out.cpu().numpy(), ob), (lvl, dec)
            assert same_bits(err.cpu().numpy(), oe), (lvl, dec)


def test_simd_profile_zero_is_plain_and_invalid_rejected(gpu_lib):
    ig = gpu_lib
    cols, w = synth.mixed_blocks(300, seed=3)
    a, ea = ig.compress_blocks(cols, w, 8, 0)
    b, eb = ig.compress_blocks(cols, w, 8, 0, simd_profile=ig.SIMD_SCALAR)
    assert np.array_equal(a, b) and same_bits(ea, eb)
    for bad in (6, -2):
        with pytest.raises(ig.IcbcGpuError):
            ig.compress_blocks(cols, w, 8, 0, simd_profile=bad)
