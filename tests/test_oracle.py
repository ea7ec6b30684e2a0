"""CPU: the oracle against the reference's golden vectors and, where the
reference checkout exists, against the compiled reference itself."""
import hashlib
import os

import numpy as np
import pytest

from icbc_gb300 import synth
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLAGS = ((1, 1), (1, 0), (0, 0))
CWS = ((1.0, 1.0, 1.0), (0.299, 0.587, 0.114))


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "blocks.npz"))


@pytest.mark.parametrize("level", range(10))
def test_oracle_matches_golden_blocks(golden, level):
    colors, wr = golden["colors"], golden["weights_rand"]
    wu = np.ones_like(wr)
    for dec in range(4):
        for tc, tcb in FLAGS:
            for wn, wt in (("u", wu), ("r", wr)):
                cw = CWS[(dec + (wn == "r")) % 2]
                key = "L%d_D%d_tc%d_tcb%d_w%s" % (level, dec, tc, tcb, wn)
                b, e = O.compress_blocks(colors, wt, level, dec, cw, tc, tcb)
                assert np.array_equal(b, golden[key + "_blocks"]), key
                assert np.array_equal(e.view(np.uint32), golden[key + "_errors"].view(np.uint32)), key


def test_oracle_matches_golden_image():
    g = np.load(os.path.join(GOLDEN, "image512.npz"))
    img = synth.gradient_noise_rects(512, 512, 0)
    assert hashlib.sha256(img.tobytes()).digest() == g["sha256"].tobytes(), "generator output changed"
    b, e = O.encode_image(img, 8, 0, (1, 1, 1), 0, None, True, True, nthreads=4)
    assert np.array_equal(b, g["blocks"])
    assert np.array_equal(e.view(np.uint32), g["errors"].view(np.uint32))


def test_oracle_decode_evaluate_golden():
    g = np.load(os.path.join(GOLDEN, "decode.npz"))
    for d in range(4):
        assert np.array_equal(O.decode_bc1(g["blocks"], d), g["decoded_D%d" % d])
        e = O.evaluate_bc1_error(g["rgba"], g["blocks"], d)
        assert np.array_equal(e.view(np.uint32), g["error_D%d" % d].view(np.uint32))


def test_oracle_bc3_golden():
    """decode_bc3 / evaluate_bc3_error as the reference implements them
    (4-colour palette, alpha0 everywhere), against its own outputs."""
    g = np.load(os.path.join(GOLDEN, "bc3.npz"))
    for d in range(4):
        assert np.array_equal(O.decode_bc3(g["blocks"], d), g["decoded_D%d" % d])
        for ab in (0, 1):
            e = O.evaluate_bc3_error(g["rgba"], g["blocks"], ab, d)
            assert np.array_equal(e.view(np.uint32), g["error_D%d_blend%d" % (d, ab)].view(np.uint32)), (d, ab)


def test_image_path_equals_block_path():
    """Image encode (edge replication, u8/255, alpha weights) equals the block
    API on the gathered texels, for a size that is not a multiple of 4."""
    img = synth.quality_sweep_image(70, 45, seed=3)
    cols, w, _ = O.image_blocks(img, weight_mode=1)
    for level in (0, 5, 9):
        b1, e1 = O.encode_image(img, level, 2, (0.299, 0.587, 0.114), 1, None, True, True)
        b2, e2 = O.compress_blocks(cols, w, level, 2, (0.299, 0.587, 0.114), True, True)
        assert np.array_equal(b1, b2) and np.array_equal(e1, e2)


def test_threaded_equals_single():
    cols, w = synth.mixed_blocks(3000, seed=8)
    b1, e1 = O.compress_blocks(cols, w, 9, 1, (1, 1, 1), True, True, nthreads=1)
    b8, e8 = O.compress_blocks(cols, w, 9, 1, (1, 1, 1), True, True, nthreads=8)
    assert np.array_equal(b1, b8) and np.array_equal(e1, e8)


@pytest.mark.skipif(O.ref() is None, reason="reference checkout not available")
@pytest.mark.parametrize("level", range(10))
def test_oracle_matches_compiled_reference(level):
    cols, w = synth.mixed_blocks(1500, seed=100 + level)
    for dec in range(4):
        for tc, tcb in FLAGS:
            cw = CWS[dec % 2]
            a, ea = O.compress_blocks(cols, w, level, dec, cw, tc, tcb)
            b, eb = O.ref_compress_blocks(cols, w, level, dec, cw, tc, tcb)
            assert np.array_equal(a, b), (level, dec, tc, tcb)
            assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32)), (level, dec, tc, tcb)


@pytest.mark.skipif(O.ref() is None, reason="reference checkout not available")
def test_oracle_prior_output_semantics():
    """Weights so large the cluster-fit error overflows: the reference keeps the
    caller's prior bytes at levels 4..9; so must the oracle."""
    cols, _ = synth.mixed_blocks(200, seed=9)
    w = np.full((200, 16), 3e38, np.float32)
    prior = np.arange(200 * 8, dtype=np.uint8).reshape(200, 8)
    for level in (4, 8, 9):
        a, ea = O.compress_blocks(cols, w, level, 0, (1, 1, 1), True, True, out=prior)
        b, eb = O.ref_compress_blocks(cols, w, level, 0, (1, 1, 1), True, True, out=prior)
        assert np.array_equal(a, b)
        assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32))


SIMD_LEVELS = (2, 4, 8, 9)
SIMD_FLAGS = ((1, 1), (0, 0))


@pytest.mark.parametrize("profile", range(1, 6))
def test_oracle_simd_profiles_match_golden(profile):
    """The oracle's SIMD profiles against the golden vectors the reference's
    SSE2 / SSE4.1 / AVX / AVX2 / AVX-512 builds produced."""
    g = np.load(os.path.join(GOLDEN, "simd.npz"))
    for si in range(2):
        cols, wt, cw = g["set%d_colors" % si], g["set%d_weights" % si], tuple(g["set%d_cw" % si])
        for lvl in SIMD_LEVELS:
            for dec in range(4):
                for tc, tcb in SIMD_FLAGS:
                    key = "set%d_P%d_L%d_D%d_tc%d_tcb%d" % (si, profile, lvl, dec, tc, tcb)
                    b, e = O.compress_blocks(cols, wt, lvl, dec, cw, tc, tcb, profile=profile)
                    assert np.array_equal(b, g[key + "_blocks"]), key
                    assert np.array_equal(e.view(np.uint32), g[key + "_errors"].view(np.uint32)), key


def test_oracle_neon_profile():
    """The NEON profile (ICBC_SIMD=-1 without FP contraction) runs the SSE4.1
    build's arithmetic -- four lanes, half-even vround01, unfused vmadd --
    except that vsaturate keeps a NaN.  No NaN reaches a winning combination
    on ordinary blocks, so there it must give the SSE4.1 build's golden
    output; blocks with weights spread over 1e-30..1e30 make degenerate
    combinations NaN, and there the two profiles must part on some blocks."""
    g = np.load(os.path.join(GOLDEN, "simd.npz"))
    neon = O.PROFILES["neon"]
    for si in range(2):
        cols, wt, cw = g["set%d_colors" % si], g["set%d_weights" % si], tuple(g["set%d_cw" % si])
        for lvl in SIMD_LEVELS:
            for dec in range(4):
                for tc, tcb in SIMD_FLAGS:
                    key = "set%d_P2_L%d_D%d_tc%d_tcb%d" % (si, lvl, dec, tc, tcb)
                    b, e = O.compress_blocks(cols, wt, lvl, dec, cw, tc, tcb, profile=neon)
                    assert np.array_equal(b, g[key + "_blocks"]), key
                    assert np.array_equal(e.view(np.uint32), g[key + "_errors"].view(np.uint32)), key
    cols, w = synth.extreme_weight_blocks(4000, seed=5)
    a, _ = O.compress_blocks(cols, w, 8, 0, (1, 1, 1), True, True, nthreads=8, profile=O.PROFILES["sse41"])
    b, _ = O.compress_blocks(cols, w, 8, 0, (1, 1, 1), True, True, nthreads=8, profile=neon)
    assert 0 < (a != b).any(1).sum() < 4000


def _exact_colour_blocks(n, ncol, seed):
    """n blocks of exactly ncol distinct colours (half of them close
    together), with weights mixing 1 and random values."""
    rng = np.random.default_rng(seed)
    pal = rng.integers(0, 256, (n, ncol, 3))
    pal[: n // 2] = np.clip(pal[: n // 2, :1] + rng.integers(-20, 21, (n // 2, ncol, 3)), 0, 255)
    idx = np.concatenate([np.tile(np.arange(ncol), (n, 1)), rng.integers(0, ncol, (n, 16 - ncol))], 1)
    idx = rng.permuted(idx, axis=1)
    cols = np.ones((n, 16, 4), np.float32)
    cols[:, :, :3] = np.take_along_axis(pal, idx[:, :, None], 1) / 255.0
    w = np.where(rng.random((n, 16)) < 0.5, 1.0, rng.random((n, 16))).astype(np.float32)
    return cols, w


@pytest.mark.parametrize("profile", ["sse2", "sse41", "neon"])
def test_oracle_vector_loops_match_lane_loops(profile):
    """The 4-lane vector form of the cluster loops (the timed CPU encoder)
    against the scalar-lane form, bit for bit: mixed blocks, blocks of exactly
    8 and 12 colours (where AVX2's and NEON's gathers read past their tables),
    extreme weights (NaN combinations, kept by NEON's vsaturate)."""
    pr = O.PROFILES[profile]
    sets = [synth.mixed_blocks(600, seed=31), _exact_colour_blocks(400, 8, 32), _exact_colour_blocks(400, 12, 33),
            synth.extreme_weight_blocks(600, seed=34)]
    for cols, w in sets:
        for lvl in (1, 5, 7, 9):
            for dec in (0, 1):
                for tc, tcb in SIMD_FLAGS:
                    a, ea = O.compress_blocks(cols, w, lvl, dec, (1, .7, .3), tc, tcb, nthreads=4, profile=pr)
                    b, eb = O.compress_blocks(cols, w, lvl, dec, (1, .7, .3), tc, tcb, nthreads=4, profile=pr,
                                              vector=True)
                    assert np.array_equal(a, b), (profile, lvl, dec, tc, tcb)
                    assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32)), (profile, lvl, dec, tc, tcb)


@pytest.mark.parametrize("profile", [1, 2])
def test_oracle_vector_loops_match_golden(profile):
    """The vector form under the SSE2 and SSE4.1 profiles against the golden
    vectors of the reference's own SSE2 and SSE4.1 builds."""
    g = np.load(os.path.join(GOLDEN, "simd.npz"))
    for si in range(2):
        cols, wt, cw = g["set%d_colors" % si], g["set%d_weights" % si], tuple(g["set%d_cw" % si])
        for lvl in SIMD_LEVELS:
            for dec in range(4):
                for tc, tcb in SIMD_FLAGS:
                    key = "set%d_P%d_L%d_D%d_tc%d_tcb%d" % (si, profile, lvl, dec, tc, tcb)
                    b, e = O.compress_blocks(cols, wt, lvl, dec, cw, tc, tcb, profile=profile, vector=True)
                    assert np.array_equal(b, g[key + "_blocks"]), key
                    assert np.array_equal(e.view(np.uint32), g[key + "_errors"].view(np.uint32)), key


@pytest.mark.parametrize("profile", range(1, 6))
def test_oracle_simd_profiles_match_compiled_builds(profile):
    """The same against the SIMD builds themselves on other blocks (x86 hosts
    with the reference checkout only)."""
    if O.ref(profile) is None:
        pytest.skip("the reference's SIMD builds are not available here")
    cols, w = synth.mixed_blocks(400, seed=21)
    img = synth.quality_sweep_image(128, 64, seed=9)
    ci, wi, _ = O.image_blocks(img, weight_mode=1)
    for c, wt in ((cols, w), (ci, wi)):
        for lvl in SIMD_LEVELS:
            for dec in range(4):
                for tc, tcb in SIMD_FLAGS:
                    cw = (0.299, 0.587, 0.114) if dec % 2 else (1.0, 1.0, 1.0)
                    rb, re = O.ref_compress_blocks(c, wt, lvl, dec, cw, tc, tcb, profile=profile)
                    ob, oe = O.compress_blocks(c, wt, lvl, dec, cw, tc, tcb, nthreads=4, profile=profile)
                    assert np.array_equal(rb, ob), (lvl, dec, tc, tcb)
                    assert np.array_equal(re.view(np.uint32), oe.view(np.uint32)), (lvl, dec, tc, tcb)
