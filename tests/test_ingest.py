"""The input side: stbi_load(..., 4)-style channel expansion and 2x2 box
mip chains, on the device against the numpy restatement in oracle/, and mip
chains encoded in one batch against the oracle."""
import numpy as np
import pytest

from icbc_gb300 import synth
from oracle import oracle as O


def _loop_mip_down(img):
    h, w = img.shape[:2]
    dh, dw = max(1, h >> 1), max(1, w >> 1)
    out = np.zeros((dh, dw, 4), np.uint8)
    for y in range(dh):
        for x in range(dw):
            for c in range(4):
                s = 2
                for yy in (2 * y, 2 * y + 1):
                    for xx in (2 * x, 2 * x + 1):
                        s += int(img[min(yy, h - 1), min(xx, w - 1), c])
                out[y, x, c] = s >> 2
    return out


def test_numpy_mip_step_matches_loops():
    for w, h in ((1, 1), (5, 1), (1, 6), (7, 3), (16, 9)):
        img = synth.quality_sweep_image(w, h, seed=w * 31 + h)
        assert np.array_equal(O.mip_down(img), _loop_mip_down(img)), (w, h)
    chain = O.mip_chain(synth.quality_sweep_image(37, 21, seed=1))
    assert [c.shape[:2] for c in chain] == [(21, 37), (10, 18), (5, 9), (2, 4), (1, 2), (1, 1)]


def test_numpy_expand_semantics():
    g = np.array([[0, 7], [200, 255]], np.uint8)
    e = O.expand_rgba8(g)
    assert e[1, 0].tolist() == [200, 200, 200, 255]
    ga = np.stack([g, 255 - g], -1)
    assert O.expand_rgba8(ga)[0, 1].tolist() == [7, 7, 7, 248]
    rgb = np.arange(2 * 2 * 3, dtype=np.uint8).reshape(2, 2, 3)
    assert O.expand_rgba8(rgb)[1, 1].tolist() == [9, 10, 11, 255]


@pytest.mark.gpu
def test_expand_rgba8_matches(gpu_lib):
    import torch
    ig = gpu_lib
    rng = np.random.default_rng(4)
    for c in (1, 2, 3, 4):
        for w, h in ((1, 1), (33, 7), (257, 130)):
            px = rng.integers(0, 256, (h, w, c), dtype=np.uint8)
            out = ig.expand_rgba8(torch.from_numpy(px).cuda())
            assert np.array_equal(out.cpu().numpy(), O.expand_rgba8(px)), (c, w, h)


@pytest.mark.gpu
def test_build_mips_matches(gpu_lib):
    import torch
    ig = gpu_lib
    for w, h in ((37, 21), (256, 128), (1, 9), (600, 3)):
        img = synth.quality_sweep_image(w, h, seed=w + h)
        chain = ig.build_mips(torch.from_numpy(img).cuda())
        ref = O.mip_chain(img)
        assert len(chain) == len(ref) == ig.mip_levels(w, h)
        for k, (a, b) in enumerate(zip(chain, ref)):
            assert np.array_equal(a.cpu().numpy(), b), (w, h, k)


@pytest.mark.gpu
def test_compress_mips_matches_oracle(gpu_lib):
    import torch
    ig = gpu_lib
    img = synth.quality_sweep_image(300, 172, seed=8)
    dev = torch.from_numpy(img).cuda()
    for level, dec, wm in ((8, 0, ig.WEIGHTS_ALPHA), (9, 1, ig.WEIGHTS_UNIFORM), (3, 3, ig.WEIGHTS_ALPHA)):
        cw = (0.299, 0.587, 0.114)
        blocks, errors, off = ig.compress_mips(dev, level, None, dec, cw, wm, with_errors=True)
        blocks, errors = blocks.cpu().numpy(), errors.cpu().numpy()
        for k, m in enumerate(O.mip_chain(img)):
            ob, oe = O.encode_image(m, level, dec, cw, 1 if wm == ig.WEIGHTS_ALPHA else 0, None, True, True,
                                    nthreads=8)
            assert np.array_equal(blocks[off[k]:off[k + 1]], ob), (level, k)
            assert np.array_equal(errors[off[k]:off[k + 1]].view(np.uint32), oe.view(np.uint32)), (level, k)
    with pytest.raises(ig.IcbcGpuError):
        ig.compress_mips(dev, 8, ig.mip_levels(300, 172) + 1)
