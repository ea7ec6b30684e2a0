"""GPU: the sm_103a kernels against the oracle and the reference's golden
vectors.  Integer/byte outputs must be bit-identical, and so must the float
error each block returns (the arithmetic is the reference's, operation for
operation), so every comparison here is exact equality."""
import os

import numpy as np
import pytest

from icbc_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLAGS = ((1, 1), (1, 0), (0, 0))
CWS = ((1.0, 1.0, 1.0), (0.299, 0.587, 0.114))


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("level", range(10))
def test_blocks_match_golden(gpu_lib, level):
    ig = gpu_lib
    g = np.load(os.path.join(GOLDEN, "blocks.npz"))
    colors, wr = g["colors"], g["weights_rand"]
    wu = np.ones_like(wr)
    for dec in range(4):
        for tc, tcb in FLAGS:
            for wn, wt in (("u", wu), ("r", wr)):
                cw = CWS[(dec + (wn == "r")) % 2]
                key = "L%d_D%d_tc%d_tcb%d_w%s" % (level, dec, tc, tcb, wn)
                b, e = ig.compress_blocks(colors, wt, level, dec, cw, tc, tcb)
                assert np.array_equal(b, g[key + "_blocks"]), key
                assert same_bits(e, g[key + "_errors"]), key


@pytest.mark.parametrize("level", range(10))
def test_blocks_match_oracle_mixture(gpu_lib, level):
    ig = gpu_lib
    cols, w = synth.mixed_blocks(6000, seed=200 + level)
    for dec in range(4):
        cw = CWS[dec % 2]
        b, e = ig.compress_blocks(cols, w, level, dec, cw, True, True)
        ob, oe = O.compress_blocks(cols, w, level, dec, cw, True, True, nthreads=8)
        bad = np.nonzero((b != ob).any(1))[0]
        assert bad.size == 0, (level, dec, bad[:10])
        assert same_bits(e, oe)


def test_default_decoder_follows_init(gpu_lib):
    ig = gpu_lib
    cols, w = synth.mixed_blocks(500, seed=17)
    try:
        for dec in range(4):
            ig.init(dec)
            b, e = ig.compress_blocks(cols, w, 8, ig.DECODER_DEFAULT, (1, 1, 1), True, True)
            ob, oe = O.compress_blocks(cols, w, 8, dec, (1, 1, 1), True, True)
            assert np.array_equal(b, ob) and same_bits(e, oe)
    finally:
        ig.init(ig.Decoder_D3D10)


def test_single_block_api(gpu_lib):
    ig = gpu_lib
    cols, w = synth.mixed_blocks(40, seed=21)
    for i in range(40):
        out = bytearray(8)
        err = ig.compress_bc1(9, cols[i], w[i], (1, 1, 1), True, True, out)
        ob, oe = O.compress_blocks(cols[i:i + 1], w[i:i + 1], 9, 0, (1, 1, 1), True, True)
        assert bytes(out) == bytes(ob[0]) and same_bits(err, oe[0])


def _to_dev(img):
    import torch
    return torch.from_numpy(np.ascontiguousarray(img)).cuda()


def test_image512_quality_default_golden(gpu_lib):
    ig = gpu_lib
    g = np.load(os.path.join(GOLDEN, "image512.npz"))
    img = synth.gradient_noise_rects(512, 512, 0)
    out, err = ig.compress_image(_to_dev(img), 8, 0, (1, 1, 1), with_errors=True)
    assert np.array_equal(out.cpu().numpy(), g["blocks"])
    assert same_bits(err.cpu().numpy(), g["errors"])


@pytest.mark.parametrize("level", range(10))
def test_image_alpha_weights_all_levels(gpu_lib, level):
    ig = gpu_lib
    img = synth.quality_sweep_image(256, 192, seed=5)
    cw = (0.299, 0.587, 0.114)
    for dec in (0, 1, 2, 3):
        out, err = ig.compress_image(_to_dev(img), level, dec, cw, weight_mode=ig.WEIGHTS_ALPHA, with_errors=True)
        ob, oe = O.encode_image(img, level, dec, cw, 1, None, True, True, nthreads=8)
        assert np.array_equal(out.cpu().numpy(), ob), (level, dec)
        assert same_bits(err.cpu().numpy(), oe)


@pytest.mark.parametrize("size", [(1, 1), (3, 5), (5, 3), (4, 4), (7, 9), (130, 66), (66, 130), (33, 1)])
def test_image_edge_sizes(gpu_lib, size):
    ig = gpu_lib
    w, h = size
    img = synth.hard_mixture_image(w, h, seed=w * 100 + h)
    for level in (0, 1, 4, 8, 9):
        out = ig.compress_image(_to_dev(img), level, 0, (1, 1, 1), weight_mode=ig.WEIGHTS_ALPHA)
        ob, _ = O.encode_image(img, level, 0, (1, 1, 1), 1, None, True, True)
        assert np.array_equal(out.cpu().numpy(), ob), (size, level)


def test_image_unaligned_pitch_and_weight_plane(gpu_lib):
    import torch
    ig = gpu_lib
    img = synth.gradient_noise_rects(61, 47, seed=8)
    # rows padded to an odd number of pixels: pitch not a multiple of 16 bytes
    padded = np.zeros((47, 63, 4), np.uint8)
    padded[:, :61] = img
    dev = torch.from_numpy(padded).cuda()
    plane = (synth.uniform(3, 0, (47, 61)) * 2).astype(np.float32)
    plane[::3, ::2] = 0
    dplane = torch.from_numpy(plane).cuda()
    nb = ig.blocks_of(61, 47)
    out = torch.zeros((nb, 8), dtype=torch.uint8, device="cuda")
    d = ig.image_desc(dev, 9, out, None, 1, (1, 1, 1), ig.WEIGHTS_PLANE, dplane, width=61, height=47,
                      pitch=63 * 4)
    import ctypes
    ig._check(ig.load().icbc_gpu_compress_bc1_image(ctypes.byref(d), ig._stream_ptr()), "image")
    torch.cuda.synchronize()
    ob, _ = O.encode_image(img, 9, 1, (1, 1, 1), 2, plane, True, True)
    assert np.array_equal(out.cpu().numpy(), ob)


def test_prior_output_kept_when_no_finite_error(gpu_lib):
    ig = gpu_lib
    cols, _ = synth.mixed_blocks(300, seed=9)
    w = np.full((300, 16), 3e38, np.float32)
    prior = np.arange(300 * 8, dtype=np.uint8).reshape(300, 8)
    for level in (4, 8, 9):
        b, e = ig.compress_blocks(cols, w, level, 0, (1, 1, 1), True, True, initial=prior)
        ob, oe = O.compress_blocks(cols, w, level, 0, (1, 1, 1), True, True, out=prior)
        assert np.array_equal(b, ob) and same_bits(e, oe)


def test_batch_matches_plain_and_oracle(gpu_lib):
    import torch
    ig = gpu_lib
    specs = synth.batch_specs(40, seed=5, lo=8, hi=300)
    imgs, outs, descs, plain = [], [], [], []
    for s in specs:
        img = synth.gradient_noise_rects(s.width, s.height, s.seed)
        dev = _to_dev(img)
        nb = ig.blocks_of(s.width, s.height)
        out = torch.zeros((nb, 8), dtype=torch.uint8, device="cuda")
        imgs.append((img, dev))
        outs.append(out)
        descs.append(ig.image_desc(dev, s.level, out, None, s.decoder))
        plain.append(ig.compress_image(dev, s.level, s.decoder))
    batch = ig.Batch(descs)
    for _ in range(2):  # a planned batch relaunches (graph replay) with the same result
        batch.launch()
        torch.cuda.synchronize()
        for (img, _), s, out, p in zip(imgs, specs, outs, plain):
            assert np.array_equal(out.cpu().numpy(), p.cpu().numpy()), (s.width, s.height, s.level)
    batch.close()
    for (img, _), s, out in list(zip(imgs, specs, outs))[::5]:
        ob, _ = O.encode_image(img, s.level, s.decoder, (1, 1, 1), 0, None, True, True, nthreads=8)
        assert np.array_equal(out.cpu().numpy(), ob)


_FIRST_CALL_BATCH = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import icbc_gb300 as ig
from icbc_gb300 import synth
ig.init(ig.Decoder_D3D10)
imgs = [torch.from_numpy(synth.hard_mixture_image(4096, 4096, 7)).cuda(),
        torch.from_numpy(synth.gradient_noise_rects(200, 120, 3)).cuda()]
outs = [[torch.zeros((ig.blocks_of(im.shape[1], im.shape[0]), 8), dtype=torch.uint8, device="cuda")
         for im in imgs] for _ in range(2)]
descs = [[ig.image_desc(im, lv, o, None, 0, (1, 1, 1), ig.WEIGHTS_ALPHA) for im, o, lv in zip(imgs, outs[k], (9, 8))]
         for k in range(2)]
batch = ig.Batch(descs[0])   # the first encode of the process
batch.launch()
ig.compress_images_each(descs[1])
torch.cuda.synchronize()
assert all(torch.equal(a, b) for a, b in zip(outs[0], outs[1]))
print("ok")
"""


def test_batch_as_first_call_of_a_process(gpu_lib):
    """A batch whose image is large enough (2^20 blocks) for its own kernels
    takes stream-ordered scratch inside the batch's graph capture; that must
    work when the batch is the first encode of a process (the scratch pool is
    created before the capture)."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FIRST_CALL_BATCH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr[-2000:]


def test_batch_level9_refinement_pass(gpu_lib):
    """Level-9 images of a batch refine in a second launch whose lanes serve
    blocks of different images: each image's decoder, flags, colour weights
    and alpha weights must reach its blocks.  Errors are checked too."""
    import torch
    ig = gpu_lib
    rng = np.random.default_rng(11)
    cases = []
    for i in range(24):
        w, h = int(rng.integers(5, 160)), int(rng.integers(5, 160))
        level = 9 if i % 4 else int(rng.choice([2, 8]))
        cases.append(dict(w=w, h=h, level=level, decoder=i % 4, tcm=bool(i % 3), tcb=bool(i % 5),
                          cw=(1.0, 1.0, 1.0) if i % 2 else (0.299, 0.587, 0.114),
                          wm=ig.WEIGHTS_ALPHA if i % 3 == 1 else ig.WEIGHTS_UNIFORM, seed=100 + i))
    imgs, outs, errs, descs = [], [], [], []
    for c in cases:
        img = synth.quality_sweep_image(c["w"], c["h"], seed=c["seed"])
        dev = _to_dev(img)
        nb = ig.blocks_of(c["w"], c["h"])
        out = torch.zeros((nb, 8), dtype=torch.uint8, device="cuda")
        err = torch.zeros(nb, dtype=torch.float32, device="cuda")
        imgs.append((img, dev))
        outs.append(out)
        errs.append(err)
        descs.append(ig.image_desc(dev, c["level"], out, err, c["decoder"], c["cw"], c["wm"], None, c["tcm"], c["tcb"]))
    batch = ig.Batch(descs)
    batch.launch()
    torch.cuda.synchronize()
    for (img, dev), c, out, err in zip(imgs, cases, outs, errs):
        pe = torch.zeros_like(err)
        po = ig.compress_image(dev, c["level"], c["decoder"], c["cw"], c["wm"], None, c["tcm"], c["tcb"], errors=pe)
        assert np.array_equal(out.cpu().numpy(), po.cpu().numpy()), c
        assert same_bits(err.cpu().numpy(), pe.cpu().numpy()), c
    batch.close()
    for (img, _), c, out, err in list(zip(imgs, cases, outs, errs))[::3]:
        ob, oe = O.encode_image(img, c["level"], c["decoder"], c["cw"], c["wm"], None, c["tcm"], c["tcb"], nthreads=8)
        assert np.array_equal(out.cpu().numpy(), ob), c
        assert same_bits(err.cpu().numpy(), oe), c


def test_batch_with_own_launch_images(gpu_lib):
    """Images of 2^20 blocks or more run as their level's own kernels inside
    the batch graph (level 9 with the batch's refinement slots); the rest
    share the batch kernel.  Both kinds equal the plain launches, twice."""
    import torch
    ig = gpu_lib
    specs = [(4096, 4096, 9, 0), (4100, 4096, 2, 1), (64, 64, 9, 2), (100, 52, 5, 3), (33, 17, 9, 0)]
    descs, outs, plains, devs = [], [], [], []  # the descriptors hold raw pointers: keep the images alive
    for i, (w, h, level, dec) in enumerate(specs):
        dev = synth.hard_mixture_torch(w, h, 50 + i, torch.device("cuda")) if w >= 4096 else \
            _to_dev(synth.quality_sweep_image(w, h, seed=60 + i))
        devs.append(dev)
        nb = ig.blocks_of(w, h)
        out = torch.zeros((nb, 8), dtype=torch.uint8, device="cuda")
        descs.append(ig.image_desc(dev, level, out, None, dec, (1, 1, 1), ig.WEIGHTS_ALPHA))
        outs.append(out)
        plains.append(ig.compress_image(dev, level, dec, (1, 1, 1), ig.WEIGHTS_ALPHA))
    batch = ig.Batch(descs)
    for _ in range(2):
        batch.launch()
        torch.cuda.synchronize()
        for s_, out, p in zip(specs, outs, plains):
            assert torch.equal(out, p), s_
    batch.close()


def test_host_buffer_path_in_bands(gpu_lib):
    """Images of 128+ block rows go through the host path in bands (copies
    of one band overlapping the encode of another); results equal the device
    path and the oracle, weight planes and level 4+ prior output included."""
    import torch
    ig = gpu_lib
    w, h = 1030, 2050  # 513 block rows: 8 bands (2 at level 9), the last one with a partial block row
    img = synth.quality_sweep_image(w, h, seed=21)
    plane = np.random.default_rng(3).random((h, w), dtype=np.float32)
    dev = _to_dev(img)
    dplane = torch.from_numpy(plane).cuda()
    nb = ig.blocks_of(w, h)
    for level, wm in ((9, ig.WEIGHTS_ALPHA), (8, ig.WEIGHTS_ALPHA), (4, ig.WEIGHTS_PLANE), (1, ig.WEIGHTS_UNIFORM)):
        errs = np.zeros(nb, np.float32)
        out = ig.compress_image_host(img, level, 1, (0.299, 0.587, 0.114), wm, errors=errs,
                                     weight_plane=plane if wm == ig.WEIGHTS_PLANE else None)
        db, de = ig.compress_image(dev, level, 1, (0.299, 0.587, 0.114), wm,
                                   dplane if wm == ig.WEIGHTS_PLANE else None, with_errors=True)
        assert np.array_equal(out, db.cpu().numpy()), level
        assert same_bits(errs, de.cpu().numpy()), level
        if level == 8:
            ob, oe = O.encode_image(img, level, 1, (0.299, 0.587, 0.114), 1, None, True, True, nthreads=16)
            assert np.array_equal(out, ob) and same_bits(errs, oe)


def test_byte_rows_equal_float_rows(gpu_lib):
    """The RGBA8 kernels keep texels as bytes (alpha weights read through the
    i/255 table); a weight plane holding the same alpha/255 floats takes the
    float-row kernels.  Same floats in, so the same bytes and errors out."""
    import torch
    ig = gpu_lib
    img = synth.quality_sweep_image(260, 140, seed=31)
    dev = _to_dev(img)
    plane = torch.from_numpy((img[..., 3].astype(np.float64) / 255.0).astype(np.float32)).cuda()
    lut = (np.arange(256, dtype=np.float32) / np.float32(255.0)).astype(np.float32)
    assert np.array_equal(plane.cpu().numpy(), lut[img[..., 3]])
    for level in range(2, 10):
        for dec in (0, 3):
            ob, oe = ig.compress_image(dev, level, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA, with_errors=True)
            fb, fe = ig.compress_image(dev, level, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_PLANE, plane,
                                       with_errors=True)
            assert torch.equal(ob, fb), (level, dec)
            assert same_bits(oe.cpu().numpy(), fe.cpu().numpy()), (level, dec)


def test_concurrent_calls_on_own_streams(gpu_lib):
    """Calls are thread-safe per stream: four host threads encode different
    images (levels 3, 8 and 9, image, float-block and host-buffer forms) on
    their own streams at once; every result equals the same call made alone."""
    import threading
    import torch
    ig = gpu_lib
    jobs = []
    for i in range(4):
        img = synth.quality_sweep_image(300 + 40 * i, 200 + 24 * i, seed=70 + i)
        jobs.append((img, _to_dev(img), (3, 8, 9, 9)[i], i % 4))
    alone = []
    for img, dev, level, dec in jobs:
        a = ig.compress_image(dev, level, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA).cpu().numpy()
        cols, w, _ = O.image_blocks(img, weight_mode=1)
        b, _ = ig.compress_blocks(cols, w, level, dec, (0.299, 0.587, 0.114))
        c = ig.compress_image_host(img, level, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA)
        alone.append((a, b, c, cols, w))
    results = [None] * 4
    errors = []

    def work(k):
        try:
            img, dev, level, dec = jobs[k]
            s = torch.cuda.Stream()
            got = []
            for _ in range(3):
                with torch.cuda.stream(s):
                    out = ig.compress_image(dev, level, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA, stream=s)
                s.synchronize()
                b, _ = ig.compress_blocks(alone[k][3], alone[k][4], level, dec, (0.299, 0.587, 0.114), stream=s)
                c = ig.compress_image_host(img, level, dec, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA)
                got.append((out.cpu().numpy(), b, c))
            results[k] = got
        except Exception as e:  # surfaced below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k in range(4):
        for a, b, c in results[k]:
            assert np.array_equal(a, alone[k][0]) and np.array_equal(b, alone[k][1]) and np.array_equal(c, alone[k][2]), k


def test_two_pass_levels_edge_cases(gpu_lib):
    """Levels 2-9 list the blocks of two or more reduced colours in a first
    pass: an image with none (flat), one with all (noise) and a mixed one with
    partial edge blocks all equal the oracle, blocks and errors."""
    ig = gpu_lib
    rng = np.random.default_rng(17)
    flat = np.full((36, 52, 4), 200, np.uint8)
    noise = rng.integers(0, 256, (40, 44, 4), dtype=np.uint8)
    mixed = synth.quality_sweep_image(101, 67, seed=5)
    for img in (flat, noise, mixed):
        dev = _to_dev(img)
        for level in range(2, 10):
            out, err = ig.compress_image(dev, level, 1, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA, with_errors=True)
            ob, oe = O.encode_image(img, level, 1, (0.299, 0.587, 0.114), 1, None, True, True, nthreads=8)
            assert np.array_equal(out.cpu().numpy(), ob), (img.shape, level)
            assert same_bits(err.cpu().numpy(), oe), (img.shape, level)


def test_two_pass_batch_edge_cases(gpu_lib):
    """A batch without weight planes finishes the blocks of 0 or 1 reduced
    colours of its level-2..9 images in a first pass and lists the others per
    image for the encoder: flat images (empty lists), noise (every block
    listed), mixed ones and level-0/1 images in the same batch equal the plain
    launches, blocks and errors, on two launches; a subset equals the oracle."""
    import torch
    ig = gpu_lib
    rng = np.random.default_rng(23)
    sources = [np.full((36, 52, 4), 200, np.uint8), rng.integers(0, 256, (40, 44, 4), dtype=np.uint8),
               synth.quality_sweep_image(101, 67, seed=9), np.full((1, 1, 4), 7, np.uint8),
               synth.quality_sweep_image(5, 3, seed=10)]
    cases, devs = [], []
    for i in range(30):
        img = sources[i % len(sources)]
        cases.append(dict(img=img, level=i % 10, decoder=i % 4, cw=(1.0, 1.0, 1.0) if i % 2 else (0.299, 0.587, 0.114),
                          wm=ig.WEIGHTS_ALPHA if i % 3 == 0 else ig.WEIGHTS_UNIFORM, tcm=bool(i % 4), tcb=bool(i % 7)))
        devs.append(_to_dev(img))
    outs, errs, descs = [], [], []
    for c, dev in zip(cases, devs):
        nb = ig.blocks_of(c["img"].shape[1], c["img"].shape[0])
        outs.append(torch.zeros((nb, 8), dtype=torch.uint8, device="cuda"))
        errs.append(torch.zeros(nb, dtype=torch.float32, device="cuda"))
        descs.append(ig.image_desc(dev, c["level"], outs[-1], errs[-1], c["decoder"], c["cw"], c["wm"], None,
                                   c["tcm"], c["tcb"]))
    plain = []
    for c, dev in zip(cases, devs):
        pe = torch.zeros(ig.blocks_of(c["img"].shape[1], c["img"].shape[0]), dtype=torch.float32, device="cuda")
        po = ig.compress_image(dev, c["level"], c["decoder"], c["cw"], c["wm"], None, c["tcm"], c["tcb"], errors=pe)
        plain.append((po.cpu().numpy(), pe.cpu().numpy()))
    batch = ig.Batch(descs)
    for _ in range(2):
        for o, e in zip(outs, errs):
            o.zero_()
            e.zero_()
        batch.launch()
        torch.cuda.synchronize()
        for c, out, err, (po, pe) in zip(cases, outs, errs, plain):
            key = (c["img"].shape, c["level"], c["decoder"])
            assert np.array_equal(out.cpu().numpy(), po), key
            assert same_bits(err.cpu().numpy(), pe), key
    batch.close()
    for c, out, err in list(zip(cases, outs, errs))[::4]:
        ob, oe = O.encode_image(c["img"], c["level"], c["decoder"], c["cw"], c["wm"], None, c["tcm"], c["tcb"],
                                nthreads=8)
        assert np.array_equal(out.cpu().numpy(), ob), (c["img"].shape, c["level"])
        assert same_bits(err.cpu().numpy(), oe), (c["img"].shape, c["level"])


def test_batch_with_weight_plane_image(gpu_lib):
    """A batch holding an image with a float weight plane runs the all-levels
    float-row kernel in one pass (no lists); its images at every level, the
    plane image included, equal the plain launches, blocks and errors."""
    import torch
    ig = gpu_lib
    rng = np.random.default_rng(41)
    w, h = 67, 45
    plane = torch.from_numpy((rng.random((h, w)) * 2).astype(np.float32)).cuda()
    imgs = [synth.quality_sweep_image(w, h, seed=70 + i) for i in range(10)]
    devs = [_to_dev(im) for im in imgs]
    nb = ig.blocks_of(w, h)
    outs = [torch.zeros((nb, 8), dtype=torch.uint8, device="cuda") for _ in imgs]
    errs = [torch.zeros(nb, dtype=torch.float32, device="cuda") for _ in imgs]
    descs, plain = [], []
    for i, (dev, out, err) in enumerate(zip(devs, outs, errs)):
        wm, wp = (ig.WEIGHTS_PLANE, plane) if i == 4 else (ig.WEIGHTS_ALPHA, None)
        descs.append(ig.image_desc(dev, i, out, err, i % 4, (0.299, 0.587, 0.114), wm, wp))
        pe = torch.zeros(nb, dtype=torch.float32, device="cuda")
        po = ig.compress_image(dev, i, i % 4, (0.299, 0.587, 0.114), wm, wp, errors=pe)
        plain.append((po.cpu().numpy(), pe.cpu().numpy()))
    batch = ig.Batch(descs)
    batch.launch()
    torch.cuda.synchronize()
    for i, (out, err, (po, pe)) in enumerate(zip(outs, errs, plain)):
        assert np.array_equal(out.cpu().numpy(), po), i
        assert same_bits(err.cpu().numpy(), pe), i
    batch.close()


def test_decode_evaluate_golden(gpu_lib):
    import torch
    ig = gpu_lib
    g = np.load(os.path.join(GOLDEN, "decode.npz"))
    blocks = torch.from_numpy(g["blocks"]).cuda()
    rgba = torch.from_numpy(g["rgba"]).cuda()
    for d in range(4):
        assert np.array_equal(ig.decode_blocks(blocks, d).cpu().numpy(), g["decoded_D%d" % d])
        assert same_bits(ig.evaluate_errors(rgba, blocks, d).cpu().numpy(), g["error_D%d" % d])


def test_bc3_decode_evaluate_golden(gpu_lib):
    import torch
    ig = gpu_lib
    g = np.load(os.path.join(GOLDEN, "bc3.npz"))
    blocks = torch.from_numpy(g["blocks"]).cuda()
    rgba = torch.from_numpy(g["rgba"]).cuda()
    for d in range(4):
        assert np.array_equal(ig.decode_bc3_blocks(blocks, d).cpu().numpy(), g["decoded_D%d" % d])
        for ab in (0, 1):
            e = ig.evaluate_bc3_errors(rgba, blocks, bool(ab), d).cpu().numpy()
            assert same_bits(e, g["error_D%d_blend%d" % (d, ab)]), (d, ab)


def test_host_buffer_path(gpu_lib):
    ig = gpu_lib
    img = synth.quality_sweep_image(200, 120, seed=2)
    for level in (1, 8):
        errs = np.zeros(ig.blocks_of(200, 120), np.float32)
        out = ig.compress_image_host(img, level, 0, (0.299, 0.587, 0.114), ig.WEIGHTS_ALPHA, errors=errs)
        ob, oe = O.encode_image(img, level, 0, (0.299, 0.587, 0.114), 1, None, True, True)
        assert np.array_equal(out, ob) and same_bits(errs, oe)


@pytest.fixture(scope="module")
def sweep_image():
    return synth.quality_sweep_image(4096, 4096, seed=1)


@pytest.mark.parametrize("level", range(10))
def test_full_size_parity(gpu_lib, sweep_image, level):
    """The 4096x4096 quality-sweep workload (alpha weights, luma colour
    weights, D3D10): every block and every returned error equals the
    oracle's, at every level; the GPU's decode + evaluate over the whole image
    equals the oracle's FP64 decode-and-compare."""
    import torch
    ig = gpu_lib
    img = sweep_image
    cw = (0.299, 0.587, 0.114)
    out, err = ig.compress_image(_to_dev(img), level, 0, cw, weight_mode=ig.WEIGHTS_ALPHA, with_errors=True)
    blocks = out.cpu().numpy()
    ob, oe = O.encode_image(img, level, 0, cw, 1, None, True, True, nthreads=os.cpu_count() or 1)
    bad = np.flatnonzero((blocks != ob).any(1))
    assert bad.size == 0, (level, bad[:10])
    assert same_bits(err.cpu().numpy(), oe)
    _, _, tex = O.image_blocks(img, weight_mode=1)
    rgba = torch.from_numpy(np.ascontiguousarray(tex.reshape(-1, 64))).cuda()
    e = ig.evaluate_errors(rgba, out, 0).cpu().numpy()
    sse = e.astype(np.float64).sum()
    assert sse == O.image_sse(img, blocks, 0)
    assert 20 * np.log10(255 / np.sqrt(sse / (16 * blocks.shape[0]))) > 30


def test_launch_shapes_do_not_change_results(gpu_lib):
    """Every launch shape the autotuner may pick gives the same bytes, and
    autotune() applies and reports a valid shape per level."""
    import torch
    ig = gpu_lib
    img = _to_dev(synth.quality_sweep_image(320, 200, seed=4))
    saved = {lv: ig.get_launch_config(lv) for lv in range(10)}
    try:
        for lv in (0, 5, 9):
            ref = ig.compress_image(img, lv, 0, (1, 1, 1), weight_mode=ig.WEIGHTS_ALPHA).cpu().numpy()
            for g, p in ig.TUNE_CANDIDATES:
                for c in (ig.TUNE_CTA_WARPS if lv >= 2 else (0,)):
                    ig.set_launch_config(lv, g, p, c)
                    out = ig.compress_image(img, lv, 0, (1, 1, 1), weight_mode=ig.WEIGHTS_ALPHA).cpu().numpy()
                    assert np.array_equal(out, ref), (lv, g, p, c)
        table = ig.autotune(img, levels=(1, 8), repeats=1)
        for lv in (1, 8):
            t = table[lv]
            assert (t["groups_per_warp"], t["persistent"]) == ig.get_launch_config(lv)[:2]
            assert len(t["candidates"]) == len(ig.TUNE_CANDIDATES) + (len(ig.TUNE_CTA_WARPS) if lv >= 2 else 0)
        assert table[8]["cta_warps"] == ig.get_launch_config(8)[2] in ig.TUNE_CTA_WARPS
        with pytest.raises(ig.IcbcGpuError):
            ig.set_launch_config(8, 2, 0, 12)
    finally:
        for lv, cfg in saved.items():
            ig.set_launch_config(lv, *cfg)


@pytest.mark.parametrize("cta_warps", [8, 16])
def test_cta_wide_search_matches_oracle(gpu_lib, cta_warps):
    """The listed pass with CTA-wide cluster searches (8 or 16 warps moving
    through the encoder together): every block and error equals the
    oracle's, on the hard block mixture (all block kinds, zero weights,
    three-colour black) and the quality-sweep image, with every decoder and a
    partial CTA group at the end of each list.  The images are large enough
    for the CTA-wide pass (two rounds of CTAs over every SM); smaller ones
    take 4-warp CTAs."""
    ig = gpu_lib
    saved = {lv: ig.get_launch_config(lv) for lv in range(10)}
    side = 1700 if cta_warps == 16 else 1200
    try:
        for img, cw in ((synth.hard_mixture_image(side, side - 4, 77), (1, 1, 1)),
                        (synth.quality_sweep_image(side - 2, side, seed=9), (0.299, 0.587, 0.114))):
            dev = _to_dev(img)
            for lv, decs in ((2, (0, 3)), (5, (2, 3)), (8, (1, 2)), (9, (0, 3))):
                g, p, _ = saved[lv]
                ig.set_launch_config(lv, g, p, cta_warps)
                for dec in decs:
                    out, err = ig.compress_image(dev, lv, dec, cw, weight_mode=ig.WEIGHTS_ALPHA, with_errors=True)
                    ob, oe = O.encode_image(img, lv, dec, cw, 1, None, True, True, nthreads=os.cpu_count() or 1)
                    assert np.array_equal(out.cpu().numpy(), ob), (lv, dec)
                    assert same_bits(err.cpu().numpy(), oe), (lv, dec)
    finally:
        for lv, cfg in saved.items():
            ig.set_launch_config(lv, *cfg)


@pytest.mark.parametrize("cta_warps", [4, 8, 16])
def test_batch_cta_sizes_match_oracle(gpu_lib, cta_warps):
    """The batched form's per-level kernels at each CTA size, in one batch of
    30 images over levels 2-9 (the per-level kernels run side by side, so a
    CTA may serve several rounds, the last with warps that drew no task).
    CTA rounds take consecutive tasks, which may mix images with different
    decoders, colour weights and flags (the round then searches per warp).
    Every image's blocks and errors equal the oracle's, on three replays."""
    import torch
    ig = gpu_lib
    saved = {lv: ig.get_batch_cta_warps(lv) for lv in range(2, 10)}
    try:
        for lv in range(2, 10):
            ig.set_batch_cta_warps(lv, cta_warps)
        rng = np.random.default_rng(23)
        cases = []
        for i in range(30):
            w, h = int(rng.integers(5, 170)), int(rng.integers(5, 170))
            img = synth.hard_mixture_image(w, h, seed=500 + i) if i % 2 else synth.quality_sweep_image(w, h, seed=i)
            cases.append(dict(img=img, level=int(rng.integers(2, 10)), decoder=int(rng.integers(0, 4)),
                              cw=(1.0, 1.0, 1.0) if i % 3 else (0.299, 0.587, 0.114), tcm=bool(i % 4), tcb=bool(i % 5)))
        descs, outs, errs = [], [], []
        for c in cases:
            c["dev"] = _to_dev(c["img"])
            c["oracle"] = O.encode_image(c["img"], c["level"], c["decoder"], c["cw"], 1, None, c["tcm"], c["tcb"],
                                         nthreads=8)
            nb = ig.blocks_of(c["img"].shape[1], c["img"].shape[0])
            outs.append(torch.zeros((nb, 8), dtype=torch.uint8, device="cuda"))
            errs.append(torch.zeros(nb, dtype=torch.float32, device="cuda"))
            descs.append(ig.image_desc(c["dev"], c["level"], outs[-1], errs[-1], c["decoder"], c["cw"],
                                       ig.WEIGHTS_ALPHA, None, c["tcm"], c["tcb"]))
        batch = ig.Batch(descs)
        for _ in range(3):
            for o, e in zip(outs, errs):
                o.zero_()
                e.zero_()
            batch.launch()
            torch.cuda.synchronize()
            for c, out, err in zip(cases, outs, errs):
                ob, oe = c["oracle"]
                assert np.array_equal(out.cpu().numpy(), ob), (c["level"], c["decoder"])
                assert same_bits(err.cpu().numpy(), oe), (c["level"], c["decoder"])
        batch.close()
        if cta_warps == 16:
            table = ig.autotune_batch(descs, repeats=1)
            assert table["batch_cta_warps"] in ig.TUNE_CTA_WARPS
            assert all(ig.get_batch_cta_warps(lv) == table["batch_cta_warps"] for lv in range(2, 10))
    finally:
        for lv, c in saved.items():
            ig.set_batch_cta_warps(lv, c)
