"""GPU: the batched entry point that allocates nothing.

icbc_gpu_compress_bc1_images_noalloc serves callers that may not allocate
device memory -- an engine that reserves the whole device budget itself,
code running inside such an allocator, or a latency-critical path that cannot
pay for cudaMalloc/cudaFree.  Its work queue lives in a fixed array inside the
library's device code, shared by every call, and keeps the last call's
contents.  These tests call it through the C ABI and require:

* the same bytes and per-block errors as the existing batched entry point
  (icbc_gpu_compress_bc1_images) and as the oracle, on two calls in a row
  where the second has fewer images and fewer blocks than the first, so that
  descriptors or offsets left in the shared array by the first call would
  show in the second;
* uniform, alpha and weight-plane images, explicit decoders and
  ICBC_GPU_DECODER_DEFAULT, and a batch of exactly the maximum size;
* no change in the device's free memory or in torch's allocations across
  calls after the first;
* a batch beyond the maximum refused before any device work.

The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

import icbc_gb300 as ig
from icbc_gb300 import synth

pytestmark = pytest.mark.gpu

CW = (1.0, 0.8, 0.6)


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _items(torch, specs, mixed_weights=True):
    """Device images (with weight planes where the mode asks) and two sets of
    zeroed outputs + error buffers per image."""
    items = []
    for i, s in enumerate(specs):
        img = synth.gradient_noise_rects(s.width, s.height, s.seed)
        wm = i % 3 if mixed_weights else ig.WEIGHTS_UNIFORM
        if wm == ig.WEIGHTS_ALPHA:
            img[:, :, 3] = synth.quality_sweep_image(s.width, s.height, seed=s.seed)[:, :, 3]
        plane = None
        if wm == ig.WEIGHTS_PLANE:
            plane = (synth.uniform(s.seed, 5, (s.height, s.width)) * 2.0).astype(np.float32)
        nb = ig.blocks_of(s.width, s.height)
        items.append(dict(
            spec=s, img=img, wm=wm, plane=plane, d_img=torch.from_numpy(img).cuda(),
            d_plane=None if plane is None else torch.from_numpy(plane).cuda(),
            outs=[torch.zeros((nb, 8), dtype=torch.uint8, device="cuda") for _ in range(2)],
            errs=[torch.zeros(nb, dtype=torch.float32, device="cuda") for _ in range(2)]))
    return items


def _descs(items, k, decoder=None):
    descs = [ig.image_desc(it["d_img"], it["spec"].level, it["outs"][k], it["errs"][k],
                           it["spec"].decoder if decoder is None else decoder, CW, it["wm"], it["d_plane"])
             for it in items]
    return (ig.ImageDesc * len(descs))(*descs)


def _stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _same(items, what):
    for it in items:
        s = it["spec"]
        a, b = it["outs"][0].cpu().numpy(), it["outs"][1].cpu().numpy()
        assert np.array_equal(a, b), (what, s.width, s.height, s.level, s.decoder, it["wm"])
        ea, eb = it["errs"][0].cpu().numpy(), it["errs"][1].cpu().numpy()
        assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32)), (what, s.level, it["wm"])


def test_noalloc_two_calls_match_batched_and_oracle():
    torch = _torch()
    from oracle import oracle as O
    lib = ig.load()
    stream = _stream(torch)
    # First call: 24 images; second: 9 smaller ones (fewer images and blocks),
    # so a stale descriptor, offset or task count from the first would show.
    for call, (n, seed, hi) in enumerate(((24, 31, 260), (9, 32, 90))):
        items = _items(torch, synth.batch_specs(n, seed=seed, lo=8, hi=hi))
        # Explicit decoders: the allocation-free call needs no icbc_gpu_init.
        assert lib.icbc_gpu_compress_bc1_images_noalloc(_descs(items, 0), len(items), stream) == 0, call
        ig.init(ig.Decoder_D3D10)  # the existing batched entry point uses the init-time tables
        assert lib.icbc_gpu_compress_bc1_images(_descs(items, 1), len(items), stream) == 0
        torch.cuda.synchronize()
        _same(items, "call %d" % call)
        for it in items[::2] if call == 0 else items:
            s = it["spec"]
            ob, oe = O.encode_image(it["img"], s.level, s.decoder, CW, it["wm"], it["plane"], True, True, nthreads=8)
            assert np.array_equal(it["outs"][0].cpu().numpy(), ob), ("oracle", call, s.level, it["wm"])
            assert np.array_equal(it["errs"][0].cpu().numpy().view(np.uint32), oe.view(np.uint32))


def test_noalloc_default_decoder_and_full_batch():
    torch = _torch()
    lib = ig.load()
    stream = _stream(torch)
    # ICBC_GPU_DECODER_DEFAULT resolves to the decoder icbc_gpu_init selected.
    ig.init(ig.Decoder_NVIDIA)
    try:
        items = _items(torch, synth.batch_specs(12, seed=33, lo=8, hi=130))
        assert lib.icbc_gpu_compress_bc1_images_noalloc(_descs(items, 0, ig.DECODER_DEFAULT), len(items),
                                                         stream) == 0
        assert lib.icbc_gpu_compress_bc1_images(_descs(items, 1, ig.Decoder_NVIDIA), len(items), stream) == 0
        torch.cuda.synchronize()
        _same(items, "default decoder")
    finally:
        ig.init(ig.Decoder_D3D10)
    # Exactly the maximum batch of small images.
    items = _items(torch, synth.batch_specs(ig.NOALLOC_MAX_IMAGES, seed=34, lo=4, hi=40))
    assert lib.icbc_gpu_compress_bc1_images_noalloc(_descs(items, 0), len(items), stream) == 0
    assert lib.icbc_gpu_compress_bc1_images(_descs(items, 1), len(items), stream) == 0
    torch.cuda.synchronize()
    _same(items, "full batch")


def test_noalloc_allocates_nothing_after_first_call():
    torch = _torch()
    lib = ig.load()
    stream = _stream(torch)
    batches = [_items(torch, synth.batch_specs(n, seed=40 + n, lo=8, hi=200)) for n in (20, 7, 33)]
    arrays = [_descs(items, 0) for items in batches]
    assert lib.icbc_gpu_compress_bc1_images_noalloc(arrays[0], len(batches[0]), stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    torch0 = torch.cuda.memory_allocated()
    for rep in range(2):
        for arr, items in zip(arrays, batches):
            assert lib.icbc_gpu_compress_bc1_images_noalloc(arr, len(items), stream) == 0, rep
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == torch0
    # A batch beyond the stated maximum is refused before any device work.
    too_many = (ig.ImageDesc * (ig.NOALLOC_MAX_IMAGES + 1))()
    assert lib.icbc_gpu_compress_bc1_images_noalloc(too_many, ig.NOALLOC_MAX_IMAGES + 1, stream) == 1
