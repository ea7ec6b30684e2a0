"""GPU: the batched entry point that allocates nothing.

icbc_gpu_compress_bc1_images_noalloc serves callers that may not allocate
device memory -- an engine that reserves the whole device budget itself,
code running inside such an allocator, or a latency-critical path that cannot
pay for cudaMalloc/cudaFree.  Its work queue lives in a fixed array inside the
library's device code, shared by every call.  This test calls it through the
C ABI and requires the same bytes and the same per-block errors as the
existing batched entry point (icbc_gpu_compress_bc1_images), on two calls in
a row with different batches, so that state left in the shared array by the
first call would show in the second.  The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

import icbc_gb300 as ig
from icbc_gb300 import synth

pytestmark = pytest.mark.gpu


def _batch(specs, torch):
    """Device images and two sets of zeroed outputs + error buffers."""
    items = []
    for s in specs:
        img = torch.from_numpy(synth.gradient_noise_rects(s.width, s.height, s.seed)).cuda()
        nb = ig.blocks_of(s.width, s.height)
        outs = [torch.zeros((nb, 8), dtype=torch.uint8, device="cuda") for _ in range(2)]
        errs = [torch.zeros(nb, dtype=torch.float32, device="cuda") for _ in range(2)]
        items.append((s, img, outs, errs))
    return items


def test_noalloc_matches_batched_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = ig.load()
    noalloc = lib.icbc_gpu_compress_bc1_images_noalloc
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, seed in enumerate((31, 32)):
        # Explicit decoders: the allocation-free call needs no icbc_gpu_init.
        specs = synth.batch_specs(24, seed=seed, lo=8, hi=260)
        items = _batch(specs, torch)
        descs = [[ig.image_desc(img, s.level, outs[k], errs[k], s.decoder, (1.0, 0.8, 0.6))
                  for s, img, outs, errs in items] for k in range(2)]
        arr0 = (ig.ImageDesc * len(items))(*descs[0])
        assert noalloc(arr0, len(items), stream) == 0, "call %d" % call
        ig.init(ig.Decoder_D3D10)  # the existing batched entry point uses the init-time tables
        arr1 = (ig.ImageDesc * len(items))(*descs[1])
        assert lib.icbc_gpu_compress_bc1_images(arr1, len(items), stream) == 0
        torch.cuda.synchronize()
        for s, _, outs, errs in items:
            a, b = outs[0].cpu().numpy(), outs[1].cpu().numpy()
            assert np.array_equal(a, b), ("call", call, s.width, s.height, s.level, s.decoder)
            ea, eb = errs[0].cpu().numpy(), errs[1].cpu().numpy()
            assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32)), ("call", call, s.level)
    # A batch beyond the stated maximum is refused before any device work.
    too_many = (ig.ImageDesc * 257)()
    assert noalloc(too_many, 257, stream) == 1
