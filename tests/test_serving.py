"""GPU: the serving form.  Requests of different sizes and levels arrive
while others run; each result must be byte-identical to encoding the same
image alone (plain single-image launch), whether the request ran alone or in
the mix.  Admission, back-pressure, rejection and cancellation are checked
on the host side of the same server."""
import time

import numpy as np
import pytest

import icbc_gb300 as ig
from icbc_gb300 import synth

pytestmark = pytest.mark.gpu

SIDES = (8, 20, 64, 100, 128, 256)


def _requests(n, seed):
    rng = synth.uniform(seed, 0, (n, 4))
    base = synth.gradient_noise_rects(256, 256, seed)
    reqs = []
    for i in range(n):
        w = SIDES[int(rng[i, 0] * len(SIDES))]
        h = SIDES[int(rng[i, 1] * len(SIDES))]
        img = np.ascontiguousarray(base[:h, :w])
        reqs.append((img, int(rng[i, 2] * 10), int(rng[i, 3] * 3)))
    return reqs


def _plain(img, level, decoder):
    import torch
    out = ig.compress_image(torch.from_numpy(img).cuda(), level, decoder)
    return out.cpu().numpy()


def test_alone_equals_mix_equals_plain(gpu_lib):
    reqs = _requests(40, 3)
    srv = ig.Server(64 << 20, max_inflight=2, max_batch_images=16)
    try:
        alone = []
        for img, lv, dec in reqs[:12]:
            rid = srv.submit(img, lv, dec)
            assert srv.wait(rid, 20000) == 0
            alone.append(srv.result(rid)[0].copy())
        ids = [srv.submit(img, lv, dec) for img, lv, dec in reqs]          # all at once: mixed batches
        for rid in ids:
            assert srv.wait(rid, 20000) == 0
        for k, ((img, lv, dec), rid) in enumerate(zip(reqs, ids)):
            mix = srv.result(rid)[0]
            ref = _plain(img, lv, dec)
            assert np.array_equal(mix, ref), (img.shape, lv, dec)
            if k < 12:
                assert np.array_equal(alone[k], ref)
        st = srv.stats()
        assert st["completed"] == 52 and st["failed"] == 0
        assert st["latency_p99_ms"] >= st["latency_p50_ms"] > 0
    finally:
        srv.close()


def test_heavy_and_light_requests(gpu_lib):
    """Heavy requests (1024^2 at levels 7-9: over 0.2 ms of GPU time each,
    and more tasks than the GPU has CTA slots, so their launches take three
    quarters of the slots) and light ones submitted together: they go to
    separate launches, light first and in turn, and every result equals the
    plain encode."""
    big = synth.gradient_noise_rects(1024, 1024, 17)
    heavy = [(np.ascontiguousarray(np.roll(big, 64 * k, axis=1)), 7 + k % 3, k % 3) for k in range(4)]
    light = _requests(30, 5)
    order = light[:10] + heavy[:2] + light[10:20] + heavy[2:] + light[20:]
    srv = ig.Server(1 << 30, max_inflight=8, max_batch_images=64)
    try:
        ids = [srv.submit(img, lv, dec) for img, lv, dec in order]
        for rid in ids:
            assert srv.wait(rid, 60000) == 0
        for (img, lv, dec), rid in zip(order, ids):
            assert np.array_equal(srv.result(rid)[0], _plain(img, lv, dec)), (img.shape, lv, dec)
        st = srv.stats()
        assert st["completed"] == len(order) and st["failed"] == 0
        assert st["batches"] >= 2  # the heavy ones never share the light ones' launch
    finally:
        srv.close()


def test_two_pass_edge_requests(gpu_lib):
    """Launches finish the blocks of 0 or 1 reduced colours of level-2..9
    requests first and list the rest: flat requests (empty lists), noise
    (every block listed) and ragged sizes at every level, in one mix, equal
    the plain launches."""
    rng = np.random.default_rng(31)
    imgs = [np.full((20, 36, 4), 90, np.uint8), rng.integers(0, 256, (28, 20, 4), dtype=np.uint8),
            synth.quality_sweep_image(37, 29, seed=4), np.full((1, 1, 4), 3, np.uint8)]
    reqs = [(imgs[i % 4], i % 10, i % 3) for i in range(40)]
    srv = ig.Server(64 << 20, max_inflight=2, max_batch_images=24)
    try:
        ids = [srv.submit(img, lv, dec) for img, lv, dec in reqs]
        for rid in ids:
            assert srv.wait(rid, 20000) == 0
        for (img, lv, dec), rid in zip(reqs, ids):
            assert np.array_equal(srv.result(rid)[0], _plain(img, lv, dec)), (img.shape, lv, dec)
    finally:
        srv.close()


def test_budget_backpressure_and_rejection(gpu_lib):
    budget = 1 << 20  # 1 MiB: only a few small requests fit at once
    srv = ig.Server(budget, max_inflight=2, max_batch_images=8)
    try:
        big = np.zeros((1024, 1024, 4), np.uint8)
        with pytest.raises(ig.IcbcGpuError) as exc:
            srv.submit(big, 1)
        assert exc.value.status == 6  # ICBC_GPU_ERR_BUDGET
        reqs = _requests(30, 5)
        ids = [srv.submit(img, lv, dec) for img, lv, dec in reqs]
        for rid in ids:
            assert srv.wait(rid, 30000) == 0
        st = srv.stats()
        assert st["rejected"] == 1 and st["completed"] == 30
        assert 0 < st["arena_peak"] <= st["arena_bytes"] <= budget + 4096
        for (img, lv, dec), rid in zip(reqs, ids):
            assert np.array_equal(srv.result(rid)[0], _plain(img, lv, dec))
    finally:
        srv.close()


def test_cancel_and_shutdown(gpu_lib):
    srv = ig.Server(256 << 10, max_inflight=1, max_batch_images=1)
    img = synth.gradient_noise_rects(200, 200, 9)
    ids = [srv.submit(img, 9, 0) for _ in range(12)]
    last = ids[-1]
    assert srv.cancel(last) in (0, 7)          # cancelled while queued, or already on the GPU
    status = srv.wait(last, 30000)
    assert status in (0, 8)
    assert srv.poll(10 ** 9) == 9              # unknown id
    srv.close()                                 # the rest finish or are cancelled, no hang
    assert srv._h is None
