"""CPU: the seeded workload generators are deterministic and have the
configured shapes and mixtures."""
import numpy as np

from icbc_gb300 import synth


def test_generators_deterministic():
    a = synth.gradient_noise_rects(96, 64, 4)
    b = synth.gradient_noise_rects(96, 64, 4)
    assert a.shape == (64, 96, 4) and np.array_equal(a, b)
    assert (a[..., 3] == 255).all()
    c = synth.hard_mixture_image(67, 33, 2)
    assert c.shape == (33, 67, 4)
    z = (c[..., 3] == 0).mean()
    assert 0.15 < z < 0.35


def test_batch_specs():
    specs = synth.batch_specs(2000, seed=7)
    assert len(specs) == 2000
    w = np.array([s.width for s in specs])
    h = np.array([s.height for s in specs])
    assert w.min() >= 64 and w.max() <= 2048 and h.min() >= 64 and h.max() <= 2048
    odd = np.mean((w % 4 != 0) | (h % 4 != 0))
    assert 0.03 < odd < 0.15
    assert set(s.level for s in specs) == set(range(10))
    assert set(s.decoder for s in specs) == {0, 1, 2}


def test_serving_requests():
    reqs = synth.serving_requests(5000, 1000.0, seed=3)
    t = np.array([r.arrival_s for r in reqs])
    assert np.all(np.diff(t) > 0)
    rate = len(t) / t[-1]
    assert 900 < rate < 1100
    sides = np.array([r.side for r in reqs])
    assert abs(np.mean(sides == 64) - 0.30) < 0.03
