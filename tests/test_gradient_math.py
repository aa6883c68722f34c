"""CPU: the FP64 analytic gradient used by the GPU autograd tests,
2 F^H (w * F x), against FP64 central finite differences on 64 random
coordinates (the differentiation workload's check)."""
import numpy as np

import oracle


def loss(x, w):
    X = oracle.fft_1d(x)
    return float(np.sum(w * np.abs(X) ** 2))


def test_analytic_gradient_matches_central_differences():
    rng = np.random.default_rng(3)
    batch, n = 4, 256
    x = rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))
    w = rng.uniform(0, 1, (batch, n))
    g = oracle.fft_1d(2 * w * oracle.fft_1d(x), sign=+1)  # F^H (2 w F x)
    h = 1e-6
    for _ in range(64):
        b, i = rng.integers(batch), rng.integers(n)
        for comp, unit in ((0, 1.0), (1, 1j)):
            xp = x.copy()
            xp[b, i] += h * unit
            xm = x.copy()
            xm[b, i] -= h * unit
            fd = (loss(xp, w) - loss(xm, w)) / (2 * h)
            an = g[b, i].real if comp == 0 else g[b, i].imag
            assert abs(fd - an) < 1e-5 * max(1.0, abs(an)), (b, i, comp, fd, an)
