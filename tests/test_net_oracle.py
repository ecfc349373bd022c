"""The CPU FP64 restatement of the closure network checks itself: its
analytic gradient against central finite differences, and the BF16 rounding
it uses to emulate the GPU storage points."""
from __future__ import annotations

import numpy as np

import net_oracle as NO


def _random_net(rng):
    p = rng.standard_normal(NO.NPARAMS) * 0.3 * NO.mask()
    return p


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(4)
    p = _random_net(rng)
    samples = rng.standard_normal((2, 6, 3, 4, 5))
    norm = (np.array([0.1, -0.2, 0.0, 0.3]), np.array([1.0, 2.0, 0.5, 1.5]), np.array([0.7, 1.3]))
    loss, g = NO.loss_and_grad(p, samples, norm)
    live = np.flatnonzero(NO.mask())
    pick = rng.choice(live, 40, replace=False)
    h = 1e-6
    for i in pick:
        q = p.copy()
        q[i] += h
        lp, _ = NO.loss_and_grad(q, samples, norm)
        q[i] -= 2 * h
        lm, _ = NO.loss_and_grad(q, samples, norm)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])
    # padded channels carry no gradient
    assert np.all(g[NO.mask() == 0] == 0)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -3.0e-5, 65504.0, 1.0 + 3 * 2 ** -9])
    r = NO.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # tie rounds to even
    assert r[2] == 1.0 + 2 ** -7  # nearest of the two neighbours (spacing 2^-7 above 1)
    assert abs(r[3] - x[3]) <= 2 ** -9 * abs(x[3])
    assert r[5] == 1.0 + 2 ** -7  # above the tie rounds up
    # every BF16 value is exactly representable: rounding is idempotent
    assert np.array_equal(NO.bf16(r), r)
