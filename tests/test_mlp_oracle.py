"""The closure network's CPU oracle checked on its own (no GPU): its backward
pass against central finite differences of its forward pass (exact FP64
network, roundings off), and its BF16 rounding against known values."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding_known_values():
    vals = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159265, 65504.0, 1e-3], np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even -> 1; 1 + 1.5*2^-8 rounds up
    expect = np.array([1.0, 1.0, 1.0078125, 1.0078125, -3.140625, 65536.0, 0.00099945068359375])
    np.testing.assert_array_equal(mo.bf16(vals), expect)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 40
    x = np.stack([rng.uniform(-4, 3, n), rng.uniform(-0.2, 0.2, n), rng.uniform(-4, 3, n),
                  rng.uniform(0.98, 1.05, n), np.full(n, 1.3), rng.integers(20, 90, n)], 1).astype(np.float32)
    y = rng.uniform(0.0, 0.1, n)
    norm = np.concatenate([x.mean(0), 1.0 / x.std(0).clip(1e-6), x.min(0), x.max(0)]).astype(np.float32)
    norm[4 + 6] = 1.0
    p = rng.uniform(-0.3, 0.3, mo.NPARAMS)
    _, g = mo.loss_grad(p, norm, x, y, quantize=False)
    idx = np.concatenate([rng.choice(np.arange(s, e), 6, replace=False) for s, e in
                          [(mo.OW1, mo.OB1), (mo.OB1, mo.OW2), (mo.OW2, mo.OB2), (mo.OW3, mo.OB3),
                           (mo.OW4, mo.OB4)]] + [np.array([mo.OB4])])
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (mo.loss_grad(pp, norm, x, y, quantize=False)[0] - mo.loss_grad(pm, norm, x, y, quantize=False)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g).max()), (k, fd, g[k])
