"""The proposer network's CPU reference (oracle/mlp_oracle.py) against
finite differences, and its BF16 rounding against known bit patterns.  red.cuda
has no learned component, so the reference is pinned by the mathematics:
central differences of the FP64 loss agree with the analytic gradient to
1e-6 relative."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from oracle import mlp_oracle as mo  # noqa: E402


def test_bf16_rounding_known_values():
    x = np.array([1.0, -2.5, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, 3.0e38], np.float32)
    bits = mo.bf16_bits(x)
    assert bits[0] == 0x3F80 and bits[1] == 0xC020
    assert bits[2] == 0x3F80          # 1 + 2^-8 is half way: ties to even
    assert bits[3] == 0x3F81          # 1 + 3 * 2^-9 rounds up to 1 + 2^-7
    assert np.isfinite(mo.bf16_value(bits)).all()


def test_gradient_matches_central_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0, 0.3, mo.NPARAM)
    xn = rng.normal(0, 1, (37, mo.NFEAT))
    tn = rng.normal(0, 1, 37)
    loss, g = mo.loss_and_grad(p, xn, tn)
    idx = rng.choice(mo.NPARAM, 60, replace=False)
    idx = np.concatenate([idx, [mo.O_B3, mo.O_W3, mo.O_B1, mo.O_W2 + 5]])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mo.loss_and_grad(pp, xn, tn)[0] - mo.loss_and_grad(pm, xn, tn)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, (k, fd, g[k])
    assert loss > 0


def test_adam_reduces_loss():
    rng = np.random.default_rng(4)
    p = rng.normal(0, 0.3, mo.NPARAM)
    xn = rng.normal(0, 1, (64, mo.NFEAT))
    tn = np.tanh(xn[:, 0]) + 0.1 * xn[:, 1]
    m = np.zeros(mo.NPARAM)
    v = np.zeros(mo.NPARAM)
    l0 = mo.loss_and_grad(p, xn, tn)[0]
    for step in range(1, 51):
        _, g = mo.loss_and_grad(p, xn, tn)
        p, m, v, _ = mo.adam(p, m, v, g, step, 1e-2)
    assert mo.loss_and_grad(p, xn, tn)[0] < 0.5 * l0
