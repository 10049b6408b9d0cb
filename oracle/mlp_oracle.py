"""CPU reference of the learned step proposer's network (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the checker that the CUDA kernels of the proposer
(red.cuda_gb300/csrc/proposer.cu) are compared against.  Only tests/ load it;
the product path never does.

The network is 12 -> 64 -> 64 -> 1 with SiLU activations; the parameters are
flat: W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3 (5057 values), used
as their BF16-rounded values.  The loss over n rows is
    L = sum_r (y_r - t_r)^2 / (2 n)
on normalised features and targets.  Adam follows Kingma & Ba (2015) with the
bias corrections 1 - beta^step.  red.cuda has no learned component; this
reference is pinned against finite differences (tests/test_mlp_oracle.py).
"""
import numpy as np

NFEAT, NHID = 12, 64
O_W1 = 0
O_B1 = O_W1 + NHID * NFEAT
O_W2 = O_B1 + NHID
O_B2 = O_W2 + NHID * NHID
O_W3 = O_B2 + NHID
O_B3 = O_W3 + NHID
NPARAM = O_B3 + 1


def bf16_bits(x):
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_value(bits):
    """BF16 bit patterns -> float64 values."""
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[O_W1:O_B1].reshape(NHID, NFEAT), p[O_B1:O_W2], p[O_W2:O_B2].reshape(NHID, NHID), p[O_B2:O_W3],
            p[O_W3:O_B3], p[O_B3])


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, xn):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    z1 = xn @ W1.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    return h2 @ w3 + b3, (z1, h1, z2, h2)


def loss_and_grad(p, xn, tn):
    """Loss and its gradient with respect to the flat parameters p."""
    xn = np.asarray(xn, np.float64)
    tn = np.asarray(tn, np.float64)
    n = len(tn)
    W1, b1, W2, b2, w3, b3 = unpack(p)
    y, (z1, h1, z2, h2) = forward(p, xn)
    e = y - tn
    loss = float(np.sum(e * e) / (2.0 * n))
    dy = e / n
    g = np.zeros(NPARAM)
    g[O_W3:O_B3] = h2.T @ dy
    g[O_B3] = dy.sum()
    dz2 = np.outer(dy, w3) * silu_grad(z2)
    g[O_W2:O_B2] = (dz2.T @ h1).reshape(-1)
    g[O_B2:O_W3] = dz2.sum(axis=0)
    dz1 = (dz2 @ W2) * silu_grad(z1)
    g[O_W1:O_B1] = (dz1.T @ xn).reshape(-1)
    g[O_B1:O_W2] = dz1.sum(axis=0)
    return loss, g


def adam(master, m, v, grad, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step; returns (master, m, v, bf16 bits of master)."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    c1 = 1 - beta1 ** step
    c2 = 1 - beta2 ** step
    master = master - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return master, m, v, bf16_bits(master.astype(np.float32))
