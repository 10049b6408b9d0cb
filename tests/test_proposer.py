"""The learned step proposer: its kernels against the CPU reference
(oracle/mlp_oracle.py), its features against the state they come from.

Tolerances: gradients and forward values are FP32 sums of FP32 products of
BF16 weights against the FP64 reference on the same BF16 values: 2e-4 of the
largest gradient entry, 1e-5 relative for the loss and the predictions.
Features are FP32 from the truncated FP64 state: 2e-4 relative.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from oracle import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def test_mlp_gradient_matches_oracle(rg):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    p = rng.normal(0, 0.3, mo.NPARAM).astype(np.float32)
    bits = mo.bf16_bits(p)
    n = 100                                   # not a multiple of the 16-row tile
    xn = rng.normal(0, 1, (n, mo.NFEAT)).astype(np.float32)
    tn = rng.normal(0, 1, n).astype(np.float32)
    w = dev(torch, bits.view(np.int16))
    grad = torch.zeros(mo.NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    X, T = dev(torch, xn), dev(torch, tn)
    rg.lib.mlp_grad(w.data_ptr(), X.data_ptr(), T.data_ptr(), n, grad.data_ptr(), loss.data_ptr())
    torch.cuda.synchronize()
    ref_loss, ref = mo.loss_and_grad(mo.bf16_value(bits), xn, tn)
    g = grad.cpu().numpy()
    assert abs(loss.item() - ref_loss) <= 1e-5 * ref_loss
    assert np.abs(g - ref).max() <= 2e-4 * np.abs(ref).max()
    g2 = torch.zeros_like(grad)                # deterministic: the same bits again
    rg.lib.mlp_grad(w.data_ptr(), X.data_ptr(), T.data_ptr(), n, g2.data_ptr(), loss.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(grad, g2)


def test_mlp_predict_matches_oracle(rg):
    pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    p = rng.normal(0, 0.3, mo.NPARAM).astype(np.float32)
    bits = mo.bf16_bits(p)
    x = rng.normal(3, 2, (77, mo.NFEAT)).astype(np.float32)
    nm = rg.lib.MlpNorm()
    for c in range(mo.NFEAT):
        nm.x_mean[c] = 3.0 + 0.1 * c
        nm.x_std[c] = 2.0
    nm.y_mean, nm.y_std = -1.5, 0.7
    got = rg.proposer.predict(bits, nm, x)
    xn = (x.astype(np.float64) - np.array(nm.x_mean, np.float64)) / np.array(nm.x_std, np.float64)
    y, _ = mo.forward(mo.bf16_value(bits), xn)
    ref = y * nm.y_std + nm.y_mean
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-5)


def test_adam_matches_oracle(rg):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    master = rng.normal(0, 0.3, mo.NPARAM).astype(np.float32)
    m = rng.normal(0, 1e-2, mo.NPARAM).astype(np.float32)
    v = rng.uniform(0, 1e-3, mo.NPARAM).astype(np.float32)
    g = rng.normal(0, 1e-2, mo.NPARAM).astype(np.float32)
    M, Mm, Mv, G = dev(torch, master), dev(torch, m), dev(torch, v), dev(torch, g)
    W = torch.zeros(mo.NPARAM, dtype=torch.int16, device="cuda")
    rg.lib.mlp_adam(M.data_ptr(), W.data_ptr(), Mm.data_ptr(), Mv.data_ptr(), G.data_ptr(), 3, 1e-3)
    torch.cuda.synchronize()
    rm, rmm, rv, rbits = mo.adam(master.astype(np.float64), m.astype(np.float64), v.astype(np.float64),
                                 g.astype(np.float64), 3, 1e-3)
    assert np.allclose(M.cpu().numpy(), rm, rtol=1e-5, atol=1e-7)
    assert np.allclose(Mm.cpu().numpy(), rmm, rtol=1e-5, atol=1e-9)
    bits = W.cpu().numpy().view(np.uint16)
    assert np.abs(mo.bf16_value(bits) - mo.bf16_value(rbits)).max() <= 2.0 ** -7 * np.abs(rm).max()


def features_np(s, dt_did, acc0):
    """The proposer's features 0, 2 .. 11 of System s (numpy, FP64)."""
    n_star = int(s.playing[0])
    n_si = int(sum(s.playing[:4]))
    r = np.stack([s.r["x"], s.r["y"], s.r["z"]], 1)
    v = np.stack([s.v["x"], s.v["y"], s.v["z"]], 1)
    ms = s.p["mass"][0]
    sel = (s.md["id"] >= 0) & (np.arange(s.n) >= n_star)
    rr, vv, mm = r[sel], v[sel], s.p["mass"][sel]
    mu = ms + mm
    rn = np.linalg.norm(rr, axis=1)
    h = np.cross(rr, vv)
    ev = np.cross(vv, h) / mu[:, None] - rr / rn[:, None]
    e = np.linalg.norm(ev, axis=1)
    inc = np.arccos(np.clip(h[:, 2] / np.linalg.norm(h, axis=1), -1, 1))
    vr = np.sqrt(np.sum(vv * vv, 1) * rn / mu)
    amax = np.linalg.norm(acc0[sel], axis=1).max()
    dmin = np.inf
    idx = np.nonzero(sel)[0]
    for k in range(n_star, n_si):
        rh = np.linalg.norm(r[k]) * (s.p["mass"][k] / (3 * ms)) ** (1 / 3)
        d = np.linalg.norm(r[idx] - r[k], axis=1)[idx != k]
        dmin = min(dmin, (d / rh).min())
    f = np.zeros(12)
    f[0] = np.log(abs(dt_did))
    f[2] = np.log(dmin)
    f[3] = np.log(amax)
    f[4] = vr.max()
    f[5] = np.log(sel.sum())
    f[6], f[7], f[8] = e.mean(), np.sqrt((e * e).mean()), e.max()
    f[9], f[10], f[11] = inc.mean(), np.sqrt((inc * inc).mean()), inc.max()
    return f


def test_features_match_the_state(rg):
    s = rg.ic.config4_system(3, n_min=300, n_max=400)
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K) as sim:
        a0 = sim.calc_dydx(0, 1, 0.0)
        acc0 = np.stack([a0["x"], a0["y"], a0["z"]], 1)
        sim.log_features(1024)
        dt1 = sim.step()
        st = sim.get_state(0)
        dt2 = sim.step()
        recs = sim.feature_log(cap=64)
    assert len(recs) == 1
    f = recs[0]
    ref = features_np(st, dt1, acc0)
    keep = [0, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11]
    assert np.allclose(f[keep], ref[keep], rtol=2e-4, atol=2e-5), (f[keep], ref[keep])
    assert f[1] <= 0.0                              # the accepted step's error was within tolerance
    assert f[12] == pytest.approx(np.log(abs(dt2)), rel=1e-6)
    assert f[13] <= 0.0                             # log(err / tol) of the second accepted step


def test_trained_proposer_reduces_rejected_tries(rg):
    """What the network gains over the classical controller: trained on the
    feature log of plain runs of an ensemble of 64 disks (N ~ U[128, 512],
    2-8 protoplanets, RKF7(8) at tolerance 1e-10), it cuts the rejected tries
    of the same ensemble while simulated time and |dE/E| stay those of the plain
    run.  Training and the kernels are deterministic (seeded permutations,
    fixed-order reductions), so the figures are reproducible."""
    pytest.importorskip("torch")
    systems = [rg.ic.config4_system(i, n_min=128, n_max=512) for i in range(64)]
    kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K, precision="mixed")

    def run(proposer=None, log=False):
        with rg.Sim(systems, **kw) as sim:
            if log:
                sim.log_features(1 << 20)
            if proposer is not None:
                sim.set_step_proposer(*proposer, safety=1.0, ratio_lo=0.25, ratio_hi=4.0)
            e0 = np.array([sim.energy_interacting(k)[0] for k in range(len(systems))])
            for _ in range(10):
                sim.launch_tries(200)
                sim.synchronize()
            infos = [sim.info(k) for k in range(len(systems))]
            e1 = np.array([sim.energy_interacting(k)[0] for k in range(len(systems))])
            recs = sim.feature_log(cap=1 << 20) if log else None
        return (sum(i.n_failed for i in infos), sum(i.n_tried for i in infos), sum(i.t for i in infos),
                float(np.median(np.abs((e1 - e0) / e0))), recs)

    f0, n0, t0, de0, recs = run(log=True)
    assert len(recs) > 100000
    bits, nm, hist = rg.proposer.train(recs, epochs=30, batch=2048, lr=2e-3)
    assert hist[-1][2] < 0.2 * hist[0][2] or hist[-1][2] < 0.01      # validation loss fell
    f1, n1, t1, de1, _ = run(proposer=(bits, nm))
    assert abs(n1 - n0) <= 0.001 * n0            # the same number of tries (a system may stop early)
    assert f1 <= 0.9 * f0, (f0, f1)             # fewer rejected tries
    assert t1 >= 0.99 * t0, (t0, t1)            # at no loss of simulated time
    assert de1 <= 1.2 * de0 + 1e-12, (de0, de1)  # and no loss of accuracy
