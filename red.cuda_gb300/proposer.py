"""Training of the learned step proposer on the GPU.

The network (12 -> 64 -> 64 -> 1, SiLU, BF16 weights, FP32 accumulation) and
its forward, backward and Adam kernels live in libredgb (proposer.cu); this
module only moves the data: it standardises the logged (features, log|dt|,
log(err / tol)) records, keeps the parameters, the Adam moments and the batches in device
memory (torch tensors as plain buffers) and calls red_mlp_grad /
red_mlp_adam for every batch.  Records come from Sim.log_features /
Sim.feature_log on plain runs of the integrator.
"""
import numpy as np

from . import lib

NFEAT = lib.MLP_NFEAT
NHID = 64
# flat parameter layout: W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3
O_W1 = 0
O_B1 = O_W1 + NHID * NFEAT
O_W2 = O_B1 + NHID
O_B2 = O_W2 + NHID * NHID
O_W3 = O_B2 + NHID
O_B3 = O_W3 + NHID


def bf16_bits(x):
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def init_params(seed=0):
    """He-uniform weights, zero biases."""
    rng = np.random.default_rng(seed)
    p = np.zeros(lib.mlp_param_count(), np.float32)
    p[O_W1:O_B1] = rng.uniform(-1, 1, O_B1 - O_W1) * np.sqrt(6.0 / NFEAT)
    p[O_W2:O_B2] = rng.uniform(-1, 1, O_B2 - O_W2) * np.sqrt(6.0 / NHID)
    p[O_W3:O_B3] = rng.uniform(-1, 1, O_B3 - O_W3) * np.sqrt(3.0 / NHID)
    return p


def records_xt(records, target="accepted", order=7):
    """Inputs and targets of logged records (n, 14): the 12 features and either
    the log|dt| of the step accepted next ("accepted": the network imitates
    the classical controller's outcome) or the log of the largest step that
    would have met the tolerance there ("largest": log|dt| - log(err/tol) / order,
    the correction clipped to a factor 4 either way), so that safety * exp(y)
    aims just inside the tolerance."""
    x = records[:, :NFEAT]
    t = records[:, NFEAT].astype(np.float64)
    if target == "largest":
        t = t + np.clip(-records[:, NFEAT + 1].astype(np.float64) / order, -np.log(4.0), np.log(4.0))
    elif target != "accepted":
        raise ValueError("unknown target " + target)
    return x, t


def make_norm(x, t):
    """red_mlp_norm_t from features x (n, 12) and targets t (n,)."""
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    nm = lib.MlpNorm()
    mu = x.mean(axis=0)
    sd = np.maximum(x.std(axis=0), 1e-3)
    for c in range(NFEAT):
        nm.x_mean[c] = float(mu[c])
        nm.x_std[c] = float(sd[c])
    nm.y_mean = float(t.mean())
    nm.y_std = float(max(t.std(), 1e-3))
    return nm


def normalise(x, t, nm):
    x = (np.asarray(x, np.float32) - np.array(nm.x_mean, np.float32)) / np.array(nm.x_std, np.float32)
    t = (np.asarray(t, np.float32) - np.float32(nm.y_mean)) / np.float32(nm.y_std)
    return np.ascontiguousarray(x, np.float32), np.ascontiguousarray(t, np.float32)


def train(records, epochs=30, batch=2048, lr=2e-3, seed=0, val_frac=0.1, device="cuda", target="accepted",
          order=7):
    """Trains on the GPU; returns (BF16 weights as uint16, MlpNorm, history of
    (epoch, train loss, validation loss)).  `target`: see records_xt."""
    import torch
    records = np.asarray(records, np.float32)
    records = records[np.isfinite(records).all(axis=1)]
    # the device appends records in atomic order: sort them so that the split and
    # the batches, and so the trained network, depend only on the records
    records = records[np.lexsort(records.T[::-1])]
    if len(records) < 64:
        raise ValueError("too few records to train on: %d" % len(records))
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(records))
    n_val = max(16, int(val_frac * len(records)))
    val, tr = records[perm[:n_val]], records[perm[n_val:]]
    nm = make_norm(*records_xt(tr, target, order))
    xtr, ttr = normalise(*records_xt(tr, target, order), nm)
    xval, tval = normalise(*records_xt(val, target, order), nm)
    dev = torch.device(device)
    X = torch.from_numpy(xtr).to(dev)
    T = torch.from_numpy(ttr).to(dev)
    Xv = torch.from_numpy(xval).to(dev)
    Tv = torch.from_numpy(tval).to(dev)
    p0 = init_params(seed)
    master = torch.from_numpy(p0).to(dev)
    w = torch.from_numpy(bf16_bits(p0).view(np.int16)).to(dev)   # BF16 bits
    m = torch.zeros_like(master)
    v = torch.zeros_like(master)
    grad = torch.zeros_like(master)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    vloss = torch.zeros(1, dtype=torch.float32, device=dev)
    gv = torch.zeros_like(master)
    stream = torch.cuda.current_stream(dev).cuda_stream
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    history = []
    step = 0
    n = X.shape[0]
    for ep in range(epochs):
        order = torch.randperm(n, generator=gen, device=dev)
        tot = torch.zeros(1, dtype=torch.float32, device=dev)
        nb = 0
        for b0 in range(0, n, batch):
            idx = order[b0:b0 + batch]
            xb = X.index_select(0, idx).contiguous()
            tb = T.index_select(0, idx).contiguous()
            lib.mlp_grad(w.data_ptr(), xb.data_ptr(), tb.data_ptr(), xb.shape[0], grad.data_ptr(), loss.data_ptr(),
                         stream)
            step += 1
            lib.mlp_adam(master.data_ptr(), w.data_ptr(), m.data_ptr(), v.data_ptr(), grad.data_ptr(), step, lr,
                         stream=stream)
            tot += loss
            nb += 1
        lib.mlp_grad(w.data_ptr(), Xv.data_ptr(), Tv.data_ptr(), Xv.shape[0], gv.data_ptr(), vloss.data_ptr(), stream)
        history.append((ep, float(tot.item()) / max(nb, 1), float(vloss.item())))
    bits = w.cpu().numpy().view(np.uint16).copy()
    return bits, nm, history


def predict(bits, nm, features, device="cuda"):
    """Predicted log|dt| for rows of raw features (through red_mlp_predict)."""
    import torch
    dev = torch.device(device)
    x = torch.from_numpy(np.ascontiguousarray(features, np.float32)).to(dev)
    w = torch.from_numpy(np.ascontiguousarray(bits, np.uint16).view(np.int16)).to(dev)
    out = torch.zeros(x.shape[0], dtype=torch.float32, device=dev)
    lib.mlp_predict(w.data_ptr(), nm, x.data_ptr(), out.data_ptr(), x.shape[0],
                    torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()
