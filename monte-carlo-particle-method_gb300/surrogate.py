"""Training, storage and loading of the learned 2-D Vlasov force.

The network (include/mcpm.h, "learned Vlasov force of a 2-D box") has no
counterpart in the reference.  It is trained on snapshots of the library's
own plain node-grid force (compute_SP_2D, src/FEM.cpp:249-610, restated in
mcpm_lr2d.cu): each snapshot is a random packing-fraction field
    n b(x, y) = nbar + sum_k a_k sin(2 pi (kx x / L0 + ky y / L1) + phi_k),
nbar ~ U[0.15, 0.35], sum |a_k| ~ U[0.05, 0.1], integer wave vectors of norm
1..8, clipped to [0.05, 0.45], sampled with Poisson-like count noise per
cell quadrant; its input is what the particle step feeds the force (nodal
and cell densities) and its target the plain path's corner-potential
differences.  Forward, backward and Adam run in libmcpm's kernels (BF16
tensor cores, FP32 accumulation); device buffers are torch tensors, used only
as memory.

Usage (one GB300; the committed weights were made by exactly this command,
about 10 s of snapshot generation and 70 s of training):
    python monte-carlo-particle-method_gb300/surrogate.py train \
        --snapshots 20000 --epochs 12 --batch 4 --lr 2e-3 --log-every 5000 \
        --out monte-carlo-particle-method_gb300/weights/vlasov2d_sp_256.npz
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import mcpm  # noqa: E402
import workloads as W  # noqa: E402

WEIGHTS = os.path.join(HERE, "weights", "vlasov2d_sp_256.npz")
N_WAVES = 6


def random_fields(rng, n, n_waves=N_WAVES):
    """[n][1 + 4 n_waves] field parameters: nbar, then (a, kx, ky, phi) per
    wave, drawn as workloads.density_field draws them."""
    F = np.zeros((n, 1 + 4 * n_waves))
    for i in range(n):
        F[i, 0] = rng.uniform(0.15, 0.35)
        amp = rng.uniform(0.0, 1.0, n_waves)
        amp *= rng.uniform(0.05, 0.1) / max(amp.sum(), 1e-12)
        for w in range(n_waves):
            while True:
                kx, ky = rng.integers(-8, 9, 2)
                if 1.0 <= math.hypot(kx, ky) <= 8.0:
                    break
            F[i, 1 + 4 * w:5 + 4 * w] = (amp[w], kx, ky, rng.uniform(0.0, 2.0 * math.pi))
    return F


def bench_config(n):
    """The 2-D Enskog-Vlasov box of n x n unit cells at the benchmark's
    particles per cell (16.0M at n = 256), FP32, screened-Poisson force."""
    cfg, _ = W.vlasov_box_2d(n_cells=(n, n), total=int(round(16_000_000 * n * n / 65536)), precision=mcpm.FP32,
                             long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE, particles=False)
    return cfg


def init_params(seed, n_in=11, n_out=4):
    """He-normal weights over the used input channels, zero biases (the same
    layout and draw as the CPU oracle's init_params)."""
    rng = np.random.default_rng(seed)
    Wd, CIN, COUT = 64, 16, 16
    W1 = np.zeros((Wd, 9, CIN), np.float32)
    W1[:, :, :n_in] = rng.normal(0, math.sqrt(2.0 / (9 * n_in)), (Wd, 9, n_in))
    W2 = rng.normal(0, math.sqrt(2.0 / (9 * Wd)), (Wd, 9, Wd)).astype(np.float32)
    W3 = rng.normal(0, math.sqrt(2.0 / (9 * Wd)), (Wd, 9, Wd)).astype(np.float32)
    W4 = np.zeros((COUT, 9, Wd), np.float32)
    W4[:n_out] = rng.normal(0, math.sqrt(1.0 / (9 * Wd)), (n_out, 9, Wd))
    z = np.zeros(Wd, np.float32)
    return np.concatenate([W1.ravel(), z, W2.ravel(), z, W3.ravel(), z, W4.ravel(), np.zeros(COUT, np.float32)])


def kick_error(out, target):
    """Relative L2 error of the kick coefficients (d0, d1 - d0, d2, d3 - d2)
    computed from network outputs against those of the targets, both in the
    same units, arrays [..., 4]."""
    def coef(a):
        a = np.asarray(a, dtype=np.float64)
        return np.stack([a[..., 0], a[..., 1] - a[..., 0], a[..., 2], a[..., 3] - a[..., 2]], axis=-1)
    c, t = coef(out), coef(target)
    return float(np.sqrt(((c - t) ** 2).sum() / max((t ** 2).sum(), 1e-300)))


def make_snapshots(session, n, seed, device="cuda"):
    """n snapshots of the session's plain force: (x bf16 [n][C][16], y fp32
    [n][C][4]) torch tensors on the device."""
    import torch
    C = session.C
    x = torch.empty((n, C, mcpm.SUR_IN), dtype=torch.bfloat16, device=device)
    y = torch.empty((n, C, mcpm.SUR_OUT), dtype=torch.float32, device=device)
    rng = np.random.default_rng(seed)
    chunk = 512
    for i in range(0, n, chunk):
        k = min(chunk, n - i)
        F = random_fields(rng, k)
        session.vlasov_snapshots(F, N_WAVES, seed + i, x[i].data_ptr(), y[i].data_ptr())
    torch.cuda.synchronize()
    return x, y


def validate(sur, x, y, scale, batch):
    """Kick-coefficient error of the network on snapshots x, y."""
    import torch
    n = x.shape[0]
    out = torch.empty_like(y)
    for i in range(0, n, batch):
        k = min(batch, n - i)
        sur.forward(x[i].data_ptr(), k, out[i].data_ptr())
    torch.cuda.synchronize()
    return kick_error(out.cpu().numpy() * scale, y.cpu().numpy())


def train(cfg, n_snap=20000, n_val=256, batch=4, epochs=12, lr=2e-3, seed=0x5352, log=print, x=None, y=None,
          log_every=500):
    """Trains a network for the session geometry of cfg; returns (params,
    out_scale, info)."""
    import torch
    session = mcpm.Session(cfg)
    N0, N1 = cfg.n_cells[0], cfg.n_cells[1]
    t0 = time.time()
    if x is None:
        x, y = make_snapshots(session, n_snap + n_val, seed)
    t_gen = time.time() - t0
    n_tr = x.shape[0] - n_val
    scale = float(y[:min(n_tr, 512)].double().pow(2).mean().sqrt())
    sur = mcpm.Surrogate(N0, N1, max_batch=batch)
    sur.set_params(init_params(seed), scale)
    steps = epochs * (n_tr // batch)
    t1 = time.time()
    hist = []
    t = 0
    for ep in range(epochs):
        for b in range(n_tr // batch):
            t += 1
            lr_t = lr * (0.02 + 0.98 * 0.5 * (1.0 + math.cos(math.pi * t / steps)))
            want = (t - 1) % log_every == 0 or t == steps
            loss = sur.train_step(x[b * batch].data_ptr(), y[b * batch].data_ptr(), batch, 1.0 / scale, lr_t, t,
                                  want_loss=want)
            if want:
                rel = math.sqrt(loss[0] / max(loss[1], 1e-300))
                hist.append((t, rel))
                log("epoch %d step %d lr %.2e rel-rms %.4e" % (ep, t, lr_t, rel))
    sur.sync()
    t_train = time.time() - t1
    val = validate(sur, x[n_tr:], y[n_tr:], scale, batch) if n_val > 0 else None
    log("validation kick error %.4e (generation %.1f s, training %.1f s)" % (val if val is not None else -1, t_gen,
                                                                              t_train))
    params = sur.get_params()
    info = dict(n_snap=int(n_tr), n_val=int(n_val), batch=batch, epochs=epochs, lr=lr, seed=seed,
                val_kick_error=val, gen_s=t_gen, train_s=t_train, steps=t, history=hist,
                grid=[int(N0), int(N1)], dx=cfg.length[0] / N0, bst=cfg.bst, sigma=cfg.sigma, b=cfg.b,
                Fn=cfg.Fn, long_range=int(cfg.long_range))
    sur.close()
    session.close()
    return params, scale, info


def save(path, params, scale, info):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=params.astype(np.float32), out_scale=np.float64(scale), info=json.dumps(info))


def load(path=WEIGHTS):
    """(params float32 [MCPM_SUR_NPARAM], out_scale, info dict)."""
    d = np.load(path, allow_pickle=False)
    return d["params"], float(d["out_scale"]), json.loads(str(d["info"]))


def attach(session, path=WEIGHTS, judge_every=10, threshold=0.01, tcgen05=True):
    """Loads trained weights into a network for the session's grid and attaches it."""
    params, scale, _ = load(path)
    sur = mcpm.Surrogate(session.cfg.n_cells[0], session.cfg.n_cells[1], 1)
    sur.set_params(params, scale)
    sur.set_tensor_path(tcgen05)
    session.attach_surrogate(sur, judge_every, threshold)
    return sur


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--cells", type=int, default=256)
    ap.add_argument("--snapshots", type=int, default=20000)
    ap.add_argument("--val", type=int, default=256)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0x5352)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--log-every", type=int, default=500)
    a = ap.parse_args(argv)
    n = a.cells
    cfg = bench_config(n)
    params, scale, info = train(cfg, n_snap=a.snapshots, n_val=a.val, batch=a.batch, epochs=a.epochs, lr=a.lr,
                                seed=a.seed, log_every=a.log_every)
    save(a.out, params, scale, info)
    print(json.dumps({k: v for k, v in info.items() if k != "history"}))


if __name__ == "__main__":
    main()
