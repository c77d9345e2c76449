"""CPU oracle of the learned 2-D Vlasov force network -- test infrastructure.

Only the tests, the smoke check and the benchmark's CPU-baseline leg may use
this module; it is the checker of the CUDA network in libmcpm, never a path of
the product.  The network has no counterpart in the reference (its only
learned model, the hybrid NN/GPR of src/hybrid.cpp, is off the particle path),
so this restates the network as the library defines it (include/mcpm.h,
"learned Vlasov force of a 2-D box"):

    x [B, N1, N0, 16] -> conv3x3 16->64, ReLU -> conv3x3 64->64, ReLU
      -> conv3x3 64->64, ReLU -> conv3x3 64->16 -> y = outputs 0..3

with zero padding, weights [co][tap][ci], tap = 3 (dy + 1) + (dx + 1), and
the loss L = mean over cells and outputs of (y - ts t)^2.

Two modes:
  * exact=True: float64 arithmetic throughout (used to pin the backward pass
    against finite differences);
  * exact=False: the GPU's rounding points -- bf16 weights, bf16 activations
    after each ReLU, the loss gradient rounded to bf16, every data gradient
    rounded to bf16 after its ReLU mask -- with float64 sums (the GPU sums
    in fp32, so results agree to fp32 rounding of the sums, not bit for bit).
"""
from __future__ import annotations

import numpy as np

W = 64
CIN = 16
COUT = 16
SIZES = [("W1", (W, 9, CIN)), ("b1", (W,)), ("W2", (W, 9, W)), ("b2", (W,)), ("W3", (W, 9, W)), ("b3", (W,)),
         ("W4", (COUT, 9, W)), ("b4", (COUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)
TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]  # (dy, dx)


def unpack(p):
    """fp32 parameter array -> dict of views in the library's layout."""
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n]).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float32).reshape(-1) for name, _ in SIZES])


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_bits_to_float(bits):
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def float_to_bf16_bits(a):
    return (bf16(a).view(np.uint32) >> 16).astype(np.uint16)


def _shift(x, dy, dx):
    """s[b, y, x] = x[b, y + dy, x + dx], zero outside the grid."""
    B, H, Wd, Cc = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(Wd, Wd - dx)
    if ys < ye and xs < xe:
        out[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv(x, w, b=None):
    """out[p][co] = sum_{tap, ci} x[p + off(tap)][ci] w[co][tap][ci] (+ b[co])."""
    out = np.zeros(x.shape[:3] + (w.shape[0],), dtype=np.float64)
    for t, (dy, dx) in enumerate(TAPS):
        out += _shift(x, dy, dx) @ w[:, t, :].T.astype(np.float64)
    if b is not None:
        out += b
    return out


def conv_data_grad(dz, w):
    """d/dx of sum(dz * conv(x, w)): dx[p][ci] = sum_{tap, co} dz[p - off(tap)][co] w[co][tap][ci]."""
    out = np.zeros(dz.shape[:3] + (w.shape[2],), dtype=np.float64)
    for t, (dy, dx) in enumerate(TAPS):
        out += _shift(dz, -dy, -dx) @ w[:, t, :].astype(np.float64)
    return out


def conv_weight_grad(x, dz):
    """dW[co][tap][ci] = sum_p dz[p][co] x[p + off(tap)][ci]; db[co] = sum_p dz[p][co]."""
    co, ci = dz.shape[3], x.shape[3]
    dW = np.zeros((co, 9, ci))
    dzf = dz.reshape(-1, co).astype(np.float64)
    for t, (dy, dx) in enumerate(TAPS):
        dW[:, t, :] = dzf.T @ _shift(x, dy, dx).reshape(-1, ci).astype(np.float64)
    return dW, dzf.sum(axis=0)


def forward(p, x, exact=False):
    """Returns (y [B,N1,N0,4], activations) for parameters p and input x
    (float values of the bf16 input)."""
    d = unpack(np.asarray(p, dtype=np.float64 if exact else np.float32))
    q = (lambda a: np.asarray(a, dtype=np.float64)) if exact else (lambda a: bf16(a).astype(np.float64))
    ws = {k: q(d[k]) for k in ("W1", "W2", "W3", "W4")}
    bs = {k: np.asarray(d[k], dtype=np.float64) for k in ("b1", "b2", "b3", "b4")}
    x = np.asarray(x, dtype=np.float64)
    a1 = q(np.maximum(conv(x, ws["W1"], bs["b1"]), 0.0))
    a2 = q(np.maximum(conv(a1, ws["W2"], bs["b2"]), 0.0))
    a3 = q(np.maximum(conv(a2, ws["W3"], bs["b3"]), 0.0))
    y = conv(a3, ws["W4"], bs["b4"])[..., :4]
    return y, dict(x=x, a1=a1, a2=a2, a3=a3, W=ws)


def loss_and_grad(p, x, t, ts, exact=False):
    """(loss, sum of squared errors, sum of squared scaled targets, gradient
    as a flat float64 array in the parameter layout)."""
    y, A = forward(p, x, exact)
    e = y - ts * np.asarray(t, dtype=np.float64)
    P = y.shape[0] * y.shape[1] * y.shape[2]
    loss = float((e * e).sum() / (4 * P))
    q = (lambda a: a) if exact else (lambda a: bf16(a).astype(np.float64))
    dz4 = np.zeros(y.shape[:3] + (COUT,))
    if exact:
        dz4[..., :4] = 2.0 * e / (4 * P)
    else:  # the GPU forms g e in fp32, g = 2 / (4 P)
        g = np.float32(2.0) / (np.float32(4.0) * np.float32(P))
        dz4[..., :4] = q(g * e.astype(np.float32))
    Wt = A["W"]
    dW4, db4 = conv_weight_grad(A["a3"], dz4)
    dz3 = q(conv_data_grad(dz4, Wt["W4"]) * (A["a3"] > 0))
    dW3, db3 = conv_weight_grad(A["a2"], dz3)
    dz2 = q(conv_data_grad(dz3, Wt["W3"]) * (A["a2"] > 0))
    dW2, db2 = conv_weight_grad(A["a1"], dz2)
    dz1 = q(conv_data_grad(dz2, Wt["W2"]) * (A["a1"] > 0))
    dW1, db1 = conv_weight_grad(A["x"], dz1)
    g = dict(W1=dW1, b1=db1, W2=dW2, b2=db2, W3=dW3, b3=db3, W4=dW4, b4=db4)
    flat = np.concatenate([np.asarray(g[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])
    return loss, float((e * e).sum()), float(((ts * np.asarray(t)) ** 2).sum()), flat


def init_params(seed, n_in=11, n_out=4):
    """He-normal weights (fan-in of the used input channels), zero biases;
    unused input channels and output rows are zero."""
    rng = np.random.default_rng(seed)
    d = {}
    d["W1"] = np.zeros((W, 9, CIN), np.float32)
    d["W1"][:, :, :n_in] = rng.normal(0, np.sqrt(2.0 / (9 * n_in)), (W, 9, n_in))
    d["W2"] = rng.normal(0, np.sqrt(2.0 / (9 * W)), (W, 9, W)).astype(np.float32)
    d["W3"] = rng.normal(0, np.sqrt(2.0 / (9 * W)), (W, 9, W)).astype(np.float32)
    d["W4"] = np.zeros((COUT, 9, W), np.float32)
    d["W4"][:n_out] = rng.normal(0, np.sqrt(1.0 / (9 * W)), (n_out, 9, W))
    for k in ("b1", "b2", "b3"):
        d[k] = np.zeros(W, np.float32)
    d["b4"] = np.zeros(COUT, np.float32)
    return pack(d)
