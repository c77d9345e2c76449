"""The CPU oracle of the learned Vlasov force network, pinned without a GPU:
its backward pass equals central finite differences of its forward pass
(float64 mode), its bfloat16 rounding is round-to-nearest-even, and its
parameter layout matches the one include/mcpm.h declares."""
import os
import re

import numpy as np

import surrogate_oracle as SO

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_layout_matches_header():
    hdr = open(os.path.join(REPO, "include", "mcpm.h")).read()
    n = int(re.search(r"#define MCPM_SUR_NPARAM (\d+)", hdr).group(1))
    assert n == SO.NPARAM == 92368
    p = np.arange(SO.NPARAM, dtype=np.float32)
    assert np.array_equal(SO.pack(SO.unpack(p)), p)


def test_bf16_rounding():
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 3 2^-8 rounds up
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e38, 1e-40], dtype=np.float32)
    r = SO.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2.0 ** -6 and r[3] == -2.5
    assert np.isfinite(r[4]) and r[5] == SO.bf16(np.float32(1e-40))
    bits = SO.float_to_bf16_bits(v)
    assert np.array_equal(SO.bf16_bits_to_float(bits), r)


def _problem(seed, shape=(2, 5, 6)):
    rng = np.random.default_rng(seed)
    p = SO.init_params(seed)
    d = SO.unpack(p.copy())
    for k in ("b1", "b2", "b3"):
        d[k][:] = rng.normal(0, 0.1, d[k].shape)  # make ReLU boundaries non-trivial
    d["b4"][:4] = rng.normal(0, 0.1, 4)
    p = SO.pack(d).astype(np.float64)
    x = np.zeros(shape + (16,))
    x[..., :11] = rng.normal(0, 1, shape + (11,))
    t = rng.normal(0, 1, shape + (4,))
    return p, x, t


def test_backward_matches_finite_differences():
    p, x, t = _problem(3)
    ts = 0.7
    _, _, _, g = SO.loss_and_grad(p, x, t, ts, exact=True)
    rng = np.random.default_rng(11)
    d = SO.unpack(np.arange(SO.NPARAM))
    # parameters of every layer (used input channels / output rows only)
    picks = []
    for name in ("W1", "W2", "W3", "W4"):
        a = d[name]
        for _ in range(6):
            co = rng.integers(0, 4 if name == "W4" else a.shape[0])
            ci = rng.integers(0, 11 if name == "W1" else a.shape[2])
            picks.append(int(a[co, rng.integers(0, 9), ci]))
    for name in ("b1", "b2", "b3"):
        picks.append(int(d[name][rng.integers(0, 64)]))
    picks.append(int(d["b4"][2]))
    h = 1e-6
    for i in picks:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (SO.loss_and_grad(pp, x, t, ts, exact=True)[0] - SO.loss_and_grad(pm, x, t, ts, exact=True)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1e-3, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_unused_channels_have_zero_gradient():
    p, x, t = _problem(5)
    _, _, _, g = SO.loss_and_grad(p, x, t, 1.0, exact=False)
    d = SO.unpack(g)
    assert np.all(d["W4"][4:] == 0) and np.all(d["b4"][4:] == 0)


def test_committed_weights_load_and_run_on_the_oracle():
    """The trained parameters shipped with the package: layout, training
    record, unused rows zero, and a finite forward pass on the oracle."""
    import surrogate as S
    p, scale, info = S.load()
    assert p.shape == (SO.NPARAM,) and p.dtype == np.float32 and scale > 0
    assert info["val_kick_error"] < 0.01 and info["n_snap"] >= 20000 and info["grid"] == [256, 256]
    d = SO.unpack(p)
    assert np.all(d["W4"][4:] == 0) and np.all(d["b4"][4:] == 0) and np.all(d["W1"][:, :, 11:] == 0)
    x = np.zeros((1, 8, 8, 16), np.float32)
    x[..., 5] = 1.0
    y, _ = SO.forward(p, x)
    assert np.all(np.isfinite(y))
