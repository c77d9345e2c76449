"""Host transfers through the C-ABI: a download queued without waiting
(mcpm_download_particles_async) delivers the state of the step it was queued
after -- bit for bit the state a synchronous download returns -- although the
next upload replaces the state and more steps run before the copies are
waited for; the upload it overlaps lands intact (the caller's arrays may be
reused once mcpm_upload_particles returns).  Pinned host arrays (the
overlapped path) and pageable ones, FP32 and FP64 sessions."""
import numpy as np
import pytest

import mcpm
import workloads as W

pytestmark = pytest.mark.gpu

KEYS = ("x1", "x2", "U1", "U2", "U3")


def _arrays(n, pinned, fill=np.nan):
    if pinned:
        torch = pytest.importorskip("torch")
        out = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for k in KEYS}
    else:
        out = {k: np.empty(n) for k in KEYS}
    for k in KEYS:
        out[k][:] = fill
    return out


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("prec", [mcpm.FP32, mcpm.FP64])
def test_async_download_overlapping_upload(cuda_ok, pinned, prec):
    cfg, parts = W.uneven_cells_2d(n_cells=(24, 20), precision=prec, hi=600)
    rng = np.random.default_rng(5)
    parts2 = {k: (rng.permutation(parts[k]) if k in ("U1", "U2", "U3") else parts[k].copy()) for k in KEYS}
    rnd = (lambda a: a.astype(np.float32).astype(np.float64)) if prec == mcpm.FP32 else (lambda a: a)
    n = len(parts["x2"])
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.step(2)
    ref1 = _arrays(n, pinned)
    ref1["x1"][:] = parts["x1"]  # left untouched where the device does not keep x1
    s.download_into(ref1)
    out1 = _arrays(n, pinned)
    out1["x1"][:] = parts["x1"]
    s.download_into(out1, wait=False)
    hin = _arrays(n, pinned)
    for k in KEYS:
        hin[k][:] = parts2[k]
    s.upload(hin["x1"], hin["x2"], hin["U1"], hin["U2"], hin["U3"])
    for k in KEYS:  # the caller's arrays are free again once the upload returns
        hin[k][:] = -1.0
    out2 = _arrays(n, pinned)
    out2["x1"][:] = parts2["x1"]
    s.download_into(out2, wait=False)
    s.step(3)
    out3 = _arrays(n, pinned)
    out3["x1"][:] = parts2["x1"]
    s.download_into(out3, wait=False)
    s.sync()
    for k in KEYS:
        assert np.array_equal(out1[k], ref1[k]), k
        assert np.array_equal(out2[k], rnd(parts2[k])), k
    # the three steps from the second state ran on what the upload delivered
    assert np.all(np.isfinite(out3["U1"])) and not np.array_equal(out3["U1"], out2["U1"])
    assert abs(np.sum(out3["U1"] ** 2 + out3["U2"] ** 2 + out3["U3"] ** 2) /
               np.sum(out2["U1"] ** 2 + out2["U2"] ** 2 + out2["U3"] ** 2) - 1.0) < 0.05
    s.close()


def test_async_upload_pipeline(cuda_ok):
    """Queued uploads and downloads back to back (the end-to-end pattern of
    the benchmark): every step's result equals the state a synchronous
    upload + step + download of the same inputs gives."""
    torch = pytest.importorskip("torch")
    cfg, parts = W.uneven_cells_2d(n_cells=(16, 16), precision=mcpm.FP64, hi=300)
    n = len(parts["x2"])
    hin = _arrays(n, True)
    for k in KEYS:
        hin[k][:] = parts[k]
    s = mcpm.Session(cfg)
    outs = []
    for i in range(3):
        s.upload(hin["x1"], hin["x2"], hin["U1"], hin["U2"], hin["U3"], wait=False)
        s.set_step(5 + i)
        s.step(1)
        o = _arrays(n, True)
        o["x1"][:] = parts["x1"]
        s.download_into(o, wait=False)
        outs.append(o)
    s.sync()
    torch.cuda.synchronize()
    for i, o in enumerate(outs):
        r = mcpm.Session(cfg)
        r.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        r.set_step(5 + i)
        r.step(1)
        g = r.download()
        r.close()
        for k in ("x2", "U1", "U2", "U3"):
            # FP64: only the in-cell summation order (atomics) may differ
            assert np.max(np.abs(o[k] - g[k])) <= 1e-10 * max(1.0, np.max(np.abs(g[k]))), (i, k)
    s.close()
