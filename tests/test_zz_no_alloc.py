"""The allocation-free screened-Poisson force (mcpm_poisson_force_1d_noalloc),
for callers that cannot allocate device memory, against the session's own
long-range force (mcpm_velocity_update with long_range 3) on the same cell
densities, on two calls in a row.  Collected last on purpose: it leaves the
library's shared scratch array in use."""
import ctypes as C

import numpy as np
import pytest

import mcpm
import workloads as W

pytestmark = pytest.mark.gpu


def _session_force(cfg, parts, step):
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(step)
    s.cell_update()
    s.random_generator()
    s.velocity_update()  # computes F2 per cell through the session path
    cells = s.get_cells()
    s.close()
    return mcpm.cell_field(cells, "N"), mcpm.cell_field(cells, "F2")


def test_noalloc_matches_session_force(cuda_ok):
    torch = pytest.importorskip("torch")
    lib = mcpm.load_library()
    cfg, parts = W.vlasov_slab_1d(n_cells=300, mean_ppc=80, long_range=mcpm.LR_SCREENED_POISSON)
    ref2 = None
    for call, seed_step in enumerate((1, 4)):
        # a second, different density field for the second call
        if call == 1:
            parts = {k: v.copy() for k, v in parts.items()}
            parts["x2"] = np.sort(parts["x2"]) * 0.97 + 0.01
        n, F2_ref = _session_force(cfg, parts, seed_step)
        d_n = torch.tensor(n, dtype=torch.float64, device="cuda")
        d_F = torch.full((cfg.n_cells[1],), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.mcpm_poisson_force_1d_noalloc(C.c_void_p(d_n.data_ptr()), cfg.n_cells[1], C.byref(cfg),
                                               C.c_void_p(d_F.data_ptr()), None)
        assert rc == mcpm.OK
        torch.cuda.synchronize()  # the call queues its work without waiting
        F2 = d_F.cpu().numpy()
        scale = np.max(np.abs(F2_ref))
        assert np.max(np.abs(F2 - F2_ref)) <= 1e-12 * scale, "call %d" % call
        if ref2 is not None:
            assert not np.allclose(F2, ref2)
        ref2 = F2


def test_noalloc_rejects_oversize(cuda_ok):
    lib = mcpm.load_library()
    cfg, _ = W.vlasov_slab_1d(n_cells=50, mean_ppc=10, long_range=mcpm.LR_SCREENED_POISSON)
    rc = lib.mcpm_poisson_force_1d_noalloc(C.c_void_p(16), 7000, C.byref(cfg), C.c_void_p(16), None)
    assert rc == mcpm.ERR_CAPACITY
