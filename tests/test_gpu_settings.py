"""A run set up by a settings file in the reference's format: the
configuration (mcpm_config_from_settings) and the initial particles
(mcpm_initialize_from_settings), then fused FP64 steps on the GPU against
the oracle under the same configuration, both drawing the same Philox
streams (1e-10)."""
import os

import numpy as np
import pytest

import mcpm
from oracle import Oracle

pytestmark = pytest.mark.gpu

SETTINGS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "settings")


@pytest.mark.parametrize("name", ["reduced_fp_ideal.in", "wall_fp_dense.in", "injection_esmc.in"])
def test_settings_drive_the_step(cuda_ok, name):
    path = os.path.join(SETTINGS, name)
    cfg, N = mcpm.config_from_settings(path)
    if cfg.model == mcpm.MODEL_ESMC:
        # ESMC pairs follow the device's in-cell order; the fused-step
        # comparison with the oracle runs the file's set-up with FP_dense
        cfg.model = mcpm.MODEL_FP_DENSE
    parts = mcpm.initialize_from_settings(path, 41, N)
    ses = mcpm.Session(cfg)
    ses.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg, parts)
    ses.set_rng(mcpm.RNG_PHILOX)
    o.set_rng(mcpm.RNG_PHILOX)
    ses.set_step(1)
    o.set_step(1)
    ses.step(3)
    o.step(3)
    g = ses.download()
    for k in ("x2", "U1", "U2", "U3"):
        a, b = g[k], getattr(o.s, k)
        assert np.max(np.abs(a - b)) / np.max(np.abs(b)) <= 1e-10, k
    assert not np.array_equal(g["U1"], parts["U1"])


def test_injection_file_runs_esmc(cuda_ok):
    """The injection set-up with its own model (ESMC and the direct 2-D
    Vlasov force, specular walls): fused steps keep every particle in the
    box and the droplet denser than the gas around it."""
    path = os.path.join(SETTINGS, "injection_esmc.in")
    cfg, N = mcpm.config_from_settings(path)
    assert cfg.model == mcpm.MODEL_ESMC and cfg.long_range == mcpm.LR_DIRECT
    parts = mcpm.initialize_from_settings(path, 43, N)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.step(4)
    s.check_status()
    g = s.download()
    assert np.all((g["x1"] >= 0) & (g["x1"] <= cfg.length[0]) & (g["x2"] >= 0) & (g["x2"] <= cfg.length[1]))
    n = mcpm.cell_field(s.get_cells(), "N").reshape(cfg.n_cells[1], cfg.n_cells[0])
    c0, c1 = cfg.n_cells[1] // 2, cfg.n_cells[0] // 2
    assert n[c0 - 2:c0 + 2, c1 - 2:c1 + 2].mean() > 3.0 * n[:4, :4].mean()
