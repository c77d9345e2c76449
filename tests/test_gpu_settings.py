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


@pytest.mark.parametrize("name", ["reduced_fp_ideal.in", "wall_fp_dense.in"])
def test_settings_drive_the_step(cuda_ok, name):
    path = os.path.join(SETTINGS, name)
    cfg, N = mcpm.config_from_settings(path)
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
