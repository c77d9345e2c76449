"""The settings-file front end (mcpm_config_from_settings, a restatement of
readSettingsFile, src/myIO.cpp:1756-3016, for problems 1, 2, 11 and 12) on the
fixtures in tests/golden/settings: bit-exact against the reference's own
reader where the reference tree is present, and against the values it
produced (tests/golden/settings_expected.json, written by
tests/golden/make_golden.py) everywhere.  No GPU needed: the reader is host
code in libmcpm.so."""
import json
import os

import numpy as np
import pytest

import mcpm
import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SETTINGS = os.path.join(HERE, "golden", "settings")
FIXTURES = sorted(f for f in os.listdir(SETTINGS) if f.endswith(".in"))


def _ref_ints(iv):
    """the reference's ints with its problem id as the session's: injection
    (12) runs between the closed box's specular walls (apply_BC,
    src/Main_Functions.cpp:1487-1489)"""
    out = [int(v) for v in iv]
    if out[6] == 12:
        out[6] = mcpm.PROBLEM_CLOSED_BOX
    return out


def _values(cfg, N):
    ints = [cfg.n_cells[0], cfg.n_cells[1], cfg.n_cells[2], cfg.direction[0], cfg.direction[1],
            cfg.direction[2], cfg.problem, cfg.long_range, cfg.model, N]
    dbl = [cfg.length[0], cfg.length[1], cfg.length[2], cfg.sigma, cfg.m, cfg.kb, cfg.n, cfg.Fn, cfg.T0, cfg.mu,
           cfg.visp, cfg.b, cfg.dt, cfg.phi, cfg.eqdist, cfg.ast, cfg.bst]
    dbl += list(cfg.T_wall) + list(cfg.U_wall) + [cfg.crref]
    return ints, dbl


def _same_velocity_distribution(a, ref):
    """the seeded draws against the reference's unseeded ones (a new sample
    every run): each velocity component's mean and variance within 5
    standard errors of the difference (the variances' from each sample's
    fourth moment)"""
    def var_se(x):
        d = x - x.mean()
        return np.sqrt(max(np.mean(d ** 4) - np.mean(d ** 2) ** 2, 0.0) / len(x))

    for k in ("U1", "U2", "U3"):
        va, vr = a[k].var(), ref[k].var()
        se = np.sqrt(va / len(a[k]) + vr / len(ref[k]))
        assert abs(a[k].mean() - ref[k].mean()) < 5 * se, k
        se_ratio = (va / vr) * np.hypot(var_se(a[k]) / va, var_se(ref[k]) / vr)
        assert abs(va / vr - 1) < 5 * se_ratio, (k, va / vr, se_ratio)


@pytest.mark.parametrize("name", FIXTURES)
def test_settings_match_golden(built, name):
    with open(os.path.join(HERE, "golden", "settings_expected.json")) as fh:
        exp = json.load(fh)[name]
    cfg, N = mcpm.config_from_settings(os.path.join(SETTINGS, name))
    ints, dbl = _values(cfg, N)
    assert ints == _ref_ints(exp["ints"])
    want = [float.fromhex(h) for h in exp["doubles"]]
    assert dbl == want, [(i, a, b) for i, (a, b) in enumerate(zip(dbl, want)) if a != b]
    assert cfg.precision == mcpm.FP64 and cfg.max_particles == N


@pytest.mark.parametrize("name", FIXTURES)
def test_settings_match_reference(built, name):
    if O.ref_lib() is None:
        pytest.skip("reference sources not available")
    path = os.path.join(SETTINGS, name)
    iv, dv = O.ref_read_settings(path)
    cfg, N = mcpm.config_from_settings(path)
    ints, dbl = _values(cfg, N)
    assert ints == _ref_ints(iv)
    assert np.array_equal(np.array(dbl), dv)


def test_settings_branches(built):
    """the three diameter branches: sigma kept (reduced units), hard spheres
    and variable hard spheres from mu; dt from the cell size or the mean free path"""
    red, _ = mcpm.config_from_settings(os.path.join(SETTINGS, "reduced_fp_ideal.in"))
    assert red.sigma == 1.0 and red.crref == 1.0 and red.dt == pytest.approx(0.05)
    hs, _ = mcpm.config_from_settings(os.path.join(SETTINGS, "closed_box_fp_dense.in"))
    assert hs.sigma != 3.405e-10 and 2e-10 < hs.sigma < 5e-10
    vhs, _ = mcpm.config_from_settings(os.path.join(SETTINGS, "dsmc_vhs.in"))
    assert vhs.model == mcpm.MODEL_DSMC_VHS and vhs.crref > 0 and vhs.visp == 0.81
    es, _ = mcpm.config_from_settings(os.path.join(SETTINGS, "couette_esmc.in"))
    assert es.problem == mcpm.PROBLEM_COUETTE and es.U_wall[1] == 50.0 and es.phi < 0


def _write(dirpath, text):
    p = os.path.join(dirpath, "case.in")
    with open(p, "w") as fh:
        fh.write(text)
    return p


BASE = "model FP_dense\nN 100\nvisp 0.5\nnualpha 1.0\nbox_len 1 10 1\nnum_cells 1 10 1\nsigma 1\nkb 1\nmass 1\nT 1\n"


@pytest.mark.parametrize("extra,needle", [
    ("bogus_key 3\n", "unknown keyword"),
    ("problem 3\n", "problems"),
    ("problem 11\n", "problem wall needs nc"),
    ("problem 11\nnc 0.7\nnv2 0.01\nTc 85\nLcN 20\nLvN 40\n", "LvN1"),
    ("problem 11\nnc 0.7\nnv2 0.01\nTc 85\nLcN 20\nLvN 40\nLvN1 5\n", "nv1"),
    ("model MD\n", "model"),
    ("box_delta_dim 1 2 1\n", "box_delta_dim"),
])
def test_settings_errors(built, extra, needle):
    """what the reference aborts on, or what lies outside the particle step,
    returns MCPM_ERR_ARG with a reason"""
    d = os.path.join(HERE, "_tmp_settings")
    os.makedirs(d, exist_ok=True)
    try:
        p = _write(d, BASE + extra)
        with pytest.raises(mcpm.MCPMError) as e:
            mcpm.config_from_settings(p)
        assert needle in str(e.value)
        p = _write(d, BASE)
        cfg, N = mcpm.config_from_settings(p)
        assert N == 100 and cfg.model == mcpm.MODEL_FP_DENSE
    finally:
        for f in os.listdir(d):
            os.remove(os.path.join(d, f))
        os.rmdir(d)


@pytest.mark.parametrize("name", ["closed_box_fp_dense.in", "couette_esmc.in"])
def test_initialize_from_settings(built, name):
    """initialization's branch for problems 1 and 2: positions uniform along
    the streaming directions (mid-box otherwise), velocities normal about U0
    at T = max(gas.T, max(T_w1 + T_w2, T_w3 + T_w4) / 2).  Repeatable for a
    seed; against the reference's own initialization (std::random_device)
    statistically: means and variances within 5 standard errors."""
    path = os.path.join(SETTINGS, name)
    cfg, N = mcpm.config_from_settings(path)
    a = mcpm.initialize_from_settings(path, 7, N)
    b = mcpm.initialize_from_settings(path, 7, N)
    assert all(np.array_equal(a[k], b[k]) for k in a)
    for d, k in ((0, "x1"), (1, "x2")):
        if cfg.direction[d]:
            assert a[k].min() > 0 and a[k].max() < cfg.length[d]
            assert abs(a[k].mean() / cfg.length[d] - 0.5) < 5 * np.sqrt(1 / 12 / N)
        else:
            assert np.all(a[k] == 0.5 * cfg.length[d])
    ref = O.ref_initialize(path, N)
    if ref is None:
        return
    for k in ("x1", "x2"):
        d = 0 if k == "x1" else 1
        if not cfg.direction[d]:
            assert np.array_equal(a[k], ref[k])
    _same_velocity_distribution(a, ref)


def test_wall_settings(built):
    """problem wall (src/myIO.cpp:2628-2726): argon's diameter with
    eqdist = sigma, densities from sigma^-3, Fn fixed at 1e13, N and the box
    height from the three layers, the liquid's temperature for dt"""
    path = os.path.join(SETTINGS, "wall_fp_dense.in")
    cfg, N = mcpm.config_from_settings(path)
    s = 3.405e-10
    assert cfg.problem == mcpm.PROBLEM_WALL and cfg.sigma == s and cfg.eqdist == s and cfg.Fn == 1e13
    assert cfg.length[1] == (40 * s + 20 * s) + 20 * s
    assert cfg.n == 0.7 / s ** 3
    nv = int(np.floor(0.05 / s ** 3 * 0.0316 * 0.0316 * 20 * s / 1e13))
    nc = int(np.floor(0.7 / s ** 3 * 0.0316 * 0.0316 * (20 * s) / 1e13))
    assert N == nc + nv + int(np.floor(0.05 / s ** 3 * 0.0316 * 0.0316 * 40 * s / 1e13))
    assert cfg.max_particles == N


def test_initialize_wall(built):
    """initialization for problem wall (src/Main_Functions.cpp:4493-4530):
    the first Nv1 particles in the lower vapour layer, the next Nc2 in the
    liquid slab, the rest in the upper vapour layer -- the same layer for
    every particle id as the reference's own initialization; velocities at
    the liquid's temperature, statistically equal to the reference's."""
    path = os.path.join(SETTINGS, "wall_fp_dense.in")
    cfg, N = mcpm.config_from_settings(path)
    a = mcpm.initialize_from_settings(path, 3, N)
    s = 3.405e-10
    edges = np.array([0.0, 20 * s, 40 * s, 80 * s])
    layer = np.searchsorted(edges, a["x2"], side="right") - 1
    assert np.all(np.diff(layer) >= 0) and set(np.unique(layer)) == {0, 1, 2}
    assert a["x2"].min() > 0 and a["x2"].max() < cfg.length[1]
    assert np.all(a["x1"] == 0.5 * cfg.length[0])
    sd = np.sqrt(cfg.kb * 85.0 / cfg.m)
    for k in ("U1", "U2", "U3"):
        assert abs(a[k].std() / sd - 1) < 0.05
    ref = O.ref_initialize(path, N)
    if ref is None:
        return
    assert np.array_equal(np.searchsorted(edges, ref["x2"], side="right") - 1, layer)
    assert np.array_equal(a["x1"], ref["x1"])
    _same_velocity_distribution(a, ref)


def _injection_layout(path, parts, cfg, N):
    """(gas particles inside the box, droplet particles inside the disc)"""
    s = 3.405e-10
    raw = {}
    with open(path) as fh:
        for line in fh:
            f = line.split()
            if f and f[0] in ("nc", "nh", "drop_dia"):
                raw[f[0]] = float(f[1])
    d = raw["drop_dia"] * s
    nh = int(np.floor((raw["nh"] - raw["nc"]) / s ** 3 * np.pi * d * d / 4.0 / cfg.Fn))
    x, y = parts["x1"], parts["x2"]
    gas = (x[:N - nh] > 0) & (x[:N - nh] < cfg.length[0]) & (y[:N - nh] > 0) & (y[:N - nh] < cfg.length[1])
    r2 = (x[N - nh:] - 0.5 * cfg.length[0]) ** 2 + (y[N - nh:] - 0.5 * cfg.length[1]) ** 2
    return nh, gas.all(), bool(np.all(r2 <= (0.5 * d) ** 2 * (1 + 1e-12)))


def test_initialize_injection(built):
    """initialization for problem injection (src/Main_Functions.cpp:4627-4643):
    the gas uniform over the box, the droplet's Nh particles uniform over the
    disc at the centre; velocities at Tc.  Against the reference's own
    initialization where present: the same droplet particles, the same
    velocity statistics."""
    path = os.path.join(SETTINGS, "injection_esmc.in")
    cfg, N = mcpm.config_from_settings(path)
    a = mcpm.initialize_from_settings(path, 5, N)
    nh, gas_ok, disc_ok = _injection_layout(path, a, cfg, N)
    assert nh > 1000 and gas_ok and disc_ok
    # the disc is uniform: half its particles within radius d / (2 sqrt 2)
    s = 3.405e-10
    r = np.hypot(a["x1"][N - nh:] - 0.5 * cfg.length[0], a["x2"][N - nh:] - 0.5 * cfg.length[1])
    assert abs(np.mean(r < 12.0 * s / 2 / np.sqrt(2)) - 0.5) < 5 * np.sqrt(0.25 / nh)
    sd = np.sqrt(cfg.kb * 100.0 / cfg.m)
    for k in ("U1", "U2", "U3"):
        assert abs(a[k].std() / sd - 1) < 0.02
    ref = O.ref_initialize(path, N)
    if ref is None:
        return
    nh_r, gas_r, disc_r = _injection_layout(path, ref, cfg, N)
    assert nh_r == nh and gas_r and disc_r
    _same_velocity_distribution(a, ref)


def test_reference_settings_file(built):
    """The reference's own settings file (its injection run, problem 12):
    read and derived as the reference does, every derived value to the last
    bit, and its initial particles laid out as the reference's."""
    src = O.ref_src_dir()
    path = os.path.join(src, "injection.in") if src else None
    if not path or not os.path.exists(path):
        pytest.skip("reference sources not available")
    cfg, N = mcpm.config_from_settings(path)
    iv, dv = O.ref_read_settings(path)
    ints, dbl = _values(cfg, N)
    assert ints == _ref_ints(iv) and np.array_equal(np.array(dbl), dv)
    assert cfg.problem == mcpm.PROBLEM_CLOSED_BOX and cfg.model == mcpm.MODEL_ESMC
    a = mcpm.initialize_from_settings(path, 9, N)
    nh, gas_ok, disc_ok = _injection_layout(path, a, cfg, N)
    assert gas_ok and disc_ok and nh > 0
