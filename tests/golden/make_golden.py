"""Generates the golden vectors in this directory from the reference itself.

Runs the reference's own routines (oracle/_ref/libref.so, compiled from the
reference sources by oracle/build.py) on small seeded inputs with injected
normals and stores inputs and outputs as .npz.  tests/test_oracle_golden.py
checks the CPU restatement against these files bit for bit, which pins the
oracle where the reference tree is not available.

    python tests/golden/make_golden.py [case ...]     (all cases by default)
    python tests/golden/make_golden.py settings       (settings_expected.json)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "monte-carlo-particle-method_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import mcpm  # noqa: E402
import oracle as O  # noqa: E402
import workloads as W  # noqa: E402


def cfg_json(cfg):
    return json.dumps(cfg.as_dict())


def case_fp_step():
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=10, ppc=50)
    r = O.Reference(cfg, parts)
    rng = np.random.default_rng(101)
    xi = [rng.standard_normal(r.N) for _ in range(3)]
    r.inject_normals(*xi)
    r.set_step(1)
    r.cell_update()
    out = dict(index=r.s.index.copy(), cells=r.cells())
    r.random_generator()
    out.update(xi1f=r.xi[0].copy(), xi2f=r.xi[1].copy(), xi3f=r.xi[2].copy())
    r.velocity_fp()
    out.update(U1=r.s.U1.copy(), U2=r.s.U2.copy(), U3=r.s.U3.copy())
    r.dfp_extra_streaming()
    out.update(x2=r.s.x2.copy())
    return cfg, parts, dict(xi1=xi[0], xi2=xi[1], xi3=xi[2], step=1), out


def case_cells_2d():
    cfg, parts = W.uneven_cells_2d(n_cells=(6, 5), hi=60)
    r = O.Reference(cfg, parts)
    r.set_step(2)
    r.cell_update()
    return cfg, parts, dict(step=2), dict(index=r.s.index.copy(), cells=r.cells())


def case_vlasov(lr):
    cfg, parts = W.vlasov_slab_1d(n_cells=60, mean_ppc=40, long_range=lr)
    r = O.Reference(cfg, parts)
    rng = np.random.default_rng(202)
    xi = [rng.standard_normal(r.N) for _ in range(3)]
    r.inject_normals(*xi)
    r.set_step(3)
    r.cell_update()
    r.random_generator()
    r.velocity_fp()
    r.long_range()
    return cfg, parts, dict(xi1=xi[0], xi2=xi[1], xi3=xi[2], step=3), dict(U2=r.s.U2.copy(), cells=r.cells())


def case_specular():
    cfg, parts = W.vlasov_slab_1d(n_cells=40, mean_ppc=30, long_range=mcpm.LR_NONE)
    parts = {k: v.copy() for k, v in parts.items()}
    parts["U2"] = parts["U2"] * 40.0
    r = O.Reference(cfg, parts)
    r.set_step(1)
    r.cell_update()
    r.dfp_extra_streaming()
    r.apply_bc()
    r.store_old_positions()
    r.stream()
    r.apply_bc()
    return cfg, parts, dict(step=1), dict(x2=r.s.x2.copy(), U2=r.s.U2.copy())


def case_fp_linear():
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=10, ppc=50)
    cfg.model = mcpm.MODEL_FP_LINEAR
    r = O.Reference(cfg, parts)
    rng = np.random.default_rng(303)
    xi = [rng.standard_normal(r.N) for _ in range(3)]
    r.inject_normals(*xi)
    r.set_step(2)
    r.cell_update()
    out = dict(index=r.s.index.copy(), cells=r.cells())
    r.random_generator()
    r.velocity_fp()
    out.update(U1=r.s.U1.copy(), U2=r.s.U2.copy(), U3=r.s.U3.copy())
    return cfg, parts, dict(xi1=xi[0], xi2=xi[1], xi3=xi[2], step=2), out


def case_density_expansion():
    cfg, parts = W.vlasov_slab_1d(n_cells=60, mean_ppc=40, long_range=mcpm.LR_DENSITY_EXPANSION)
    r = O.Reference(cfg, parts)
    r.set_step(3)
    r.cell_update()
    out = dict(cells=r.cells())
    r.long_range()
    out.update(U2=r.s.U2.copy())
    return cfg, parts, dict(step=3), out


CASES = {
    "fp_step_1d": case_fp_step,
    "cells_2d": case_cells_2d,
    "vlasov_direct_1d": lambda: case_vlasov(mcpm.LR_DIRECT),
    "vlasov_gf_1d": lambda: case_vlasov(mcpm.LR_SCREENED_POISSON),
    "specular_bc_1d": case_specular,
    "fp_linear_1d": case_fp_linear,
    "density_expansion_1d": case_density_expansion,
}


def settings_expected():
    """readSettingsFile of the reference on every settings/*.in fixture, the
    derived values as exact hex floats (settings_expected.json)"""
    out = {}
    d = os.path.join(HERE, "settings")
    for f in sorted(os.listdir(d)):
        if f.endswith(".in"):
            iv, dv = O.ref_read_settings(os.path.join(d, f))
            out[f] = dict(ints=[int(v) for v in iv], doubles=[float(v).hex() for v in dv])
    with open(os.path.join(HERE, "settings_expected.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("settings_expected.json", sorted(out))


def main():
    if O.ref_lib() is None:
        raise SystemExit("the reference build (oracle/_ref) is not available")
    if sys.argv[1:] == ["settings"]:
        settings_expected()
        return
    for name in sys.argv[1:] or list(CASES):
        cfg, parts, extra, out = CASES[name]()
        arrays = {"in_" + k: np.asarray(v) for k, v in parts.items() if k in ("x1", "x2", "U1", "U2", "U3")}
        arrays.update({"in_" + k: np.asarray(v) for k, v in extra.items()})
        arrays.update({"out_" + k: np.asarray(v) for k, v in out.items()})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), config=np.array(cfg_json(cfg)), **arrays)
        print(name, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
