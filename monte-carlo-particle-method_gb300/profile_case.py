"""A small, self-contained particle-step run for ncu captures.

    python monte-carlo-particle-method_gb300/profile_case.py [workload] [n] [fp32|fp64] [steps]

workload:
  uneven  n x n cells of the log-normal uneven-cells workload (default n=160:
          25,600 cells, ~6.3M particles, 175 MB of FP32 state -- larger than
          the 129 MB L2, a few hundred MB on the device)
  esmc    n x n cells of the 2-D ESMC Couette box (100 particles per cell)
  slab    the 1-D Enskog-Vlasov slab with n cells (1000 particles per cell)
  vlasov  n x n cells of the 2-D Enskog-Vlasov box with the screened-Poisson
          force (244 particles per cell on average: 16.0M at n = 256)
  surrogate  the same box with the trained Vlasov network attached (plain
          judge every 10 steps; the first step is a judge step)

Runs `steps` fused steps (default 3: the first launches of each kernel are
the warm-up, so an ncu capture takes `-s 2 -c 1` of the kernel it names) and
exits 0.
"""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import mcpm  # noqa: E402
import workloads as W  # noqa: E402


def main(argv):
    kind = argv[1] if len(argv) > 1 else "uneven"
    n = int(argv[2]) if len(argv) > 2 else 160
    prec = mcpm.FP64 if (len(argv) > 3 and argv[3] == "fp64") else mcpm.FP32
    steps = int(argv[4]) if len(argv) > 4 else 3
    if kind == "uneven":
        cfg, parts = W.uneven_cells_2d(n_cells=(n, n), precision=prec, streaming=True)
    elif kind == "esmc":
        cfg, parts = W.esmc_box_2d(n_cells=(n, n), precision=prec)
    elif kind in ("vlasov", "surrogate"):
        cfg, parts = W.vlasov_box_2d(n_cells=(n, n), total=244 * n * n, precision=prec,
                                     long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
    elif kind == "slab":
        cfg, parts = W.vlasov_slab_1d(n_cells=n, precision=prec)
    else:
        raise SystemExit("unknown workload %r" % kind)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    sur = None
    if kind == "surrogate":
        import surrogate as SG
        sur = SG.attach(s, judge_every=10, threshold=0.01)
    s.step(steps)
    s.sync()
    s.check_status()
    print("ok", kind, n, len(parts["x2"]), s.surrogate_stats() if sur else "")
    s.close()


if __name__ == "__main__":
    main(sys.argv)
