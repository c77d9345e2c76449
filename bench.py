#!/usr/bin/env python3
"""Particle-step throughput on GB300 (one JSON line on stdout, rank 0).

Workload (default): batched uneven cells -- 65,536 cells (256 x 256) with
log-normal occupancy (median 100, clipped 10..5000, 16.0M particles),
Enskog-Fokker-Planck (FP_dense), FP32 particle state with compensated FP32
moment sums and FP64 per-cell drift solves, free flight with specular walls.
A step is one iteration of the reference's main loop (src/main.cpp:389-669):
cell_update, random_generator, velocity_update, DFP_extra_streaming,
apply_BC, store_old_positions, stream_particles, apply_BC.

  value  particle-steps/s with the state resident in HBM (CUDA events on the
         launch stream, max over ranks).  The particle state (16M x 20 B +
         ids) is larger than L2 (129 MB), so no L2 flush is needed.
  e2e    the same metric through the C-ABI with host buffers: every step
         uploads the state from pinned host memory, steps, and downloads it.
  roofline  the dominant kernel's algorithmic bytes / its average launch
         time (per-kernel CUDA events), against the measured HBM copy peak.
  cpu_baseline  the CPU restatement of the reference step (oracle, 1 core)
         on a bounded sample of the same workload.

--impl reference times the reference's CPU path (the oracle port; the
reference's own build is not available on the GPU host) on all host cores.
--gpus N runs N independent replicas (the step does not shard in this
build), one per rank, launched by torch.distributed.run.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "monte-carlo-particle-method_gb300")
sys.path.insert(0, PKG)

METRIC = "particle-steps/s at 16M particles: plain vs surrogate-Vlasov, moment err <=1%"
UNIT = "particle-steps/s"
# algorithmic bytes per particle of one launch (FP32 state, 2-D positions):
#  update: read x1 x2 U1 U2 U3 pid (24 B), write x1 x2 U1 U2 U3 key (24 B)
#  moments: read U1 U2 U3 (12 B); scatter (not credited): read 28 B, write 24 B
#  esmc: read x1 x2 U1 U2 U3 (20 B), write U1 U2 U3 (12 B)
ALG_BYTES = {"update": 48, "moments": 12, "scatter": 52, "esmc": 32}


def _peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the GPU works."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                s, m = float(r[1]), float(r[2])
            except (ValueError, IndexError):
                continue
            mx = m
            # only samples under load count toward the median
            pw = float(r[3]) if r[3].strip() not in ("", "[N/A]") else 0.0
            if pw > 200.0:
                sm.append(s)
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(nm)
        if not sm and rows:
            try:
                sm = [float(r[1]) for r in rows]
            except ValueError:
                sm = []
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(rows)}


def aggregate_ranks(ms_local, particles_local, steps, dist=None):
    """Whole-job throughput of N replicas: the slowest rank's time (max over
    ranks) and the particles of all ranks (sum).  Returns (ms_max, value)."""
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64)
    n = torch.tensor([float(particles_local)], dtype=torch.float64)
    if dist is not None and dist.is_initialized():
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t, n = t.to(dev), n.to(dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(n, op=dist.ReduceOp.SUM)
    ms_max = float(t.item())
    return ms_max, float(n.item()) * steps / (ms_max / 1e3)


def build_workload(args):
    import mcpm
    import workloads as W
    if args.workload == "uneven16m":
        cfg, parts = W.uneven_cells_2d(precision=mcpm.FP32, streaming=True)
        desc = {"workload": "uneven-cells 256x256 log-normal(median 100, 10..5000) FP_dense fp32 "
                            "streaming+specular walls",
                "cells": 65536, "particles": int(len(parts["x2"])),
                "sigma_lognormal": round(float(parts["sigma_lognormal"]), 4)}
    elif args.workload == "esmc6m":
        cfg, parts = W.esmc_box_2d(precision=mcpm.FP32)
        desc = {"workload": "ESMC 256x256 100/cell nb=0.2 diffuse walls fp32", "cells": 65536,
                "particles": int(len(parts["x2"]))}
    elif args.workload == "vlasov16m":
        cfg, parts = W.vlasov_box_2d(n_cells=(256, 256), total=16_000_000, precision=mcpm.FP32,
                                     long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
        desc = {"workload": "2-D Enskog-Vlasov box 256x256 sinusoidal density (nb 0.05..0.45) FP_dense fp32, "
                            "screened-Poisson FEM force with Green's-function walls every step (plain path)",
                "cells": 65536, "particles": int(len(parts["x2"]))}
    elif args.workload == "slab1m":
        cfg, parts = W.vlasov_slab_1d(precision=mcpm.FP32)
        desc = {"workload": "1-D Enskog-Vlasov slab 1000 cells 1M fp32 screened-Poisson",
                "cells": 1000, "particles": int(len(parts["x2"]))}
    else:
        raise SystemExit("unknown workload " + args.workload)
    return cfg, parts, desc


def cpu_baseline_sample(seconds=12.0):
    """The oracle (FP64 CPU restatement of the reference step, 1 core) on a
    32 x 32-cell sample of the same workload; returns particle-steps/s."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import mcpm
    import workloads as W
    from oracle import Oracle
    cfg, parts = W.uneven_cells_2d(n_cells=(32, 32), precision=mcpm.FP64, streaming=True)
    o = Oracle(cfg, parts)
    o.set_step(1)
    o.step(1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        o.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el > seconds or steps >= 50:
            break
    return o.N * steps / el, o.N, steps


def run_mcpm(args):
    import numpy as np
    import torch

    import mcpm
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg, parts, desc = build_workload(args)
    N = len(parts["x2"])
    s = mcpm.Session(cfg)
    stream = torch.cuda.Stream()  # a real stream handle (the legacy default stream is 0)
    torch.cuda.set_stream(stream)
    s.set_stream(stream.cuda_stream)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    if cfg.model == mcpm.MODEL_ESMC:
        s.cell_update()
        s.init_omega_max()
    wcap = s.autotune(3)  # threads-per-cell split; the state is restored
    clocks = ClockSampler(local)
    s.step(args.warmup)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = s.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = s.kernel_launches - l0
    ms = e0.elapsed_time(e1)
    # keep the GPU busy a little longer so the clock record has samples
    t_end = time.time() + 1.5
    while time.time() < t_end:
        s.step(20)
        torch.cuda.synchronize()
    ck = clocks.stop()
    ms_max, value = aggregate_ranks(ms, N, args.steps, dist)

    # per-kernel device times (separate short run with CUDA events per launch)
    s.profile(True)
    s.step(5)
    prof = s.profile_read()
    s.profile(False)
    tot = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms = prof[dom][0] / max(1, prof[dom][1])
    hbm, peak_kind = _peaks()
    bytes_per_launch = ALG_BYTES.get(dom, 0) * N
    achieved = bytes_per_launch / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    traffic = None
    tp = os.path.join(REPO, "profiles", "traffic_%s.json" % args.workload)
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get(dom)
    roofline = {"bound": "hbm", "kernel": "k_" + dom, "achieved": round(achieved, 1), "peak": hbm,
                "unit": "GB/s", "frac": round(achieved / hbm, 4), "peak_kind": peak_kind,
                "traffic": traffic, "bytes_per_launch": bytes_per_launch, "avg_launch_ms": round(dom_ms, 4),
                "share": {k: round(v[0] / tot, 4) for k, v in prof.items() if v[0] > 0}}

    # end to end through the C-ABI with pinned host buffers
    pin = lambda: torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    hin = {k: pin() for k in ("x1", "x2", "U1", "U2", "U3")}
    for k in hin:
        hin[k][:] = parts[k]
    hout = {k: pin() for k in ("x1", "x2", "U1", "U2", "U3")}
    e2e_steps = max(2, min(5, args.steps))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.upload(hin["x1"], hin["x2"], hin["U1"], hin["U2"], hin["U3"])
        s.step(1)
        s.download_into(hout)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    e2e = {"value": N * ws / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 5 * 8 * N,
           "d2h_bytes_per_step": 5 * 8 * N, "ms_per_step": round(e2e_ms, 3)}
    ok = bool(np.all(np.isfinite(hout["U1"])))
    s.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, n, st = cpu_baseline_sample()
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle FP64 restatement, 32x32-cell sub-box of the same workload (%d particles), %d steps"
                         % (n, st)}
    if dist:
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": dict(desc, l2="inputs larger than L2 (no flush)", replicas=ws, precision="fp32 state, fp64 solves",
                       wcap_autotuned=wcap),
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": ck,
        "finite": ok,
    }
    print(json.dumps(line))


# --------------------------------------------------------- reference arm
def _ref_worker_init(cfg_dict, sub):
    global _W
    sys.path.insert(0, PKG)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import mcpm
    from oracle import Oracle
    c = mcpm.Config()
    for k, v in cfg_dict.items():
        f = getattr(c, k)
        if hasattr(f, "__len__"):
            f[:] = v
        else:
            setattr(c, k, v)
    _W = Oracle(c, sub)
    _W.set_step(1)


def _ref_worker_step(n):
    _W.step(n)
    return _W.N * n


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import multiprocessing as mp

    import numpy as np

    import mcpm
    cores = os.cpu_count() or 1
    P = max(1, min(cores, 64))
    cfg, parts, desc = build_workload(args)
    cfg.precision = mcpm.FP64
    Ntot = len(parts["x2"])
    N1 = cfg.n_cells[1]
    dy = cfg.length[1] / N1
    k = np.floor(parts["x2"] / dy).astype(np.int64)
    ctx = mp.get_context("spawn")
    pools = []
    for i in range(P):
        lo, hi = i * N1 // P, (i + 1) * N1 // P
        m = (k >= lo) & (k < hi)
        sub = {kk: np.ascontiguousarray(parts[kk][m]) for kk in ("x1", "x2", "U1", "U2", "U3")}
        sub["x2"] = sub["x2"] - lo * dy
        c = cfg.copy()
        c.n_cells[1] = hi - lo
        c.length[1] = (hi - lo) * dy
        c.max_particles = int(m.sum())
        pools.append(ctx.Pool(1, initializer=_ref_worker_init, initargs=(c.as_dict(), sub)))
    del parts
    try:
        if args.warmup:
            for r in [p.apply_async(_ref_worker_step, (args.warmup,)) for p in pools]:
                r.get()
        t0 = time.perf_counter()
        res = [p.apply_async(_ref_worker_step, (args.steps,)) for p in pools]
        done = sum(r.get() for r in res)
        el = time.perf_counter() - t0
    finally:
        for p in pools:
            p.terminate()
    value = done / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": dict(desc, precision="fp64 (reference CPU path)"), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": P, "kind": "port",
                             "sample": "the full workload (%d particles) split into %d strips of cell rows, "
                                       "one oracle process per core, every step" % (Ntot, P)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mcpm", choices=["mcpm", "reference"])
    ap.add_argument("--workload", default="uneven16m", choices=["uneven16m", "esmc6m", "slab1m", "vlasov16m"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "mcpm":
        args.warmup = 3
    if args.impl == "reference":
        # one reference step of the 16M workload is ~0.5-1 s on 16 cores
        args.steps = min(args.steps, 60)
        args.warmup = min(args.warmup, 1)
        run_reference(args)
    else:
        run_mcpm(args)


if __name__ == "__main__":
    main()
