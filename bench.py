#!/usr/bin/env python3
"""Particle-step throughput on GB300 (one JSON line on stdout, rank 0).

Workload (default, surrogate16m): the 2-D Enskog-Vlasov box -- 256 x 256
unit cells, 16.0M particles with a sinusoidally perturbed density (n b
between 0.05 and 0.45), Enskog-Fokker-Planck (FP_dense), FP32 particle state
with FP32 moment sums (per-lane runs combined pairwise) and FP64 per-cell
drift solves, specular
walls, and the Vlasov mean-field force from the learned convolutional
operator, judged every 10 steps by the plain screened-Poisson FEM path
(which takes over while the kick error exceeds 1%).  A step is one
iteration of the reference's main loop (src/main.cpp:389-669): cell_update,
random_generator, velocity_update, DFP_extra_streaming, apply_BC,
store_old_positions, stream_particles, apply_BC.  The line also carries the
plain path on the same workload (FP32 and FP64 particle-steps/s) and the
errors of the surrogate run against the FP64 plain run in n, T and the
force field.  Other workloads (--workload): uneven16m (65,536 cells with
log-normal occupancy), esmc6m, dsmc6m (the same box with Bird's DSMC), slab1m,
vlasov16m (the plain 2-D force).

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
#  update: read x1 x2 U1 U2 U3 pid (24 B), write x1 x2 U1 U2 U3 pid into the
#  new cell's region of the slotted layout (24 B; FP64 sessions write the key)
#  moments: read U1 U2 U3 (12 B); scatter (FP64 sessions, not credited): read
#  28 B, write 24 B
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


def host_link_rates(stream, n_doubles):
    """The bare host<->device copy rate on this machine for the bytes one e2e
    step moves each way: copy-engine cudaMemcpyAsync of n_doubles doubles
    between pinned host memory and the device (GB/s, CUDA events)."""
    import torch
    h = torch.empty(n_doubles, dtype=torch.float64, pin_memory=True)
    d = torch.empty(n_doubles, dtype=torch.float64, device="cuda")
    out = {}
    for name, f in (("h2d_GBs", lambda: d.copy_(h, non_blocking=True)),
                    ("d2h_GBs", lambda: h.copy_(d, non_blocking=True))):
        f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            f()
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = round(3 * 8 * n_doubles / (e0.elapsed_time(e1) / 1e3) / 1e9, 1)
    # both directions at once (a second pair of buffers, a second stream):
    # the floor of an e2e step whose upload and download overlap
    h2 = torch.empty(n_doubles, dtype=torch.float64, pin_memory=True)
    d2 = torch.empty(n_doubles, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = None
    for _ in range(4):
        torch.cuda.synchronize()
        e0.record(stream)
        side.wait_event(e0)
        d.copy_(h, non_blocking=True)
        with torch.cuda.stream(side):
            h2.copy_(d2, non_blocking=True)
        stream.wait_stream(side)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    out["both_ms"] = round(best, 3)
    out["both_GBs"] = round(2 * 8 * n_doubles / (best / 1e3) / 1e9, 1)
    del h, d, h2, d2
    return out


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
    elif args.workload == "dsmc6m":
        cfg, parts = W.esmc_box_2d(precision=mcpm.FP32)
        cfg = W.with_dsmc_vhs(cfg)
        desc = {"workload": "DSMC_VHS 256x256 100/cell diffuse walls fp32", "cells": 65536,
                "particles": int(len(parts["x2"]))}
    elif args.workload == "surrogate16m":
        cfg, parts = W.vlasov_box_2d(n_cells=(256, 256), total=16_000_000, precision=mcpm.FP32,
                                     long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
        desc = {"workload": "2-D Enskog-Vlasov box 256x256 sinusoidal density (nb 0.05..0.45) FP_dense fp32, "
                            "Vlasov force from the learned conv operator (bf16, tcgen05), plain screened-Poisson "
                            "FEM judge every 10 steps, takeover above 1% kick error",
                "cells": 65536, "particles": int(len(parts["x2"]))}
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


def _bf16_peak():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


# algorithmic FLOPs of one inference of the learned force per cell: the used
# input channels (11) and outputs (4): 2 (9 11 64 + 2 9 64 64 + 9 64 4)
SURROGATE_FLOP_PER_CELL = 2 * (9 * 11 * 64 + 2 * 9 * 64 * 64 + 9 * 64 * 4)


def force_eval_ms(s, stream, method, reps=20, replays=5):
    """Device time of one 2-D Vlasov force evaluation on the session's
    current cell state (method 0: plain path, 1: the network), from a CUDA
    graph of `reps` evaluations replayed `replays` times."""
    import torch
    s.eval_vlasov_2d(method)  # warm
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        for _ in range(reps):
            s.eval_vlasov_2d(method)
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(replays):
        g.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / (reps * replays)


def _rel(a, b):
    import numpy as np
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _field_errors(c, ref, n0, n1, blocks_of=(8, 32)):
    """Errors of the cell fields c against ref ([CF][C] as mcpm_get_cells
    returns them): relative L2 over cells of n and T; P_ij as the relative
    Frobenius norm over cells; the heat flux q_i against its thermal scale
    (rms over cells of (3 kT/m)^(3/2)); and n, T averaged over blocks of
    b x b cells (count-weighted T), where the per-cell sampling noise of two
    runs that no longer share trajectories averages out (about
    sqrt(2 / particles per block) for two independent runs)."""
    import numpy as np

    import mcpm
    F = mcpm.CF
    n, nr = c[F["N"]], ref[F["N"]]
    T, Tr = c[F["T"]], ref[F["T"]]
    P, Pr = c[F["PIJ"]:F["PIJ"] + 6], ref[F["PIJ"]:F["PIJ"] + 6]
    q, qr = c[F["Q"]:F["Q"] + 3], ref[F["Q"]:F["Q"] + 3]
    th = np.sqrt(np.mean(np.maximum(ref[F["DM2"]], 0.0) ** 3))
    cnt, cntr = c[F["NUM_INSIDE"]], ref[F["NUM_INSIDE"]]

    def blocks(v, w, b):
        s = (v * w).reshape(n1 // b, b, n0 // b, b).sum(axis=(1, 3))
        return s / np.maximum(w.reshape(n1 // b, b, n0 // b, b).sum(axis=(1, 3)), 1e-300)

    ones = np.ones_like(n)
    out = {"n_rel_l2": _rel(n, nr), "T_rel_l2": _rel(T, Tr), "P_rel_fro": _rel(P, Pr),
           "q_rel_thermal": float(np.linalg.norm(q - qr) / (th * np.sqrt(q.size)))}
    for b in blocks_of:
        if n0 % b == 0 and n1 % b == 0:
            out["n_rel_l2_%dx%d" % (b, b)] = _rel(blocks(n, ones, b), blocks(nr, ones, b))
            out["T_rel_l2_%dx%d" % (b, b)] = _rel(blocks(T, cnt, b), blocks(Tr, cntr, b))
    return out


def surrogate_comparison(args, cfg, parts, s, stream):
    """The plain path on the same workload (FP32 and FP64 particle-steps/s),
    and the accuracy of the FP32 + network run against the FP64 plain run
    (the FP64 GPU step, parity-tested against the FP64 oracle) from the same
    state with the same draws, at checkpoints up to the workload's 2,000
    steps: cell density n, temperature T, pressure tensor P_ij and heat flux
    q_i (_field_errors), and the kick field of the network against the
    plain path's on the FP32 run's state.  The FP32 plain run is carried
    beside it, which separates what the network adds from what FP32 state
    adds."""
    import torch

    import mcpm
    import surrogate as SG
    N = len(parts["x2"])
    stats = s.surrogate_stats()

    def timed(sess, k):
        sess.step(3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sess.step(k)
        e1.record(stream)
        torch.cuda.synchronize()
        return N * k / (e0.elapsed_time(e1) / 1e3)

    k = max(10, min(30, args.steps))
    s.attach_surrogate(None)
    plain32 = timed(s, k)
    cfg64 = cfg.copy()
    cfg64.precision = mcpm.FP64
    s64 = mcpm.Session(cfg64)
    s64.set_stream(stream.cuda_stream)
    s64.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s64.set_wcap(min(s.wcap, 384))
    plain64 = timed(s64, max(5, k // 3))
    # accuracy over the horizon: four runs from the same state -- FP64
    # plain, FP32 + network and FP32 plain with the same draws, and FP32
    # plain with other draws (another Philox seed): the floor that the
    # sampling noise of two independent realisations sets
    sp = mcpm.Session(cfg)
    sp.set_stream(stream.cuda_stream)
    sp.set_wcap(s.wcap)
    cfg_o = cfg.copy()
    cfg_o.seed = cfg.seed ^ 0x5EED
    so = mcpm.Session(cfg_o)
    so.set_stream(stream.cuda_stream)
    so.set_wcap(s.wcap)
    for x in (s64, s, sp, so):
        x.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    sur = SG.attach(s, judge_every=10, threshold=0.01)
    n0, n1 = cfg.n_cells[0], cfg.n_cells[1]
    checkpoints, done, acc = [c for c in (20, 200, 1000, 2000) if c <= args.horizon], 0, []
    t0 = time.perf_counter()
    for cp in checkpoints:
        for x in (s64, s, sp, so):
            x.step(cp - done)
        done = cp
        for x in (s64, s, sp, so):
            x.cell_update()
        c64, c32, cp32, co32 = s64.get_cells(), s.get_cells(), sp.get_cells(), so.get_cells()
        s.eval_vlasov_2d(0)
        kp = s.get_kick_2d()
        s.eval_vlasov_2d(1)
        kn = s.get_kick_2d()
        e = _field_errors(c32, c64, n0, n1)
        e["force_rel_l2"] = _rel(kn, kp)
        acc.append({"step": cp, "surrogate_fp32": e, "plain_fp32": _field_errors(cp32, c64, n0, n1),
                    "plain_fp32_other_draws": _field_errors(co32, c64, n0, n1)})
    acc_s = time.perf_counter() - t0
    st2 = s.surrogate_stats()
    s64.close()
    sp.close()
    so.close()
    sur_info = SG.load()[2]
    return {
        "plain": {"fp32_value": plain32, "fp64_value": plain64, "unit": UNIT,
                  "steps_timed": [k, max(5, k // 3)],
                  "note": "the same workload with the plain screened-Poisson FEM force every step"},
        "accuracy": {"against": "FP64 plain GPU step from the same state with the same draws (parity-tested "
                                "against the FP64 oracle)", "checkpoints": acc,
                     "judge": {k2: st2[k2] for k2 in ("last_error", "judged", "takeovers")},
                     "wall_s": round(acc_s, 1)},
        "surrogate": {"judge_every": 10, "threshold": 0.01, "timed_run": stats,
                      "trained_on": {kk: sur_info.get(kk) for kk in ("n_snap", "epochs", "batch", "steps",
                                                                    "val_kick_error", "train_s", "gen_s")}},
    }


def side_workloads(args, stream, steps=20):
    """The other benchmark workloads timed the same way (device-resident,
    CUDA events on the launch stream, after 3 warm-up steps), each in its
    own session: the uneven 16M box (65,536 cells of 10 to 5,000 particles;
    threads-per-cell autotuned), the 2-D ESMC box (256 x 256 cells of 100),
    the same box with Bird's DSMC (the sibling collision operator) and the
    1-D Vlasov slab (1,000 cells of 1,000 particles, FP32 and FP64).
    Returns {workload: {value, ms_per_step, particles, ...}}."""
    import torch

    import mcpm
    out = {}
    runs = [("uneven16m", mcpm.FP32), ("esmc6m", mcpm.FP32), ("dsmc6m", mcpm.FP32), ("slab1m", mcpm.FP32),
            ("slab1m", mcpm.FP64)]
    for name, prec in runs:
        a = argparse.Namespace(**vars(args))
        a.workload = name
        cfg, parts, desc = build_workload(a)
        cfg.precision = prec
        N = len(parts["x2"])
        s = mcpm.Session(cfg)
        s.set_stream(stream.cuda_stream)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        del parts
        if cfg.model == mcpm.MODEL_ESMC:
            s.cell_update()
            s.init_omega_max()
        wcap = s.autotune(3) if name == "uneven16m" else s.wcap
        s.step(3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        s.check_status()
        s.close()
        key = name + ("_fp64" if prec == mcpm.FP64 else "")
        out[key] = {"value": N / (ms / 1e3), "unit": UNIT, "ms_per_step": round(ms, 4), "steps": steps,
                    "particles": N, "precision": "fp64" if prec == mcpm.FP64 else "fp32", "wcap": wcap,
                    "workload": desc["workload"]}
    return out


def cpu_baseline_sample(args, seconds=12.0):
    """The oracle (FP64 CPU restatement of the reference step, 1 core) on a
    small sub-box of the same workload; returns particle-steps/s."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import mcpm
    import workloads as W
    from oracle import Oracle
    if args.workload in ("surrogate16m", "vlasov16m"):
        # 24 x 24 cells at the benchmark's particles per cell; the 2-D force
        # by the oracle's dense-LU FEM (the reference's PARDISO is absent)
        cfg, parts = W.vlasov_box_2d(n_cells=(24, 24), total=int(round(16_000_000 * 576 / 65536)),
                                     precision=mcpm.FP64, long_range=mcpm.LR_SCREENED_POISSON,
                                     model=mcpm.MODEL_FP_DENSE)
        what = "24x24-cell box of the same workload, plain screened-Poisson FEM force (dense LU)"
    else:
        cfg, parts = W.uneven_cells_2d(n_cells=(32, 32), precision=mcpm.FP64, streaming=True)
        what = "32x32-cell sub-box of the same workload"
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
    return o.N * steps / el, o.N, steps, what


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
    sur = None
    if args.workload == "surrogate16m":
        import surrogate as SG
        sur = SG.attach(s, judge_every=10, threshold=0.01)
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
    # the dominant HBM kernel (one with algorithmic bytes; the per-cell
    # solve of a small grid can take longer but moves almost nothing)
    top = max(prof, key=lambda k: prof[k][0])
    dom = max((k for k in prof if k in ALG_BYTES and prof[k][0] > 0), key=lambda k: prof[k][0], default=top)
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
                "longest_kernel_class": top,
                "share": {k: round(v[0] / tot, 4) for k, v in prof.items() if v[0] > 0}}
    if sur is not None:
        # the learned force: algorithmic FLOPs of one inference (used channels)
        # over its device time, against the measured bf16 peak; the time of
        # one evaluation of each force path is taken from a CUDA graph of 20
        # back-to-back evaluations on the current state (no launch gaps)
        s.cell_update()
        sur_ms = force_eval_ms(s, stream, 1)
        plain_ms = force_eval_ms(s, stream, 0)
        fl = SURROGATE_FLOP_PER_CELL * cfg.n_cells[0] * cfg.n_cells[1]
        tf, tf_kind = _bf16_peak()
        roofline["surrogate"] = {"bound": "tensor", "kernels": "k_input + 4 tcgen05 convolutions (k_conv_tc)",
                                 "achieved": round(fl / (sur_ms / 1e3) / 1e12, 2), "peak": tf, "unit": "TFLOP/s",
                                 "frac": round(fl / (sur_ms / 1e3) / 1e12 / tf, 4), "peak_kind": tf_kind,
                                 "flop_per_inference": fl, "ms_per_inference": round(sur_ms, 4),
                                 "plain_force_ms": round(plain_ms, 4)}

    # end to end through the C-ABI with pinned host buffers
    pin = lambda: torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    hin = {k: pin() for k in ("x1", "x2", "U1", "U2", "U3")}
    for k in hin:
        hin[k][:] = parts[k]
    hout = {k: pin() for k in ("x1", "x2", "U1", "U2", "U3")}
    # the same K steps as the device-resident number, so that the pipeline's
    # first upload and last download (the copies nothing overlaps) weigh
    # little against the steady state of a running simulation
    e2e_steps = max(2, args.steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step0 = s.step_count
    # every step uploads its inputs and reads its result back; the copies
    # and the step are queued (mcpm_upload_particles_async, mcpm_step_async,
    # mcpm_download_particles_async: the host arrays stay untouched until the
    # final sync), so that one step's result copies overlap the next step's
    # input copies and compute; the device status is read once at the end
    for i in range(e2e_steps):
        s.upload(hin["x1"], hin["x2"], hin["U1"], hin["U2"], hin["U3"], wait=False)
        s.set_step(step0 + i)  # the caller's simulation continues (upload restarts the counter)
        s.step(1, wait=False)
        s.download_into(hout, wait=False)
    s.sync()
    s.check_status()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    e2e = {"value": N * ws / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 5 * 8 * N,
           "d2h_bytes_per_step": 5 * 8 * N, "ms_per_step": round(e2e_ms, 3),
           "host_link": host_link_rates(stream, 5 * N)}
    ok = bool(np.all(np.isfinite(hout["U1"])))
    extra = {}
    if sur is not None:
        extra = surrogate_comparison(args, cfg, parts, s, stream)
    s.close()
    del parts
    if ws == 1 and not args.no_side and args.workload == "surrogate16m":
        extra["side_workloads"] = side_workloads(args, stream)

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, n, st, what = cpu_baseline_sample(args)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle FP64 restatement, %s (%d particles), %d steps" % (what, n, st)}
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
    line.update(extra)
    print(json.dumps(line))


# ------------------------------------------------- small case for ncu
def run_profile_case(args):
    """A small particle-step run for ncu captures: the named workload on an
    n x n grid (``--cells``; the 1-D slab: n cells), ``--steps`` fused steps
    (the first launches of each kernel are the warm-up, so a capture takes
    ``-s 2 -c 1`` of the kernel it names), exits 0.

    uneven     log-normal uneven cells (n = 160: 25,600 cells, ~6.3M particles,
               175 MB of FP32 state -- above the 129 MB L2, a few hundred MB
               on the device)
    esmc       the 2-D ESMC box with diffuse walls (100 particles per cell)
    slab       the 1-D Enskog-Vlasov slab (1000 particles per cell)
    vlasov     the 2-D Enskog-Vlasov box with the screened-Poisson force
               (244 particles per cell on average: 16.0M at n = 256)
    surrogate  the same box with the trained Vlasov network attached (plain
               judge every 10 steps; the first step is a judge step)"""
    import mcpm
    import workloads as W
    kind, n = args.profile_case, args.cells
    prec = mcpm.FP64 if args.fp64 else mcpm.FP32
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
        raise SystemExit("unknown profile case %r" % kind)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    sur = None
    if kind == "surrogate":
        import surrogate as SG
        sur = SG.attach(s, judge_every=10, threshold=0.01)
    s.step(args.steps)
    s.sync()
    s.check_status()
    print("ok", kind, n, len(parts["x2"]), s.surrogate_stats() if sur else "")
    s.close()


# --------------------------------------------------------- reference arm
def _ref_worker_init(jobs):
    global _W
    sys.path.insert(0, PKG)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import mcpm
    from oracle import Oracle
    _W = []
    for cfg_dict, sub in jobs:
        c = mcpm.Config()
        for k, v in cfg_dict.items():
            f = getattr(c, k)
            if hasattr(f, "__len__"):
                f[:] = v
            else:
                setattr(c, k, v)
        o = Oracle(c, sub)
        o.set_step(1)
        _W.append(o)


def _ref_worker_step(n):
    done = 0
    for o in _W:
        o.step(n)
        done += o.N * n
    return done


def _ref_split(cfg, parts, P):
    """Sub-boxes of the workload for P worker processes: strips of cell rows,
    or, for a 2-D box with the node-grid Vlasov force (whose dense-LU FEM
    grows as the cube of the node count), square tiles of 32 x 32 cells."""
    import numpy as np
    N0, N1 = cfg.n_cells[0], cfg.n_cells[1]
    dx, dy = cfg.length[0] / N0, cfg.length[1] / N1
    kx = np.floor(parts["x1"] / dx).astype(np.int64)
    ky = np.floor(parts["x2"] / dy).astype(np.int64)
    if cfg.long_range and cfg.direction[0] == 1:
        T = 32
        boxes = [(x0, min(N0, x0 + T), y0, min(N1, y0 + T)) for y0 in range(0, N1, T) for x0 in range(0, N0, T)]
        how = "square tiles of %d x %d cells (%d boxes, each with its own walls)" % (T, T, len(boxes))
    else:
        boxes = [(0, N0, i * N1 // P, (i + 1) * N1 // P) for i in range(P)]
        how = "%d strips of cell rows" % P
    jobs = [[] for _ in range(P)]
    for b, (x0, x1_, y0, y1) in enumerate(boxes):
        m = (kx >= x0) & (kx < x1_) & (ky >= y0) & (ky < y1)
        sub = {kk: np.ascontiguousarray(parts[kk][m]) for kk in ("x1", "x2", "U1", "U2", "U3")}
        sub["x1"] = sub["x1"] - x0 * dx
        sub["x2"] = sub["x2"] - y0 * dy
        c = cfg.copy()
        c.n_cells[0], c.n_cells[1] = x1_ - x0, y1 - y0
        c.length[0], c.length[1] = (x1_ - x0) * dx, (y1 - y0) * dy
        c.max_particles = int(m.sum())
        jobs[b % P].append((c.as_dict(), sub))
    return [j for j in jobs if j], how


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import multiprocessing as mp

    import mcpm
    cores = os.cpu_count() or 1
    P = max(1, min(cores, 64))
    cfg, parts, desc = build_workload(args)
    cfg.precision = mcpm.FP64
    Ntot = len(parts["x2"])
    jobs, how = _ref_split(cfg, parts, P)
    P = len(jobs)
    ctx = mp.get_context("spawn")
    pools = [ctx.Pool(1, initializer=_ref_worker_init, initargs=(j,)) for j in jobs]
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
            "config": dict(desc, precision="fp64 (reference CPU path: the plain force, no learned part)"),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": P, "kind": "port",
                             "sample": "the full workload (%d particles) split into %s, one oracle process per "
                                       "core, every step" % (Ntot, how)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mcpm", choices=["mcpm", "reference"])
    ap.add_argument("--workload", default="surrogate16m",
                    choices=["surrogate16m", "uneven16m", "esmc6m", "dsmc6m", "slab1m", "vlasov16m"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--horizon", type=int, default=2000,
                    help="last accuracy checkpoint of the learned-force workload (steps)")
    ap.add_argument("--no-side", action="store_true", help="skip the side workloads (configs 2-4)")
    ap.add_argument("--profile-case", choices=["uneven", "esmc", "slab", "vlasov", "surrogate"],
                    help="run a small case of a workload for an ncu capture and exit (no JSON line)")
    ap.add_argument("--cells", type=int, default=160, help="grid size n of --profile-case")
    ap.add_argument("--fp64", action="store_true", help="FP64 state for --profile-case")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.warmup < 3 and args.impl == "mcpm":
        args.warmup = 3
    if args.impl == "reference":
        # one reference step of a 16M workload is ~0.5-5 s on 16 cores
        args.steps = min(args.steps, 60 if args.workload not in ("surrogate16m", "vlasov16m") else 4)
        args.warmup = min(args.warmup, 3)
        run_reference(args)
    else:
        run_mcpm(args)


if __name__ == "__main__":
    main()
