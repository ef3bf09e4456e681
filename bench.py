"""Throughput of SWAP's hybrid PIC ion step on GB300: ion particle-steps/s.

A step is one full ion step of maind.f:385-479 (three particle passes with
four moment deposits, the field predictor-corrector with its subcycles and
the final half move) over every particle of the workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision f64] [--config 1]

With the FP32 form the line also carries "accuracy": the FP32 form and the
FP32 form with the surrogate against the FP64 drop-in after --acc-steps ion
steps of the periodic 64x32x32 box (B and n_p rel-L2, energy drift), and
"surrogate": the same step timed
with the learned field surrogate (trained on pairs collected from plain
steps of the same run) in place of the field subcycles, judged against them
every few steps.  --surrogate off skips it.

Rank 0 prints one JSON line.  --impl reference times the reference's CPU
path (the C++ restatement in oracle/, the reference itself has no Fortran
compiler here) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ion particle-steps/s on 1 GB300"
UNIT = "particle-steps/s"


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "25"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait for its first sample so that
        # the samples cover the (short) timed region
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value: float, ws: int) -> float:
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch
        import torch.distributed as dist

        dist.barrier()
        torch.cuda.synchronize()


# Algorithmic (compulsory) HBM bytes per unit for the FP64 drop-in kernels:
# each reads/writes its particle arrays once; gathered field values and the
# deposit targets are node data that stay in L2 and are not counted.
# Units: particles for particle kernels, interior nodes for stencils.
KERNEL_BYTES_F64 = {
    "interp_weights": 24 + 12 + 64,            # read xp; write ijk, wght
    "deposit_np": 12 + 64 + 8,                 # read ijk, wght, beta_p
    "deposit_u": 12 + 64 + 8 + 48,             # + two velocity arrays (worst case of the modes)
    "get_Ep": 12 + 64 + 8 + 24,                # read ijk, wght, mrat; write Ep
    "vplus_vminus": 12 + 64 + 8 + 24 + 24 + 48,  # + Ep, vp; write v+, v-
    "vp_final": 24 + 24 + 24 + 48,
    "move_half": 24 + 24 + 24,
}


# Algorithmic bytes per unit for the FP32 form (particles: cell 4 + offsets 12
# + v 12 + vp1 12 + species 1 = 41 B of state).
KERNEL_BYTES_F32 = {
    "f32_P1": 41,                # read state (deposit only)
    "f32_P2": 29,                # read cell, offsets, v, species
    "f32_P3": 29 + 40 + 4,       # + write v, vp1, cell, offsets and the sort's direction/rank
    "f32_sort_scatter": 41 + 4 + 41,
    "f32_sort_prep": 4 + 4,
}
# DRAM bytes per particle that ncu measured for these kernels
# (dram__bytes_read.sum + dram__bytes_write.sum over one launch at 128x64x64
# cells, 16 ppc, 8.4M particles; profiles/k_pass_fp32_128x64x64_16ppc.md and
# profiles/k_sort_scatter_fp32_128x64x64_16ppc.md); the roofline's traffic is
# this figure times the particles of a launch.
KERNEL_TRAFFIC_F32 = {"f32_P1": 42.8, "f32_P2": 32.4, "f32_P3": 64.8, "f32_sort_scatter": 86.0}
# per interior node (FP32 fields, double-float B levels of 8 B per component)
NODE_BYTES_F32 = {
    "f32_curlB": 12 + 4 + 12,
    "f32_aj_ct_pred": 12 + 4 + 12 + 12 + 12,        # read dB, np, up; write aj, ct
    "f32_aj_ct_corr": 12 + 4 + 12 + 12 + 12,
    "f32_bstep_pred": 12 + 12 + 4 + 24 + 12 + 12,  # read ct, aj, nu, B, dB1; write dB(m+1/2)
    "f32_bstep_corr": 12 + 12 + 4 + 24 + 24 + 12,    # read ct, aj, nu, B; write B, dB
    "f32_kit": 36 + 32,
    "f32_node_sum": 16 * 2 + 16,
    "f32_ct_up": 16 + 12,
}


def cpu_sample_oracle(cfg_full, steps: int, threads: int):
    """Time the oracle's FP64 ion step on a sub-box of the workload (same ppc,
    same physics), on `threads` host threads.  Returns (particle-steps/s, info)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    from swap_gb300.grid import grd6_setup, grd7
    from swap_gb300.hybrid import RunConfig

    cells = (64, 32, 32)
    src = dict(cfg_full.sources)
    if "cloud_x" in src:  # keep the cloud at the centre of the sub-box
        src.update(cloud_x=cells[0] / 2 + 1.0, cloud_y=cells[1] / 2 + 1.0, cloud_z=cells[2] / 2 + 1.0)
    cfg = RunConfig(name="cpu sample", cells=cells, ppc=cfg_full.ppc, vth=cfg_full.vth, u=cfg_full.u,
                    dt=cfg_full.dt, ntsub=cfg_full.ntsub, nu=cfg_full.nu, seed=cfg_full.seed, sources=src)
    nx, ny, nz = cfg.nodes
    n = cfg.ni_max_hint()
    n_load = cfg.n_particles

    class Host:  # arrays in the layout the oracle binds
        pass

    h = Host()
    h.cfg = cfg
    h.ni_max = n
    co = grd7(nx, ny, nz)
    f3 = lambda: np.zeros((n, 3), order="F")
    h.xp, h.vp, h.vp1, h.Ep, h.vplus, h.vminus = (f3() for _ in range(6))
    h.mrat, h.beta_p = np.ones(n), np.ones(n)
    h.ni_tot = np.array([n_load], dtype=np.int32)
    for k, v in grd6_setup(co, cfg.b0, cfg.nu).items():
        setattr(h, k, v)
    # the same stratified Maxwellian load as the GPU run, made by the product loader
    from swap_gb300 import abi
    import ctypes as C

    lib = abi.load()
    dims = abi.Dims(nx, ny, nz, 0, n)
    cc = abi.Coords(*[abi.dptr(getattr(co, a)) for a in co.ARRAYS])
    spec = abi.LoadSpec(cfg.seed, 0, cfg.ppc, cfg.vth, *cfg.u, 1.0, 1.0)
    cnt = C.c_int64()
    abi.check(lib, None, lib.swap_load_maxwellian_host(C.byref(dims), C.byref(cc), C.byref(spec), abi.dptr(h.xp),
                                                        abi.dptr(h.vp), abi.dptr(h.vp1), abi.dptr(h.mrat),
                                                        abi.dptr(h.beta_p), 0, C.byref(cnt)))
    o = pyoracle.from_hybrid_arrays(h, precision="f64", nthreads=threads)
    if cfg.sources:
        o.set_sources(cfg.make_sources(), 0)
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    info = {"sample": f"{cells[0]}x{cells[1]}x{cells[2]}-cell sub-box of the workload at {cfg.ppc} ppc "
                      f"({n_load:,} ions), {steps} FP64 ion steps of the oracle"
                      + (" with the workload's sources and sinks" if cfg.sources else ""),
            "seconds": dt}
    return n_load * steps / dt, info


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU path (restated) on the host cores
# ---------------------------------------------------------------------------

def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from swap_gb300.hybrid import config

    cfg = config(args.config)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample_oracle(cfg, 1, threads)
    vals = []
    info = None
    for _ in range(args.steps):
        v, info = cpu_sample_oracle(cfg, 1, threads)
        vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference",
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cfg.n_particles / value * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": cfg.name, "cells": list(cfg.cells), "ppc": cfg.ppc, "ions": cfg.n_particles,
                   "subcycles": cfg.ntsub},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": info["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def run_surrogate(h, args, N, ws):
    """The FP32 step with the learned field surrogate in place of the
    subcycles: collect training pairs from plain steps, train, attach with a
    judge every few steps, then time K steps the same way as the plain run."""
    import ctypes as C

    from swap_gb300.hybrid import Surrogate, attach_surrogate, surrogate_stats

    lib, ctx = h.lib, h.ctx
    h.f32_begin()
    net = Surrogate(seed=11, max_samples=args.sur_collect)
    t0 = time.perf_counter()
    net.collect(h, args.sur_collect)
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = net.train(args.sur_epochs, lr=2e-3)
    t_train = time.perf_counter() - t0
    attach_surrogate(h, net, judge_every=args.sur_judge, bound=args.sur_bound)
    for _ in range(args.warmup):
        h.f32_run(1)
    lib.swap_profile_reset(ctx)
    lib.swap_profile_enable(ctx, 1)
    before = surrogate_stats(h)
    barrier(ws)
    ms = C.c_double()
    h._check(lib.swap_timer_start(ctx))
    h.f32_run(args.steps)
    h._check(lib.swap_timer_stop(ctx, C.byref(ms)))
    lib.swap_profile_enable(ctx, 0)
    t_ms = barrier_max(ms.value, ws)
    st = surrogate_stats(h)
    names = (C.c_char_p * 64)()
    tot = (C.c_double * 64)()
    cnt = (C.c_int64 * 64)()
    n = C.c_int32()
    lib.swap_profile_read(ctx, 64, names, tot, cnt, C.byref(n))
    field = {names[i].decode(): tot[i] / args.steps for i in range(min(n.value, 64))
             if names[i].decode().startswith(("f32_sur", "f32_aj_ct", "f32_bstep", "f32_courant"))}
    attach_surrogate(h, None)
    h.f32_end()
    net.close()
    return {"ms_per_step": t_ms / args.steps, "value": N * args.steps * ws / (t_ms / 1e3), "unit": UNIT,
            "network": "4 periodic 3x3x3 conv layers 8-32-32-32-3, GELU, BF16 on tcgen05, FP32 accumulate",
            "collect_steps": args.sur_collect, "collect_s": t_collect, "train_epochs": args.sur_epochs,
            "train_s": t_train, "train_loss": loss, "judge_every": args.sur_judge, "bound": args.sur_bound,
            "net_steps": st["net_steps"] - before["net_steps"], "judged": st["judged"] - before["judged"],
            "fallbacks": st["fallbacks"] - before["fallbacks"], "last_err_b": st["err_b"],
            "last_err_db": st["err_db"], "field_ms_per_step": field}


def run_accuracy(args):
    """The error of the FP32 form and of the FP32 form with the surrogate
    against the FP64 GPU drop-in, after the same number of ion steps from the
    same seeded load: the periodic 64x32x32-cell box at 16 ppc (no sources,
    so the total energy is conserved up to the scheme's own drift)."""
    import numpy as np

    from swap_gb300.hybrid import Hybrid, Surrogate, attach_surrogate, config, surrogate_stats

    cfg = config(0)
    S = args.acc_steps

    def fresh():
        h = Hybrid(cfg, ni_max=cfg.n_particles)
        h.load_maxwellian(seed=cfg.seed)
        h.sync_to_device()
        return h

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    def total(e):  # kinetic + |b1 - b0|^2 field energy (part_init.f:69-84)
        return float(e[0] + e[1])

    t0 = time.perf_counter()
    h64 = fresh()
    e0 = h64.energy()
    h64.run(S)
    e64 = h64.energy()
    h64.sync_to_host()
    ref = {k: getattr(h64, k).copy() for k in ("b1", "b0", "np", "E")}
    h64.close()
    out = {"workload": f"{cfg.name} (periodic, 1,048,576 ions), {S} ion steps from the same seeded load",
           "fp64_energy_drift": (total(e64) - total(e0)) / total(e0)}
    for form in ("fp32", "fp32_surrogate"):
        h = fresh()
        h.f32_begin()
        ea = h.f32_energy()
        if form == "fp32":
            h.f32_run(S)
        else:
            ncol = min(24, S // 2)
            net = Surrogate(seed=7, max_samples=ncol)
            net.collect(h, ncol)
            net.train(12, lr=2e-3)
            attach_surrogate(h, net, judge_every=8, bound=1e-3)
            h.f32_run(S - ncol)
            st = surrogate_stats(h)
            out["surrogate_steps"] = {"collected": ncol, "network": st["net_steps"], "judged": st["judged"],
                                      "fallbacks": st["fallbacks"], "bound": 1e-3}
        eb = h.f32_energy()
        h.f32_end()
        h.sync_to_host()
        out[form] = {"b_rel_l2": rel(h.b1, ref["b1"]), "db_rel_l2": rel(h.b1 - h.b0, ref["b1"] - ref["b0"]),
                     "np_rel_l2": rel(h.np, ref["np"]), "energy_drift": (total(eb) - total(ea)) / total(ea),
                     "energy_vs_fp64": (total(eb) - total(e64)) / total(e64)}
        if form == "fp32_surrogate":
            attach_surrogate(h, None)
            net.close()
        h.close()
    out["seconds"] = time.perf_counter() - t0
    return out


def run_ours(args):
    ws, rank, local = dist_env()
    import torch

    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from swap_gb300.hybrid import Hybrid, config

    cfg = config(args.config)
    if args.cells or args.ppc:
        over = {}
        if args.cells:
            over["cells"] = tuple(args.cells)
        if args.ppc:
            over["ppc"] = args.ppc
        over["name"] = f"{cfg.name} (resized to {over.get('cells', cfg.cells)} cells, {over.get('ppc', cfg.ppc)} ppc)"
        cfg = config(args.config, **over)
    # Each rank runs its own replica of the workload: the particle-decomposed
    # exchange (an allreduce of the moments after each deposit) is not built.
    h = Hybrid(cfg, ni_max=cfg.ni_max_hint(), pinned=True)
    t_load = time.perf_counter()
    h.load_maxwellian(seed=cfg.seed + 1000 * rank)
    t_load = time.perf_counter() - t_load
    src = cfg.make_sources()
    if src is not None:
        src.seed += 1000 * rank
        h.set_sources(src, 0)
    h.sync_to_device()

    f32 = args.precision == "f32"
    if f32:
        h.f32_begin()
        run, count = h.f32_run, h.f32_count
    else:
        run, count = h.run, (lambda: int(h.ni_tot[0]))
    for _ in range(args.warmup):
        run(1)
    lib, ctx = h.lib, h.ctx
    n_before = count()

    # ---- timed region: K steps, device-resident, CUDA events on the library stream
    lib.swap_profile_reset(ctx)
    lib.swap_profile_enable(ctx, 1)
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    import ctypes as C

    ms = C.c_double()
    h._check(lib.swap_timer_start(ctx))
    run(args.steps)
    h._check(lib.swap_timer_stop(ctx, C.byref(ms)))
    clk = clocks.stop()
    # with inflow and outflow the count drifts a little: use the mean
    N = (n_before + count()) // 2
    lib.swap_profile_enable(ctx, 0)
    t_ms = barrier_max(ms.value, ws)

    names = (C.c_char_p * 64)()
    tot = (C.c_double * 64)()
    cnt = (C.c_int64 * 64)()
    n = C.c_int32()
    lib.swap_profile_read(ctx, 64, names, tot, cnt, C.byref(n))
    prof = {names[i].decode(): (tot[i], cnt[i]) for i in range(min(n.value, 64))}
    kernels = {k: v for k, v in prof.items() if not k.startswith("cuda")}
    launches = int(sum(v[1] for v in kernels.values()))
    top = max(kernels.items(), key=lambda kv: kv[1][0])
    top_name, (top_ms, top_n) = top
    part_bytes = KERNEL_BYTES_F32 if f32 else KERNEL_BYTES_F64
    node_bytes = NODE_BYTES_F32 if f32 else {}
    nodes_int = (cfg.nodes[0] - 2) * (cfg.nodes[1] - 2) * (cfg.nodes[2] - 2)
    units = N if top_name in part_bytes else nodes_int
    per_unit = part_bytes.get(top_name, node_bytes.get(top_name, 0))
    avg_s = top_ms / 1e3 / max(top_n, 1)
    achieved = per_unit * units / avg_s / 1e9 if per_unit else None
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)

    # ---- end to end through the C-ABI with host buffers (pinned): the whole
    # state starts in host memory, K steps each followed by the per-step
    # Energy_diag read (maind.f:391-393,503-505), the state ends in host memory.
    # Every array is marked host-current; the entries move what they read
    # (the particles x, v, vp1, mrat, beta_p and the fields b0, b1, b12, np,
    # nu) and sync_to_host brings back what they wrote.  In the FP32 form the
    # particle vectors cross NVLink-C2C inside the conversion kernels (host-
    # direct mode).  The library counts the bytes moved either way.
    state_arrays = [h.xp, h.vp, h.vp1, h.mrat, h.beta_p]
    in_fields = [getattr(h, a) for a in ("b0", "b1", "b12", "b1p2", "bt", "btc", "np", "up", "aj", "E", "nu")]
    if f32:
        h.f32_end()
    h.sync_to_host()
    barrier(ws)
    torch.cuda.synchronize()
    h.transfer_bytes(reset=True)
    w0 = time.perf_counter()
    for a in state_arrays + in_fields:
        h.mark_host_dirty(a)
    if f32:
        h.f32_begin()
        for _ in range(args.steps):
            h.f32_run(1)
            h.f32_energy()
        h.f32_end()
    else:
        h.sync_to_device()
        for _ in range(args.steps):
            h.run(1)
            h.energy()
    h.sync_to_host()
    torch.cuda.synchronize()
    e2e_s = barrier_max(time.perf_counter() - w0, ws)
    h2d_bytes, d2h_bytes = h.transfer_bytes(reset=True)
    d2h_bytes += 32 * args.steps  # the energy reads
    del state_arrays

    value = N * args.steps * ws / (t_ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if f32 else "f64", "data": "synthetic (seeded stratified Maxwellian load, normalized units)",
        "config": {"workload": cfg.name, "cells": list(cfg.cells), "ppc": cfg.ppc, "ions": N,
                   "subcycles": cfg.ntsub,
                   "boundary": "x inflow/outflow, periodic y,z" if cfg.sources.get("x_open") else "periodic",
                   "precision_form": "FP32 form (int32 cell + FP32 offset, FP32 moments, double-float B)" if f32
                   else "FP64 drop-in",
                   "l2": "inputs larger than L2 (particle state %.1f GB)" % (N * (41 if f32 else 72) / 1e9),
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU"},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": (KERNEL_TRAFFIC_F32[top_name] * units if f32 and top_name in KERNEL_TRAFFIC_F32
                                 else None),
                     "traffic_source": "ncu DRAM bytes per particle at 128x64x64 cells x 16 ppc, times the "
                                       "particles of one launch" if f32 and top_name in KERNEL_TRAFFIC_F32 else None,
                     "peak_source": "measured" if peaks else "fallback",
                     "bytes_per_unit": per_unit, "units_per_launch": units,
                     "note": None if f32 else "FP64 kernels on GB300 are bound by the FP64 pipe, not HBM"},
        "kernels_ms_per_step": {k: v[0] / args.steps for k, v in sorted(kernels.items(), key=lambda kv: -kv[1][0])},
        "e2e": {"value": N * args.steps * ws / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d_bytes / args.steps,
                "d2h_bytes_per_step": d2h_bytes / args.steps},
        "load_seconds": t_load,
    }
    if f32 and args.surrogate != "off":
        try:
            line["surrogate"] = run_surrogate(h, args, N, ws)
        except Exception as e:  # the headline stands without it
            line["surrogate"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and f32 and args.acc_steps > 0:
        try:
            line["accuracy"] = run_accuracy(args)
        except Exception as e:  # the headline stands without it
            line["accuracy"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and not args.no_cpu_baseline:
        v, info = cpu_sample_oracle(cfg, 1, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": info["sample"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    h.close()
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--surrogate", default="on", choices=["on", "off"],
                    help="also time the FP32 step with the learned field surrogate")
    ap.add_argument("--sur-collect", type=int, default=24, help="plain steps collected as training pairs")
    ap.add_argument("--sur-epochs", type=int, default=12)
    ap.add_argument("--sur-judge", type=int, default=8, help="judge the surrogate every this many steps")
    ap.add_argument("--sur-bound", type=float, default=1e-3, help="judge bound on the relative B error")
    ap.add_argument("--acc-steps", type=int, default=1000,
                    help="ion steps of the accuracy comparison against the FP64 drop-in (0 skips it)")
    ap.add_argument("--cells", type=int, nargs=3, default=None, help="override the workload's cells (profiling)")
    ap.add_argument("--ppc", type=int, default=None, help="override particles per cell (profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
