"""Throughput of SWAP's hybrid PIC ion step on GB300: ion particle-steps/s.

A step is one full ion step of maind.f:379-484 (the sources, three particle
passes with four moment deposits, the field predictor-corrector with its
subcycles, the final half move and the sinks) over every ion of the workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision f64] [--config 1]

The headline times the FP32 form on the 256x128x128-cell, 32-ppc workload
(134M ions, x inflow/outflow).  The line also carries
  "e2e":       the same steps through the C-ABI with host buffers;
  "surrogate": the step with the learned field surrogate in place of the
               subcycles, judged against them every few steps;
  "fp64":      the FP64 GPU drop-in (swap_run) on the same workload;
  "accuracy":  the FP32 form and the FP32 form with the surrogate against the
               FP64 drop-in after --acc-steps ion steps of the periodic
               64x32x32 box;
  "accuracy_configs": the pickup-ion workloads (256x128x128 and 512x256x256
               cells at 16 ppc, neutral cloud and charge exchange) at their
               stated sizes, FP32 form against FP64 drop-in, with the FP32
               form's ions per brick;
  "cpu_baseline": one full-size ion step of the oracle on the host cores.

--impl reference times the reference's CPU path on the host cores: the C++
restatement in oracle/ at the reference's own precision (FP32), on the whole
workload, one full ion step per timed step, with the FP64 oracle beside it.
Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
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
# cells, 16 ppc, 8.4M particles); the roofline's traffic is this figure times
# the particles of a launch.
KERNEL_TRAFFIC_F32 = {"f32_P1": 44.4, "f32_P2": 34.1, "f32_P3": 70.5, "f32_sort_scatter": 86.0}
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


def host_available() -> int:
    """MemAvailable of /proc/meminfo in bytes (0 if unreadable)."""
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def room_for(host_bytes: float, dev_bytes: float = 0.0):
    """None if the host and the current GPU have the room, else the reason."""
    avail = host_available()
    if avail and avail < host_bytes:
        return f"needs {host_bytes / 1e9:.0f} GB of host memory, {avail / 1e9:.0f} GB available"
    if dev_bytes:
        import torch

        free, _ = torch.cuda.mem_get_info()
        if free < dev_bytes:
            return f"needs {dev_bytes / 1e9:.0f} GB of device memory, {free / 1e9:.0f} GB free"
    return None


def config_line(cfg, ions, f32=True):
    """The workload's description in a bench line."""
    return {"workload": cfg.name, "cells": list(cfg.cells), "ppc": cfg.ppc, "ions": int(ions),
            "subcycles": cfg.ntsub,
            "boundary": "x inflow/outflow, periodic y,z" if cfg.sources.get("x_open") else "periodic",
            "precision_form": ("FP32 form (int32 cell + FP32 offset, FP32 moments, double-float B)" if f32
                               else "FP64 drop-in"),
            "l2": "inputs larger than L2 (particle state %.1f GB)" % (ions * (41 if f32 else 72) / 1e9)}


def oracle_run(cfg, precision: str, warmup: int, steps: int, threads: int) -> dict:
    """The reference's CPU path (the oracle's restatement) on the whole
    workload: the oracle's own seeded load, `warmup` untimed ion steps, then
    `steps` ion steps each timed by the wall clock.  Nothing of the product
    is loaded.  Particle-steps are the mean of each step's ion count before
    and after it (inflow and outflow change the count a little)."""
    if str(ROOT / "oracle") not in sys.path:
        sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    # bytes per ion of capacity: the bound particle arrays plus the oracle's
    # ijkp, weights, scratch velocities and push work arrays
    why = room_for(cfg.ni_max_hint() * (112 if precision == "f32" else 224) * 1.15)
    if why:
        return {"skipped": why, "precision": precision}
    t0 = time.perf_counter()
    o = pyoracle.standalone(cfg, precision=precision, nthreads=threads)
    t_load = time.perf_counter() - t0
    for _ in range(warmup):
        o.ion_step()
    units, secs, per_step = 0.0, 0.0, []
    for _ in range(steps):
        n0 = int(o.ni_tot[0])
        t = time.perf_counter()
        o.ion_step()
        dt = time.perf_counter() - t
        units += 0.5 * (n0 + int(o.ni_tot[0]))
        secs += dt
        per_step.append(round(dt, 3))
    o.close()
    del o
    return {"value": units / secs, "unit": UNIT, "ms_per_step": secs / steps * 1e3, "ions": units / steps,
            "steps": steps, "warmup": warmup, "load_s": t_load, "step_s": per_step, "threads": threads,
            "precision": precision}


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU path (restated) on the host cores
# ---------------------------------------------------------------------------

def run_reference(args):
    """The oracle at the reference's own precision (FP32: makefile:1 builds
    SWAP with -real-size 32) on the whole workload, every timed step a full
    ion step over all of its ions; the FP64 oracle beside it on the same
    workload for a few steps."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from swap_gb300.hybrid import config

    cfg = config(args.config)
    threads = os.cpu_count() or 1
    try:
        r = oracle_run(cfg, "f32", args.warmup, args.steps, threads)
    except Exception as e:
        r = {"skipped": f"the oracle failed: {type(e).__name__}: {e}"}
    if "skipped" in r:
        print(json.dumps({"impl": "reference", "unavailable": r["skipped"]}), flush=True)
        return 0
    sample = (f"the whole workload ({r['ions']:,.0f} ions), one full FP32 ion step of the oracle per timed step "
              f"after {args.warmup} warm-up steps, OpenMP over {threads} host threads")
    line = {
        "impl": "reference",
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded stratified Maxwellian load, normalized units)",
        "config": dict(config_line(cfg, r["ions"]), precision_form="the oracle at the reference's precision (FP32)",
                       parallelism=f"{threads} host threads"),
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_s": r["step_s"], "load_s": r["load_s"],
    }
    if args.ref_fp64_steps > 0:
        try:
            line["fp64"] = oracle_run(cfg, "f64", 1, args.ref_fp64_steps, threads)
        except Exception as e:
            line["fp64"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def train_surrogate(args, base):
    """The learned field surrogate, trained on pairs that the plain subcycles
    produce in randomized runs (swap_gb300.surrogate_data: upstream speed
    1-6 v_A, beta 0.1-2, an open x axis in half of the runs and a neutral
    cloud of radius 2-10 cells in half) of a box of --sur-cells cells that
    keeps the workload's B0, ion step, subcycles and particles per cell.
    Adam with the library's warm-up, then --sur-epochs epochs in three stages
    of falling learning rate.  Returns the network and what the training did."""
    from swap_gb300.hybrid import Surrogate
    from swap_gb300.surrogate_data import collect_randomized

    cells = (args.sur_cells,) * 3
    net = Surrogate(seed=11, max_samples=args.sur_runs * args.sur_pairs, curl_weight=args.sur_curl)
    t0 = time.perf_counter()
    collect_randomized(net, base, runs=args.sur_runs, pairs_per_run=args.sur_pairs, warmup=3, cells=cells, seed=5,
                       mixed=True)
    t_collect = time.perf_counter() - t0
    l0 = net.loss()
    t0 = time.perf_counter()
    E = max(args.sur_epochs, 3)
    done, loss = 0, l0
    for upto, lr in ((E // 4, 1e-3), (E * 5 // 8, 5e-4), (E, 1.5e-4)):
        if upto > done:
            loss = net.train(upto - done, lr=lr)
            done = upto
    t_train = time.perf_counter() - t0
    nl = len(net.layers)
    info = {"network": f"{nl} periodic 3x3x3 conv layers {Surrogate.NIN}-" + "-".join([str(net.layers[0][1])] * (nl - 1))
                       + "-3, GELU, BF16 on tcgen05, FP32 accumulate; predicts the subcycles' mean E minus the "
                       "plain E at the step's start from B, u_p, n_p, p_e, that E and B - b12",
            "training": f"{args.sur_runs} randomized runs of {cells[0]}x{cells[1]}x{cells[2]} cells at "
                        f"{base.ppc} ppc, {args.sur_pairs} pairs each (upstream speed 1-6 v_A, beta 0.1-2, "
                        f"open or periodic x, with or without a cloud of radius 2-10 cells)",
            "loss": "mean squared normalised E error" + (f" + {args.sur_curl} x relative curl error"
                                                         if args.sur_curl else ""),
            "pairs": net.samples(), "collect_s": t_collect, "train_epochs": E, "train_s": t_train,
            "loss_before": l0, "train_loss": loss}
    return net, info


def run_surrogate(h, args, N, ws, net, info):
    """The FP32 step with the learned field surrogate in place of the
    subcycles, judged against them every --sur-judge steps: K steps timed the
    same way as the plain run."""
    import ctypes as C

    from swap_gb300.hybrid import attach_surrogate, surrogate_stats

    lib, ctx = h.lib, h.ctx
    h.f32_begin()
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
    return dict(info, ms_per_step=t_ms / args.steps, value=N * args.steps * ws / (t_ms / 1e3), unit=UNIT,
                judge_every=args.sur_judge, bound=args.sur_bound,
                net_steps=st["net_steps"] - before["net_steps"], judged=st["judged"] - before["judged"],
                fallbacks=st["fallbacks"] - before["fallbacks"], last_err_b=st["err_b"], last_err_db=st["err_db"],
                field_ms_per_step=field)


def run_accuracy(args, net=None):
    """The error of the FP32 form and of the FP32 form with the surrogate
    against the FP64 GPU drop-in, after the same number of ion steps from the
    same seeded load: the periodic 64x32x32-cell box at 16 ppc (no sources,
    so the total energy is conserved up to the scheme's own drift).  net: the
    trained surrogate (None skips that leg)."""
    import numpy as np

    from swap_gb300.hybrid import Hybrid, attach_surrogate, config, surrogate_stats

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
        if form == "fp32_surrogate" and net is None:
            continue
        h = fresh()
        h.f32_begin()
        ea = h.f32_energy()
        if form == "fp32":
            h.f32_run(S)
        else:
            attach_surrogate(h, net, judge_every=args.sur_judge, bound=args.sur_bound)
            h.f32_run(S)
            st = surrogate_stats(h)
            out["surrogate_steps"] = {"network": st["net_steps"], "judged": st["judged"],
                                      "fallbacks": st["fallbacks"], "bound": args.sur_bound,
                                      "judge_every": args.sur_judge, "last_err_b": st["err_b"],
                                      "last_err_db": st["err_db"]}
            attach_surrogate(h, None)
        eb = h.f32_energy()
        h.f32_end()
        h.sync_to_host()
        out[form] = {"b_rel_l2": rel(h.b1, ref["b1"]), "db_rel_l2": rel(h.b1 - h.b0, ref["b1"] - ref["b0"]),
                     "np_rel_l2": rel(h.np, ref["np"]), "energy_drift": (total(eb) - total(ea)) / total(ea),
                     "energy_vs_fp64": (total(eb) - total(e64)) / total(e64)}
        h.close()
    out["seconds"] = time.perf_counter() - t0
    return out


def brick_load(starts: np.ndarray) -> dict:
    """Ions per 4x4x4-cell brick (one CTA of the particle passes each) and
    per cell, from the FP32 state's key starts (key = brick * 64 + cell)."""
    per_cell = np.diff(starts)
    per_brick = starts[64::64] - starts[:-1:64]
    return {"brick_mean": float(per_brick.mean()), "brick_max": int(per_brick.max()),
            "brick_min": int(per_brick.min()), "brick_max_over_mean": float(per_brick.max() / per_brick.mean()),
            "cell_min": int(per_cell.min()), "cell_max": int(per_cell.max()),
            "cell_p99": float(np.percentile(per_cell, 99))}


def run_compare(n: int, steps: int, cx: bool = True, marks=()) -> dict:
    """A named workload at its stated size, run `steps` ion steps from the
    same seeded load by the FP64 GPU drop-in and by the FP32 form: B, B - b0
    and n_p rel-L2 of the FP32 form against the FP64 run, each run's energy
    drift, the ion counts, both step times, and the FP32 form's load per
    brick.  With cx=False charge exchange is off: the FP32 form draws it per
    sorted ion and the FP64 path per array index, so with it on the two runs
    are different draws of the same process and their difference holds that
    sampling noise as well as the FP32 rounding.  marks: steps at which both
    runs' total energies are also recorded."""
    import ctypes as C

    from swap_gb300.hybrid import Hybrid, config

    cfg = config(n)
    if not cx:
        src = dict(cfg.sources)
        src.update(cx_a=0.0, cx_b=0.0)
        cfg = config(n, sources=src)
    NM = cfg.ni_max_hint(steps + 4)
    # the FP64 context holds 260 B of device memory per ion of capacity
    # (particles, weights, cell indices, push and compaction work arrays);
    # the host keeps 88 B (x, v, vp1, mrat, beta_p)
    why = room_for(NM * 88 * 1.3, NM * 270)
    if why:
        return {"workload": cfg.name, "skipped": why}

    def fresh():
        h = Hybrid(cfg, ni_max=NM, work_arrays=False)
        h.load_maxwellian(seed=cfg.seed)
        h.set_sources(cfg.make_sources(), 0)
        h.sync_to_device()
        return h

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    def timed(h, fn):
        ms = C.c_double()
        h._check(h.lib.swap_timer_start(h.ctx))
        fn()
        h._check(h.lib.swap_timer_stop(h.ctx, C.byref(ms)))
        return ms.value

    def total(e):
        return float(e[0] + e[1])

    marks = sorted(m for m in set(marks) if 0 < m < steps) + [steps]

    def segments(run, energy):
        """Run to each mark; the summed time and the total energy at each."""
        ms, done, es = 0.0, 0, []
        for m in marks:
            ms += timed(h, lambda: run(m - done))
            done = m
            es.append(total(energy()))
        return ms, es

    t0 = time.perf_counter()
    h = fresh()
    n0 = int(h.ni_tot[0])
    e0 = h.energy()
    ms64, es64 = segments(h.run, h.energy)
    e64 = h.energy()
    h.sync_to_host()
    ref = {"b1": h.b1.copy(), "b0": h.b0.copy(), "np": h.np.copy()}
    n64 = int(h.ni_tot[0])
    h.close()
    del h
    h = fresh()
    h.f32_begin()
    ea = h.f32_energy()
    ms32, es32 = segments(h.f32_run, h.f32_energy)
    eb = h.f32_energy()
    load = brick_load(h.f32_key_starts())
    n32 = h.f32_count()
    h.f32_end()
    h.sync_to_host()
    out = {"workload": cfg.name + ("" if cx else " (charge exchange off)"), "steps": steps, "ions_start": n0,
           "ions_fp64": n64, "ions_fp32": n32,
           "fp64_ms_per_step": ms64 / steps, "fp32_ms_per_step": ms32 / steps,
           "fp32_over_fp64_speed": ms64 / ms32,
           "b_rel_l2": rel(h.b1, ref["b1"]), "db_rel_l2": rel(h.b1 - h.b0, ref["b1"] - ref["b0"]),
           "np_rel_l2": rel(h.np, ref["np"]),
           "fp64_energy_drift": (total(e64) - total(e0)) / total(e0),
           "fp32_energy_drift": (total(eb) - total(ea)) / total(ea),
           "energy_vs_fp64": (total(eb) - total(e64)) / total(e64),
           "energy_marks": [{"step": m, "fp64_drift": (a - total(e0)) / total(e0), "fp32_vs_fp64": (b - a) / a}
                            for m, a, b in zip(marks, es64, es32)],
           "fp32_load_per_brick": load}
    h.close()
    del h
    out["seconds"] = time.perf_counter() - t0
    return out


def run_fp64_leg(h, steps: int, warmup: int) -> dict:
    """The FP64 GPU drop-in (swap_run) on the same workload and state:
    `warmup` untimed steps, then `steps` timed by CUDA events."""
    import ctypes as C

    h.sync_to_device()
    for _ in range(warmup):
        h.run(1)
    n0 = int(h.ni_tot[0])
    ms = C.c_double()
    h._check(h.lib.swap_timer_start(h.ctx))
    h.run(steps)
    h._check(h.lib.swap_timer_stop(h.ctx, C.byref(ms)))
    N = 0.5 * (n0 + int(h.ni_tot[0]))
    return {"ms_per_step": ms.value / steps, "value": N * steps / (ms.value / 1e3), "unit": UNIT, "steps": steps,
            "warmup": warmup, "ions": N, "dtype": "f64"}


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
        h._check(h.lib.swap_f32_set_moment_sums(h.ctx, 1 if args.moment_sums == "exact" else 0))
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

    value = N * args.steps * ws / (t_ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if f32 else "f64", "data": "synthetic (seeded stratified Maxwellian load, normalized units)",
        "config": dict(config_line(cfg, N, f32), parallelism=f"replicas x{ws}" if ws > 1 else "1 GPU"),
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
    net = None
    if f32 and args.surrogate != "off":
        try:
            net, info = train_surrogate(args, cfg)
            line["surrogate"] = run_surrogate(h, args, N, ws, net, info)
        except Exception as e:  # the headline stands without it
            line["surrogate"] = {"error": f"{type(e).__name__}: {e}"}
    if ws > 1:  # per-GPU characterisations: the 1-GPU line carries them
        line["single_gpu_legs"] = "the FP64, accuracy and CPU-baseline legs run in the 1-GPU line only"
    if f32 and args.fp64_steps > 0 and ws == 1:
        # the plain FP64 GPU drop-in on the same workload: the other side of
        # the metric's FP32-versus-FP64 comparison
        try:
            line["fp64"] = run_fp64_leg(h, args.fp64_steps, 2)
            line["fp64"]["fp32_over_fp64_speed"] = line["fp64"]["ms_per_step"] / line["ms_per_step"]
        except Exception as e:
            line["fp64"] = {"error": f"{type(e).__name__}: {e}"}
    h.close()
    del h, state_arrays, in_fields
    import gc

    gc.collect()
    if ws == 1:
        run_accuracy_legs(args, line, net)
    if net is not None:
        net.close()
    if ws == 1 and not args.no_cpu_baseline:
        try:
            r = oracle_run(cfg, "f32", 1, 1, os.cpu_count() or 1)
        except Exception as e:  # the headline stands without it
            r = {"skipped": f"{type(e).__name__}: {e}"}
        line["cpu_baseline"] = {"skipped": r["skipped"]} if "skipped" in r else {"value": r["value"], "unit": UNIT, "cores": r["threads"], "kind": "port",
                                "sample": f"one full FP32 ion step of the oracle over the whole workload "
                                          f"({r['ions']:,.0f} ions) after one warm-up step"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def run_conv_only(spec) -> int:
    """The surrogate's tensor-core convolution alone on random BF16 data, for
    profiling one launch in isolation: spec = CIN COUT NX NY NZ [REPEATS].
    CIN, COUT are 16 or 32 (the network's layer shapes); NX*NY*NZ must be a
    multiple of 128, and NX a multiple of 128 selects the line-ring form."""
    import torch

    from swap_gb300 import abi

    if len(spec) not in (5, 6):
        print(run_conv_only.__doc__)
        return 2
    cin, cout, nx, ny, nz = spec[:5]
    reps = spec[5] if len(spec) == 6 else 2
    lib = abi.load()
    V = nx * ny * nz
    X = torch.randn(V, cin, device="cuda").to(torch.bfloat16)
    W = (0.1 * torch.randn(27, cout, cin, device="cuda")).to(torch.bfloat16)
    b = torch.zeros(cout, device="cuda")
    Y = torch.empty(V, cout, dtype=torch.bfloat16, device="cuda")
    for _ in range(reps):
        r = lib.swap_conv3_check(nx, ny, nz, cin, cout, X.data_ptr(), W.data_ptr(), b.data_ptr(), Y.data_ptr(), None,
                                 1)
        if r:
            print(f"swap_conv3_check returned {r}")
            return 1
    torch.cuda.synchronize()
    print("ok")
    return 0


def run_accuracy_legs(args, line, net=None):
    """The error legs of the line: the 64x32x32 box (FP64, FP32, FP32 with
    the surrogate), then the configs --acc-configs at their stated sizes."""
    if args.precision == "f32" and args.acc_steps > 0:
        try:
            line["accuracy"] = run_accuracy(args, net)
        except Exception as e:  # the headline stands without it
            line["accuracy"] = {"error": f"{type(e).__name__}: {e}"}
    steps = {1: args.acc1_steps, 2: args.acc2_steps, 3: args.acc3_steps}
    for n in [int(x) for x in args.acc_configs.split(",") if x.strip()]:
        for cx in {"both": [True, False], "on": [True], "off": [False]}[args.acc_cx]:
            key = f"config{n}" + ("" if cx else "_no_cx")
            try:
                line.setdefault("accuracy_configs", {})[key] = run_compare(
                    n, steps.get(n, 20), cx=cx, marks=[int(x) for x in args.acc_marks.split(",") if x.strip()])
            except Exception as e:
                line.setdefault("accuracy_configs", {})[key] = {"error": f"{type(e).__name__}: {e}"}
            import gc

            gc.collect()


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
    ap.add_argument("--sur-runs", type=int, default=12, help="randomized runs that give the training pairs")
    ap.add_argument("--sur-pairs", type=int, default=6, help="training pairs per run")
    ap.add_argument("--sur-cells", type=int, default=64, help="cells per axis of the training runs' box")
    ap.add_argument("--sur-epochs", type=int, default=80)
    ap.add_argument("--sur-curl", type=float, default=1.0, help="weight of the curl term in the surrogate's loss")
    ap.add_argument("--sur-judge", type=int, default=8, help="judge the surrogate every this many steps")
    ap.add_argument("--sur-bound", type=float, default=1e-3, help="judge bound on the relative B error")
    ap.add_argument("--acc-steps", type=int, default=1000,
                    help="ion steps of the accuracy comparison against the FP64 drop-in (0 skips it)")
    ap.add_argument("--acc-configs", default="2,3",
                    help="workloads run at their stated size by both the FP64 drop-in and the FP32 form")
    ap.add_argument("--acc1-steps", type=int, default=20, help="ion steps of the 256x128x128 H+ comparison")
    ap.add_argument("--acc2-steps", type=int, default=100, help="ion steps of the 256x128x128 pickup-ion comparison")
    ap.add_argument("--acc3-steps", type=int, default=20, help="ion steps of the 512x256x256 pickup-ion comparison")
    ap.add_argument("--acc-marks", default="", help="steps at which the comparisons also record both energies")
    ap.add_argument("--acc-cx", default="both", choices=["both", "on", "off"],
                    help="comparisons with charge exchange as stated (on), off (no sampling difference), or both")
    ap.add_argument("--only-accuracy", action="store_true", help="run the accuracy legs alone")
    ap.add_argument("--conv-only", type=int, nargs="+", default=None, metavar="N",
                    help="CIN COUT NX NY NZ [REPEATS]: the surrogate's convolution alone (profiling)")
    ap.add_argument("--moment-sums", default="exact", choices=["exact", "plain"],
                    help="the FP32 form's moment sums: exact fixed-point accumulation, or plain FP32 atomics")
    ap.add_argument("--fp64-steps", type=int, default=5, help="timed steps of the FP64 GPU drop-in leg (0 skips)")
    ap.add_argument("--ref-fp64-steps", type=int, default=2,
                    help="reference arm: timed full-size steps of the FP64 oracle beside the FP32 one (0 skips)")
    ap.add_argument("--cells", type=int, nargs=3, default=None, help="override the workload's cells (profiling)")
    ap.add_argument("--ppc", type=int, default=None, help="override particles per cell (profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.conv_only:
        return run_conv_only(args.conv_only)
    if args.only_accuracy:
        import torch

        torch.cuda.set_device(0)
        line = {"accuracy_only": True}
        run_accuracy_legs(args, line)
        print(json.dumps(line), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
