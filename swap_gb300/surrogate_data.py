"""Training pairs for the learned field surrogate from randomized runs.

The network stands in for the field subcycles of one ion step (maind.f:420-476)
and is trained on pairs that the plain subcycles produce.  To cover the
conditions it will meet, the pairs come from many short runs of a small
box, each with its own upstream state: flow speed drawn uniform in 1-6 v_A
and plasma beta in 0.1-2; an open x axis with inflow in half of the runs
(periodic otherwise), and in half a neutral cloud (ionization and charge
exchange, chem_rates.f:346-432, 805-843) of radius drawn in 2-10 cells at
the box centre (mixed=False: every run has both).  The uniform, periodic
boxes matter: trained on cloud runs alone, the network's judged B error on
a source-free box was five times larger.  Every run keeps the target
workload's B0, ion step, subcycle count and particles per cell, so the
network learns the step it will replace.  All computation is the library's
FP32 form on the GPU; this module only draws the parameters.
"""
from __future__ import annotations

import numpy as np

from .hybrid import Hybrid, RunConfig, config


def run_config(base: RunConfig, rng: np.random.Generator, cells=(64, 64, 64), index: int = 0,
               mixed: bool = True) -> RunConfig:
    """One randomized run around `base`: v_A = B0 (n0 = 1); the load's velocity
    spread sigma = vth/sqrt(2) per component gives beta = vth^2 / v_A^2.
    mixed: the cloud and the open x axis are each present in half of the
    runs (periodic, source-free boxes are among the workloads too);
    otherwise every run has both."""
    va = base.b0 / np.sqrt(base.n0)
    u = float(rng.uniform(1.0, 6.0)) * va
    beta = float(rng.uniform(0.1, 2.0))
    vth = float(np.sqrt(beta)) * va
    r0 = float(rng.uniform(2.0, 10.0))
    seed = int(rng.integers(1, 2**31 - 1))
    cloud = (not mixed) or bool(rng.integers(0, 2))
    x_open = (not mixed) or bool(rng.integers(0, 2))
    cx, cy, cz = (c / 2.0 + 1.0 for c in cells)
    src = dict(seed=seed)
    if x_open:
        src.update(x_open=1, inflow_ppc=base.ppc, inflow_vth=vth, inflow_ux=u, inflow_uy=0.0, inflow_uz=0.0)
    if cloud:
        src.update(cloud_N0=1000.0, cloud_r0=r0, cloud_x=cx, cloud_y=cy, cloud_z=cz, nu_ion=1e-3,
                   mrat_heavy=1.0 / 16.0, beta_heavy=1.0, cx_a=1.0, cx_b=0.1)
    what = ("open x" if x_open else "periodic") + (f", cloud r0 {r0:.1f}" if cloud else "")
    return config(0, name=f"surrogate training run {index}: u {u:.2f}, beta {beta:.2f}, {what}",
                  cells=tuple(cells), ppc=base.ppc, vth=vth, u=(u, 0.0, 0.0), b0=base.b0, n0=base.n0, dt=base.dt,
                  ntsub=base.ntsub, nu=base.nu, seed=seed, sources=src if (x_open or cloud) else {})


def collect_randomized(net, base: RunConfig, runs: int, pairs_per_run: int, warmup: int = 4,
                       cells=(64, 64, 64), seed: int = 0, mixed: bool = True) -> list:
    """Add runs * pairs_per_run training pairs to `net` (a hybrid.Surrogate):
    each run loads its box, takes `warmup` plain FP32 steps so the upstream
    flow and the pickup ions develop, then collects one pair per step.
    Returns the runs' parameters."""
    rng = np.random.default_rng(seed)
    drawn = []
    for r in range(runs):
        cfg = run_config(base, rng, cells, r, mixed=mixed)
        h = Hybrid(cfg, ni_max=cfg.ni_max_hint(warmup + pairs_per_run + 4), work_arrays=False)
        try:
            h.load_maxwellian()
            if cfg.sources:
                h.set_sources(cfg.make_sources(), 0)
            h.sync_to_device()
            h.f32_begin()
            h.f32_run(warmup)
            net.collect(h, pairs_per_run)
        finally:
            h.close()
        drawn.append({"name": cfg.name, "u": cfg.u[0], "vth": cfg.vth, "seed": cfg.seed})
    return drawn
