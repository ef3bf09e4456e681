"""Shared set-up for the parity tests: a GPU Hybrid and an FP64 oracle built
from the same seeded load and the same perturbed initial field."""
from __future__ import annotations

import numpy as np

from swap_gb300.hybrid import Hybrid, config

FIELDS = ("b0", "b1", "b12", "b1p2", "bt", "btc", "np", "up", "aj", "E", "nu")
PARTS = ("xp", "vp", "vp1", "Ep", "vplus", "vminus", "mrat", "beta_p")


def periodic_np(a: np.ndarray) -> np.ndarray:
    """Ghost planes copy their interior images (boundary.f:9-52) -- numpy."""
    for ax in range(3):
        n = a.shape[ax]
        sl = [slice(None)] * a.ndim
        src = [slice(None)] * a.ndim
        sl[ax], src[ax] = 0, n - 2
        a[tuple(sl)] = a[tuple(src)]
        sl[ax], src[ax] = n - 1, 1
        a[tuple(sl)] = a[tuple(src)]
    return a


def make_hybrid(cells=(12, 6, 8), ppc=4, seed=3, extra=7, db=0.05, **over) -> Hybrid:
    cfg = config(0, cells=cells, ppc=ppc, seed=seed, **over)
    h = Hybrid(cfg, ni_max=cfg.n_particles + extra)
    h.load_maxwellian()
    if db:
        rng = np.random.default_rng(seed + 100)
        pert = db * rng.standard_normal(h.b1.shape)
        b = h.b0 + pert
        periodic_np(b)
        for n in ("b1", "b12", "b1p2", "bt"):
            getattr(h, n)[...] = b
    h.mark_host_dirty()
    return h


def oracle_for(h, nthreads=1):
    import pyoracle

    return pyoracle.from_hybrid_arrays(h, precision="f64", nthreads=nthreads)


def copy_state(dst_h, src_o):
    """Make the GPU's host arrays equal to the oracle's and mark them dirty."""
    for n in FIELDS + PARTS:
        getattr(dst_h, n)[...] = getattr(src_o, n)
    dst_h.ni_tot[0] = src_o.ni_tot[0]
    dst_h.mark_host_dirty()
