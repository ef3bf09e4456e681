"""Shared set-up for the parity tests: a GPU Hybrid and an FP64 oracle built
from the same seeded load and the same perturbed initial field."""
from __future__ import annotations

import ctypes as C

import numpy as np

from swap_gb300 import abi
from swap_gb300.grid import grd6_setup, grd7
from swap_gb300.hybrid import Hybrid, RunConfig, config

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


# ---- host-only state for the CPU tests (no GPU context) ----

class Host:
    """The arrays of maind.f:38-70 for a RunConfig, on the host."""

    def __init__(self, cfg, ni_max=None, load=True, coords=None):
        self.cfg = cfg
        nx, ny, nz = cfg.nodes
        n = cfg.n_particles if ni_max is None else ni_max
        self.ni_max = n
        self.coords = coords if coords is not None else grd7(nx, ny, nz)
        f3 = lambda: np.zeros((n, 3), order="F")
        self.xp, self.vp, self.vp1, self.Ep, self.vplus, self.vminus = (f3() for _ in range(6))
        self.mrat, self.beta_p = np.ones(n), np.ones(n)
        self.ni_tot = np.array([0], dtype=np.int32)
        for k, v in grd6_setup(self.coords, cfg.b0, cfg.nu).items():
            setattr(self, k, v)
        if load:
            self.load()

    def load(self, **over):
        cfg = self.cfg
        lib = abi.load()
        nx, ny, nz = cfg.nodes
        dims = abi.Dims(nx, ny, nz, 0, self.ni_max)
        co = abi.Coords(*[abi.dptr(getattr(self.coords, a)) for a in self.coords.ARRAYS])
        spec = abi.LoadSpec(over.get("seed", cfg.seed), 0, over.get("ppc", cfg.ppc), over.get("vth", cfg.vth),
                            *over.get("u", cfg.u), 1.0, 1.0)
        cnt = C.c_int64()
        abi.check(lib, None, lib.swap_load_maxwellian_host(C.byref(dims), C.byref(co), C.byref(spec),
                                                            abi.dptr(self.xp), abi.dptr(self.vp), abi.dptr(self.vp1),
                                                            abi.dptr(self.mrat), abi.dptr(self.beta_p), 0,
                                                            C.byref(cnt)))
        self.ni_tot[0] = cnt.value


def oracle(h, precision="f64"):
    import pyoracle

    return pyoracle.from_hybrid_arrays(h, precision=precision)


def small(**kw):
    base = dict(name="kat", cells=(8, 6, 6), ppc=4, seed=7)
    base.update(kw)
    return RunConfig(**base)


def fortran_records(path):
    """The records of a Fortran sequential unformatted file (4-byte markers)."""
    import struct

    out = []
    with open(path, "rb") as f:
        data = f.read()
    o = 0
    while o < len(data):
        (n,) = struct.unpack_from("<i", data, o)
        rec = data[o + 4:o + 4 + n]
        (n2,) = struct.unpack_from("<i", data, o + 4 + n)
        assert n == n2, (path, o, n, n2)
        out.append(rec)
        o += 8 + n
    return out
