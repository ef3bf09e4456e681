"""The oracle's own particle load and its multi-threaded step (CPU only).

The CPU reference arm of the benchmark builds its workload with nothing but
the oracle: its stratified Maxwellian load must give the same seeded ions as
the product's host loader, and the oracle's step on several host threads must
give the one-thread step's results (node loops and the outflow compaction are
thread-count independent; deposits sum per-thread grids, so they agree to
rounding).
"""
import ctypes as C

import numpy as np
import pytest

from swap_gb300 import abi
from swap_gb300.grid import grd7
from swap_gb300.hybrid import config


def _product_load(cfg, ni_max):
    lib = abi.load()
    nx, ny, nz = cfg.nodes
    co = grd7(nx, ny, nz)
    dims = abi.Dims(nx, ny, nz, 0, ni_max)
    cc = abi.Coords(*[abi.dptr(getattr(co, a)) for a in co.ARRAYS])
    spec = abi.LoadSpec(cfg.seed, 0, cfg.ppc, cfg.vth, *cfg.u, 1.0, 1.0)
    f3 = lambda: np.zeros((ni_max, 3), order="F")
    xp, vp, vp1 = f3(), f3(), f3()
    mrat, beta_p = np.zeros(ni_max), np.zeros(ni_max)
    cnt = C.c_int64()
    abi.check(lib, None, lib.swap_load_maxwellian_host(C.byref(dims), C.byref(cc), C.byref(spec), abi.dptr(xp),
                                                        abi.dptr(vp), abi.dptr(vp1), abi.dptr(mrat),
                                                        abi.dptr(beta_p), 0, C.byref(cnt)))
    return xp, vp, vp1, mrat, beta_p, cnt.value


@pytest.mark.parametrize("cells", [(8, 8, 12), (10, 6, 7)])  # brick order and plain cell order
def test_oracle_load_equals_product_load(oracle_mod, cells):
    cfg = config(0, cells=cells, ppc=5, seed=17)
    n = cfg.n_particles
    xp, vp, vp1, mrat, beta_p, cnt = _product_load(cfg, n + 3)
    assert cnt == n
    o = oracle_mod.standalone(cfg, ni_max=n + 3, precision="f64", nthreads=3)
    assert int(o.ni_tot[0]) == n
    for a, b in ((o.xp, xp), (o.vp, vp), (o.vp1, vp1), (o.mrat, mrat), (o.beta_p, beta_p)):
        assert np.array_equal(a[:n], b[:n])
    o32 = oracle_mod.standalone(cfg, ni_max=n + 3, precision="f32", nthreads=2)
    for a, b in ((o32.xp, xp), (o32.vp, vp)):
        assert np.array_equal(a[:n], b[:n].astype(np.float32))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_oracle_threads_do_not_change_the_step(oracle_mod, precision):
    # open x (inflow and outflow): the multi-threaded compaction must keep the
    # same ions in the same order
    cfg = config(1, cells=(16, 8, 8), ppc=6, seed=5)
    one = oracle_mod.standalone(cfg, precision=precision, nthreads=1)
    many = oracle_mod.standalone(cfg, precision=precision, nthreads=4)
    for _ in range(3):
        one.ion_step()
        many.ion_step()
    n = int(one.ni_tot[0])
    assert int(many.ni_tot[0]) == n
    tol = 1e-11 if precision == "f64" else 2e-5
    for name in ("xp", "vp", "vp1"):
        a, b = getattr(many, name)[:n], getattr(one, name)[:n]
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), name
    for name in ("b1", "np", "up", "E"):
        a, b = getattr(many, name), getattr(one, name)
        assert np.linalg.norm(a - b) <= tol * np.linalg.norm(b), name
