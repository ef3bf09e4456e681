"""Particle sources and sinks in the FP32 form, against the FP64 oracle.

The FP32 form draws new ions from the same Philox words as the oracle, so
the numbers created by Ionize_sw_mp, the x inflow and the cloud ionization
are identical; the outflow count depends on FP32 positions and res_chex
draws by sorted index, so those agree statistically.  Bars: ion counts equal
(periodic x) or within 2 (open x), every ion inside the box, B within rel-L2
1e-5 and moments within rel-L2 1e-3 of the oracle after three steps, charge
exchanges within five standard deviations (density then within 3e-2, since
different ions exchange).
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for
from swap_gb300 import abi

pytestmark = pytest.mark.gpu


def _pair(src_kw, steps=3, cells=(16, 8, 8), ppc=16, seed=7, extra=40000):
    h = make_hybrid(cells=cells, ppc=ppc, seed=seed, db=0.0, extra=extra)
    o = oracle_for(h)
    src = abi.make_sources(**src_kw)
    h.set_sources(src, 0)
    o.set_sources(src, 0)
    h.f32_begin()
    h.f32_run(steps)
    h.f32_end()
    h.sync_to_host()
    for _ in range(steps):
        o.ion_step()
    return h, o


def _inside(h, N):
    c = h.coords
    q = (c.qx, c.qy, c.qz)
    x = h.xp[:N]
    return all(np.all((x[:, m] > q[m][0]) & (x[:, m] <= q[m][-2])) for m in range(3))


def test_f32_open_x_inflow_outflow_tracks_oracle():
    h0 = make_hybrid(cells=(16, 8, 8), ppc=16, seed=7, db=0.0)
    n0 = int(h0.ni_tot[0])
    cfg = h0.cfg
    h, o = _pair(dict(seed=5, x_open=1, inflow_ppc=16, inflow_vth=cfg.vth, inflow_ux=cfg.u[0]))
    N, No = int(h.ni_tot[0]), int(o.ni_tot[0])
    assert No != n0  # ions entered and left
    assert abs(N - No) <= 2
    assert _inside(h, N)
    assert rel_l2(h.b1, o.b1) < 1e-5
    assert rel_l2(h.np, o.np) < 1e-3
    assert rel_l2(h.up, o.up) < 1e-3


def test_f32_ionize_and_cloud_counts_equal_oracle():
    h0 = make_hybrid(cells=(16, 8, 8), ppc=16, seed=7, db=0.0)
    cfg = h0.cfg
    q = h0.coords
    kw = dict(seed=9, ndot=5.0 / (cfg.dt * cfg.beta * cfg.nodes[2]), vsw=1.0, beta_pu=1.0, mrat_pu=0.5,
              delz_ref=1.0, cloud_N0=2.0, cloud_r0=2.0, cloud_x=float(q.qx[8]), cloud_y=float(q.qy[4]),
              cloud_z=float(q.qz[4]), nu_ion=0.2, mrat_heavy=1.0 / 16, beta_heavy=1.0)
    h, o = _pair(kw)
    N = int(o.ni_tot[0])
    assert int(h.ni_tot[0]) == N > int(h0.ni_tot[0])
    assert _inside(h, N)
    for m in (1.0, 0.5, 1.0 / 16):  # species populations are exact
        assert np.count_nonzero(h.mrat[:N] == m) == np.count_nonzero(o.mrat[:N] == m), m
    assert rel_l2(h.np, o.np) < 1e-3
    assert rel_l2(h.b1, o.b1) < 1e-5


def test_f32_charge_exchange_rate_matches_oracle():
    h0 = make_hybrid(cells=(16, 8, 8), ppc=16, seed=7, db=0.0)
    q = h0.coords
    kw = dict(seed=4, cloud_N0=1.0, cloud_r0=3.0, cloud_x=float(q.qx[8]), cloud_y=float(q.qy[4]),
              cloud_z=float(q.qz[4]), mrat_heavy=1.0 / 16, beta_heavy=1.0, cx_a=1.0, cx_b=0.1)
    h, o = _pair(kw)
    nh, no = h.chex_count(), o.chex_count()
    assert no > 50
    assert abs(nh - no) < 5 * np.sqrt(no) + 2
    N = int(h.ni_tot[0])
    assert N == int(o.ni_tot[0])
    heavy = h.mrat[:N] == 1.0 / 16
    assert np.count_nonzero(heavy) == nh  # every exchanged ion is heavy
    assert rel_l2(h.np, o.np) < 3e-2  # different ions exchange (draws follow the sorted order)


def test_f32_begin_end_with_sources_keeps_the_count():
    h = make_hybrid(cells=(16, 8, 8), ppc=8, seed=2, db=0.0, extra=10000)
    n0 = int(h.ni_tot[0])
    h.set_sources(abi.make_sources(seed=1, x_open=1, inflow_ppc=8, inflow_vth=0.5, inflow_ux=2.0))
    h.f32_begin()  # stages the first step's inflow
    h.f32_end()    # the step was not taken: those ions are dropped
    h.sync_to_host()
    assert int(h.ni_tot[0]) == n0
