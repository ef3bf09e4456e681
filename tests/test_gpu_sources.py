"""Particle sources and sinks on the GPU vs the FP64 oracle, through the C-ABI.

Bar: particle counts and append order bit-exact (the draws are the same
Philox words on both sides); new and surviving particle states within rel
1e-12 (positions are bit-exact; velocities of new ions go through the
device's cos/sin/log); moments within the atomic-deposit tolerance.
"""
import numpy as np
import pytest

from conftest import relerr
from helpers import make_hybrid, oracle_for
from swap_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = 1e-12
DEPOSIT_TOL = 1e-13


def _pair(extra=3000, **over):
    h = make_hybrid(extra=extra, **over)
    return h, oracle_for(h)


def _same_particles(h, o, tol=TOL):
    h.sync_to_host()
    N = int(o.ni_tot[0])
    assert int(h.ni_tot[0]) == N
    for n in ("xp", "vp", "vp1"):
        assert relerr(getattr(h, n)[:N], getattr(o, n)[:N]) <= tol, n
    for n in ("mrat", "beta_p"):
        assert np.array_equal(getattr(h, n)[:N], getattr(o, n)[:N]), n
    return N


def _cloud(h, **kw):
    q = h.coords
    d = dict(cloud_N0=2.0, cloud_r0=2.0, cloud_x=float(q.qx[5]), cloud_y=float(q.qy[3]), cloud_z=float(q.qz[4]),
             nu_ion=0.7, mrat_heavy=1.0 / 16, beta_heavy=1.0)
    d.update(kw)
    return d


def test_ionize_sw_mp_matches_oracle():
    h, o = _pair()
    cfg = h.cfg
    src = abi.make_sources(seed=11, ndot=37.4 / (cfg.dt * cfg.beta * cfg.nodes[2]), vsw=3.0, beta_pu=1.0,
                           mrat_pu=0.5, delz_ref=1.0)
    N0 = int(h.ni_tot[0])
    for x in (h, o):
        x.set_sources(src)
        x.Ionize_sw_mp(x.np, x.vp, x.vp1, x.xp, 4, x.input_p, x.up)
    N = _same_particles(h, o)
    assert N == N0 + 37
    assert relerr(h.np, o.np) < DEPOSIT_TOL and relerr(h.up, o.up) < DEPOSIT_TOL


@pytest.mark.parametrize("step", [0, 1, 5])
def test_inflow_x_matches_oracle(step):
    h, o = _pair()
    src = abi.make_sources(seed=3, x_open=1, inflow_ppc=8, inflow_vth=0.5, inflow_ux=4.0, inflow_uy=0.3)
    N0 = int(h.ni_tot[0])
    for x in (h, o):
        x.set_sources(src)
        x.inflow_x(step)
    assert _same_particles(h, o) > N0


def test_ionize_cloud_matches_oracle():
    h, o = _pair()
    src = abi.make_sources(seed=9, **_cloud(h))
    N0 = int(h.ni_tot[0])
    for x in (h, o):
        x.set_sources(src)
        x.ionize_cloud(5)
    assert _same_particles(h, o, tol=0.0) > N0  # no transcendental on this path: bit-exact


def test_res_chex_matches_oracle():
    h, o = _pair()
    src = abi.make_sources(seed=4, **_cloud(h, cloud_N0=20.0), cx_a=2.0, cx_b=0.1)
    for x in (h, o):
        x.mrat[:7] = 1.0 / 16
        x.set_sources(src)
    h.mark_host_dirty()
    n_h = h.res_chex(h.xp, h.vp, 2)
    n_o = o.res_chex(o.xp, o.vp, 2)
    assert n_h == n_o and n_h > 0
    _same_particles(h, o, tol=0.0)


def test_remove_ion_shifts_particles_and_weights():
    h, o = _pair(extra=0)
    h.get_interp_weights(h.xp)
    h.remove_ion(h.xp, h.vp, h.vp1, 5)
    o.remove_ion(o.xp, o.vp, o.vp1, 5)
    _same_particles(h, o, tol=0.0)
    # the device ijkp/wght moved with the particles (gutsp.f:33-39): no re-weighting before the deposit
    h.update_np(h.np)
    o.get_interp_weights(o.xp)
    o.update_np(o.np)
    h.sync_to_host()
    assert relerr(h.np, o.np) < DEPOSIT_TOL
    with pytest.raises(abi.SwapError):
        h.remove_ion(h.xp, h.vp, h.vp1, 0)


def test_open_x_move_and_outflow_match_oracle():
    h, o = _pair(u=(30.0, 0.0, 0.0))
    N0 = int(h.ni_tot[0])
    for x in (h, o):
        x.set_sources(abi.make_sources(x_open=1))
        x.move_ion_half(x.xp, x.vp, x.vp1, x.input_p)
        x.remove_outflow_x()
    assert 0 < _same_particles(h, o, tol=0.0) < N0


def test_fused_steps_with_every_source():
    h, o = _pair(extra=6000)
    cfg = h.cfg
    src = abi.make_sources(seed=21, ndot=10.0 / (cfg.dt * cfg.beta * cfg.nodes[2]), vsw=2.0, beta_pu=1.0,
                           mrat_pu=0.5, delz_ref=1.0, x_open=1, inflow_ppc=4, inflow_vth=0.5, inflow_ux=2.0,
                           **_cloud(h, cloud_N0=0.5, nu_ion=0.2), cx_a=2.0, cx_b=0.1)
    for x in (h, o):
        x.set_sources(src, 0)
    counts = []
    for _ in range(3):
        h.ion_step()
        o.ion_step()
        counts.append(_same_particles(h, o))
    assert len(set(counts)) > 1
    assert h.chex_count() == o.chex_count() > 0


def test_source_errors_leave_the_context_usable():
    h, o = _pair(extra=5)
    with pytest.raises(abi.SwapError):
        h.inflow_x(0)  # no swap_set_sources yet
    cfg = h.cfg
    h.set_sources(abi.make_sources(seed=1, ndot=40.0 / (cfg.dt * cfg.beta * cfg.nodes[2]), vsw=1.0, beta_pu=1.0,
                                   mrat_pu=1.0, delz_ref=1.0))
    N0 = int(h.ni_tot[0])
    with pytest.raises(abi.SwapError):
        h.Ionize_sw_mp(h.np, h.vp, h.vp1, h.xp, 0, h.input_p, h.up)  # 40 ions, room for 5
    assert int(h.ni_tot[0]) == N0
    h.get_interp_weights(h.xp)
    h.update_np(h.np)
