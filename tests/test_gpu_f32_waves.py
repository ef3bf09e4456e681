"""The FP32 form over 2000 steps against the oracle's wave physics.

The parallel-wave start of tests/test_oracle_waves.py (a quiet lattice of
cold ions, a circularly polarized B perturbation along B0) run through the
FP32 form: the whistler rate with the ions held still, and the ion-cyclotron
and whistler frequencies with mobile ions, must match what the FP64 oracle
measures on the same start (the wave is uniform across the box, so the
oracle's 4-cell-wide box stands for the FP32 form's 8-cell-wide one).  Bars:
1e-5 relative for the Hall rate, 2e-4 for the two branches.
"""
import numpy as np
import pytest

from swap_gb300.hybrid import Hybrid, config
from test_oracle_waves import NZ_CELLS, _roots, _wave

pytestmark = pytest.mark.gpu


def _f32_wave(steps, every, eps=0.02, frozen=False):
    q = np.array([0.25, 0.75])
    cfg = config(0, cells=(8, 8, NZ_CELLS), ppc=8, vth=0.0, u=(0.0, 0.0, 0.0), nu=0.0 if frozen else 0.002)
    h = Hybrid(cfg, ni_max=cfg.n_particles)
    co = h.coords
    k = 2.0 * np.pi / (NZ_CELLS * co.delz)
    ncx, ncy, ncz = cfg.cells
    px, py, pz = np.meshgrid(np.arange(ncx), np.arange(ncy), np.arange(ncz), indexing="ij")
    x = np.concatenate([np.stack([co.qx[px.ravel()] + a * co.dx, co.qy[py.ravel()] + b * co.dy,
                                  co.qz[pz.ravel()] + c * co.delz], axis=1) for a in q for b in q for c in q])
    n = len(x)
    h.ni_tot[0] = n
    h.xp[:n] = x
    h.vp[:n] = 0.0
    h.vp1[:n] = 0.0
    if frozen:
        h.mrat[:n] = 0.0
    zb = co.qz + 0.5 * co.delz
    for name in ("b1", "b12", "b1p2", "bt"):
        f = getattr(h, name)
        f[..., 0] = eps * np.cos(k * zb)[None, None, :]
        f[..., 1] = eps * np.sin(k * zb)[None, None, :]
    h.mark_host_dirty()
    nz = cfg.nodes[2]
    a = []
    h.f32_begin()
    for _ in range(steps // every):
        h.f32_run(every)
        h.f32_end()  # the state back in FP64 (exact: 48-bit B, FP32 offsets)
        h.sync_to_host(h.b1)
        b = (h.b1[1:-1, 1:-1, 1:nz - 1, 0] + 1j * h.b1[1:-1, 1:-1, 1:nz - 1, 1]).mean(axis=(0, 1))
        a.append(np.sum(b * np.exp(-1j * k * zb[1:nz - 1])))
        h.f32_begin()
    h.close()
    return np.array(a), cfg.dt * every, k


def test_f32_whistler_rate_with_the_ions_held_still():
    a, dt, k = _f32_wave(steps=400, every=10, frozen=True)
    rate = np.polyfit(dt * np.arange(1, len(a) + 1), np.unwrap(np.angle(a)), 1)[0]
    ao, dto, _ = _wave(steps=400, every=10, frozen=True)
    rate_o = np.polyfit(dto * np.arange(1, len(ao) + 1), np.unwrap(np.angle(ao)), 1)[0]
    assert abs(rate - rate_o) < 1e-5 * rate_o, (rate, rate_o)


def test_f32_ion_cyclotron_and_whistler_branches_match_oracle():
    a, dt, _ = _f32_wave(steps=2000, every=10)
    ao, dto, _ = _wave(steps=2000, every=10)
    om = _roots(a, dt)
    om_o = _roots(ao, dto)
    for x, y in zip(om, om_o):
        assert abs(x - y) < 2e-4 * abs(y), (om, om_o)
