"""Known-answer tests of the field and particle step together: small-amplitude
circularly polarized waves along B0 in a cold plasma.

Normalized units (d_i = 1, Omega_i = 1, v_A = 1).  For b = dBx + i dBy with
space dependence e^{ikz} and time dependence e^{-i omega t}, the cold-fluid
hybrid model (massless electrons, no pressure term) gives

    omega^2 + k^2 omega - k^2 = 0,  omega = k (-k/2 +- sqrt(1 + k^2/4)),

the ion-cyclotron branch omega_L > 0 and the whistler branch omega_R < 0;
with the ions held still the Hall term alone gives omega = -k^2.  On the grid
the curl-curl operator sees k_eff^2 = 4 sin^2(k/2).

Measured on the oracle (the reference's step restated; the GPU forms match it
to rounding, tests/test_gpu_parity.py):
  - ions held still (mrat = 0): the whistler rate equals -k_eff^2 to 1e-8;
  - mobile ions: the product of the two roots equals -k_eff^2 to 0.3%, and
    the roots themselves lie within 2.5% of the fluid values at 32 cells per
    wavelength;
  - their sum (the Hall splitting) falls short of the fluid -k^2 by an amount
    first order in dz/d_i, independent of k, the time step and the subcycle
    count: the ions' velocity reaches the grid (deposit) and comes back
    (gather) smoothed over a cell, a correction of the same order k^2 as the
    Hall term when dz ~ d_i.  With one ion per cell: 0.75, 0.87, 0.94 of -k^2
    at dz = 1, 1/2, 1/4 d_i.
"""
import numpy as np

from helpers import Host, oracle, small
from swap_gb300.grid import grd7

NZ_CELLS = 32


def _wave(steps, every, eps=0.02, frozen=False, nz_cells=NZ_CELLS, delz=1.0, q=(0.25, 0.75)):
    """B-only circularly polarized start on a quiet lattice (q: the ions'
    places inside a cell, per axis; the box is nz_cells * delz = 32 d_i long);
    the spatial Fourier coefficient of dBx + i dBy at k, sampled every
    `every` steps.  beta = ppc for a cell of volume delz makes the density
    n = 1/delz, and then d_i v_A = 1/n and v_A^2 = 1/n."""
    q = np.asarray(q)
    cfg = small(cells=(4, 4, nz_cells), ppc=len(q) ** 3, vth=0.0, u=(0.0, 0.0, 0.0),
                nu=0.0 if frozen else 0.002)
    nx, ny, nz = cfg.nodes
    h = Host(cfg, load=False, coords=grd7(nx, ny, nz, delz=delz))
    co = h.coords
    k = 2.0 * np.pi / (nz_cells * co.delz)
    ncx, ncy, ncz = cfg.cells
    px, py, pz = np.meshgrid(np.arange(ncx), np.arange(ncy), np.arange(ncz), indexing="ij")
    x = np.concatenate([np.stack([co.qx[px.ravel()] + a * co.dx, co.qy[py.ravel()] + b * co.dy,
                                  co.qz[pz.ravel()] + c * co.delz], axis=1) for a in q for b in q for c in q])
    n = len(x)
    assert n == cfg.n_particles
    h.ni_tot[0] = n
    h.xp[:n] = x
    if frozen:
        h.mrat[:] = 0.0  # no force on the ions: they stay at rest, up = 0
    zb = co.qz + 0.5 * co.delz  # dBx and dBy sit half a cell up in z from their node
    for name in ("b1", "b12", "b1p2", "bt"):
        f = getattr(h, name)
        f[..., 0] = eps * np.cos(k * zb)[None, None, :]
        f[..., 1] = eps * np.sin(k * zb)[None, None, :]
    o = oracle(h)
    nz = cfg.nodes[2]
    a = []
    for s in range(1, steps + 1):
        o.ion_step()
        if s % every == 0:
            b = (o.b1[1:-1, 1:-1, 1:nz - 1, 0] + 1j * o.b1[1:-1, 1:-1, 1:nz - 1, 1]).mean(axis=(0, 1))
            a.append(np.sum(b * np.exp(-1j * k * zb[1:nz - 1])))
    return np.array(a), cfg.dt * every, k


def test_whistler_rate_with_the_ions_held_still():
    a, dt, k = _wave(steps=400, every=1, frozen=True)
    rate = np.polyfit(dt * np.arange(1, len(a) + 1), np.unwrap(np.angle(a)), 1)[0]
    k_eff2 = (2.0 * np.sin(k / 2.0)) ** 2
    assert abs(rate - k_eff2) < 1e-6 * k_eff2  # phase turns at +k_eff^2: omega = -k_eff^2
    assert abs(abs(a[-1]) / abs(a[0]) - 1.0) < 1e-9  # no resistivity: no damping


def test_ion_cyclotron_and_whistler_branches():
    # both branches from one start; two-term linear prediction (Prony) of the
    # samples gives their frequencies
    a, dt, k = _wave(steps=2000, every=10)
    lhs = np.stack([a[1:-1], a[:-2]], axis=1)
    c, *_ = np.linalg.lstsq(lhs, a[2:], rcond=None)
    roots = np.roots([1.0, -c[0], -c[1]])
    om_r, om_l = sorted(-np.angle(roots) / dt)
    root = np.sqrt(1.0 + k * k / 4.0)
    ex_l, ex_r = k * (root - k / 2.0), -k * (root + k / 2.0)
    assert abs(om_l - ex_l) < 0.03 * ex_l, (om_l, ex_l)
    assert abs(om_r - ex_r) < 0.03 * abs(ex_r), (om_r, ex_r)
    k_eff2 = (2.0 * np.sin(k / 2.0)) ** 2
    assert abs(om_l * om_r + k_eff2) < 0.005 * k_eff2  # the Alfven part: -k_eff^2
    assert 0.78 < (om_l + om_r) / (-k * k) < 0.84  # the scheme's Hall splitting at dz = d_i (see above)
    assert np.all(np.abs(roots) <= 1.0 + 1e-9)  # no growth


def _roots(a, dt):
    lhs = np.stack([a[1:-1], a[:-2]], axis=1)
    c, *_ = np.linalg.lstsq(lhs, a[2:], rcond=None)
    return sorted(-np.angle(np.roots([1.0, -c[0], -c[1]])) / dt)


def test_hall_splitting_converges_at_first_order_in_dz():
    """One ion per cell at the centre; the same 32 d_i wavelength on 32 and
    64 cells: the shortfall of the splitting from the fluid value halves."""
    short = []
    for nz_cells, delz in ((32, 1.0), (64, 0.5)):
        a, dt, k = _wave(steps=2000, every=10, nz_cells=nz_cells, delz=delz, q=(0.5,))
        om_r, om_l = _roots(a, dt)
        n = 1.0 / delz
        k_eff2 = (2.0 * np.sin(k * delz / 2.0) / delz) ** 2
        assert abs(-om_l * om_r / (k_eff2 / n) - 1.0) < 0.005  # the Alfven part
        short.append(1.0 - (om_l + om_r) / (-k * k / n))
    assert 0.2 < short[0] < 0.3
    assert 0.45 < short[1] / short[0] < 0.55
