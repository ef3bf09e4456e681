"""Particle sources and sinks in the CPU oracle.

The generator is pinned to the published Philox4x32-10 known-answer vectors
(Salmon et al., SC'11; Random123's kat_vectors), then each rule is checked
against its defining property: Ionize_sw_mp's count and ring
(chem_rates.f:551-620), remove_ion's order-preserving shift (gutsp.f:29-41),
the open-x move and outflow, the x inflow, cloud ionization counts, and
res_chex at probability 0 and 1 (chem_rates.f:823-840).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import Host, oracle, small
from swap_gb300 import abi

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

RNG_IONIZE, RNG_INFLOW, RNG_CLOUD, RNG_CHEX = 1, 2, 3, 4


def _lib():
    import pyoracle

    return pyoracle.load()


def uniforms(seed, stream, step, a, b):
    u = (C.c_double * 4)()
    f = _lib().oracle_source_uniforms
    f.argtypes = [C.c_uint64, C.c_uint32, C.c_int64, C.c_int64, C.c_uint32, C.POINTER(C.c_double)]
    f.restype = None
    f(seed, stream, step, a, b, u)
    return np.array(list(u))


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    f = _lib().oracle_philox4x32_10
    f.restype = None
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    out = (C.c_uint32 * 4)()
    f(c, k, out)
    assert tuple(out) == want


def test_source_uniforms_open_interval_and_counters():
    u = np.array([uniforms(5, s, m, a, b) for s in (1, 2) for m in (0, 1) for a in (-1, 0, 7) for b in (0, 1)])
    assert np.all((u > 0) & (u < 1))
    assert len(np.unique(u)) == u.size  # every counter gives new words


def _setup(extra=400, **cfg):
    h = Host(small(**cfg), ni_max=small(**cfg).n_particles + extra)
    o = oracle(h)
    return h, o


def _inside(o, N):
    q = [o.coords()[a] for a in ("qx", "qy", "qz")]
    x = o.xp[:N]
    return all(np.all((x[:, m] > q[m][0]) & (x[:, m] <= q[m][-2])) for m in range(3))


def test_ionize_sw_count_ring_and_placement():
    h, o = _setup()
    N0 = int(o.ni_tot[0])
    cfg = h.cfg
    nz = cfg.nodes[2]
    ndot = 37.4 / (cfg.dt * cfg.beta * nz)  # dNi = ndot*dt*beta*beta_pu*dx*dy*delz*nz = 37.4
    o.set_sources(abi.make_sources(seed=11, ndot=ndot, vsw=3.0, beta_pu=1.0, mrat_pu=0.5, delz_ref=1.0))
    o.Ionize_sw_mp(o.np, o.vp, o.vp1, o.xp, 4, o.input_p, o.up)
    n = int(o.ni_tot[0]) - N0
    assert n == 37  # nint (chem_rates.f:562)
    v = o.vp[N0:N0 + n]
    assert np.allclose(np.hypot(v[:, 0] - 3.0, v[:, 1]), 3.0, rtol=1e-12, atol=0)
    assert np.all(v[:, 2] == 0) and np.array_equal(o.vp1[N0:N0 + n], v)
    assert np.all(o.mrat[N0:N0 + n] == 0.5) and np.all(o.beta_p[N0:N0 + n] == 1.0)
    assert _inside(o, N0 + n)
    # the deposit that follows counts every ion: total weight = N/beta per unit volume
    assert abs(o.np[1:-1, 1:-1, 1:-1].sum() - (N0 + n) / cfg.beta) < 1e-9 * (N0 + n)


@pytest.mark.parametrize("step", [0, 1, 2, 3])
@pytest.mark.parametrize("dni", [0.3, 0.7])
def test_ionize_sw_bernoulli_below_one(step, dni):
    h, o = _setup()
    N0 = int(o.ni_tot[0])
    cfg = h.cfg
    ndot = dni / (cfg.dt * cfg.beta * cfg.nodes[2])
    o.set_sources(abi.make_sources(seed=3, ndot=ndot, vsw=1.0, beta_pu=1.0, mrat_pu=1.0, delz_ref=1.0))
    o.Ionize_sw_mp(o.np, o.vp, o.vp1, o.xp, step, o.input_p, o.up)
    u = uniforms(3, RNG_IONIZE, step, -1, 0)[0]
    # chem_rates.f:555-562: a trial when dNi < 1, then nint -- so dNi >= 0.5 always gives one ion
    want = 1 if (dni > u or dni >= 0.5) else 0
    assert int(o.ni_tot[0]) - N0 == want


def test_remove_ion_shifts_in_order():
    h, o = _setup(extra=0)
    N = int(o.ni_tot[0])
    before = {n: getattr(o, n).copy() for n in ("xp", "vp", "vp1", "mrat", "beta_p")}
    o.mrat[:N] = np.arange(N)  # make the scalar shift visible
    before["mrat"] = o.mrat.copy()
    o.remove_ion(o.xp, o.vp, o.vp1, 5)
    assert int(o.ni_tot[0]) == N - 1
    for n, b in before.items():
        a = getattr(o, n)
        assert np.array_equal(a[:4], b[:4]) and np.array_equal(a[4:N - 1], b[5:N]), n
    with pytest.raises(RuntimeError):
        o.remove_ion(o.xp, o.vp, o.vp1, 0)
    with pytest.raises(RuntimeError):
        o.remove_ion(o.xp, o.vp, o.vp1, N)


def test_open_x_move_and_outflow():
    h, o = _setup(u=(30.0, 0.0, 0.0), vth=0.5)
    N = int(o.ni_tot[0])
    q = o.coords()["qx"]
    dth = h.cfg.dt / 2.0
    xn = o.xp[:N, 0] + dth * o.vp[:N, 0]
    keep = (xn > q[0]) & (xn <= q[-2])
    assert 0 < keep.sum() < N
    expect = {n: getattr(o, n)[:N][keep].copy() for n in ("vp", "vp1", "mrat", "beta_p")}
    o.set_sources(abi.make_sources(x_open=1))
    o.move_ion_half(o.xp, o.vp, o.vp1, o.input_p)
    assert np.array_equal(o.xp[:N, 0], xn)  # no x wrap
    o.remove_outflow_x()
    n = int(o.ni_tot[0])
    assert n == keep.sum()
    assert np.array_equal(o.xp[:n, 0], xn[keep])
    for k, v in expect.items():
        assert np.array_equal(getattr(o, k)[:n], v), k


def test_inflow_enters_through_the_x_face():
    h, o = _setup(extra=2000)
    N0 = int(o.ni_tot[0])
    cfg = h.cfg
    ppc, ux, vth = 8, 4.0, 0.5
    o.set_sources(abi.make_sources(seed=3, x_open=1, inflow_ppc=ppc, inflow_vth=vth, inflow_ux=ux))
    o.inflow_x(2)
    n = int(o.ni_tot[0]) - N0
    q = o.coords()
    x, v = o.xp[N0:N0 + n].copy(), o.vp[N0:N0 + n].copy()
    # entered this step from the one-cell slab before q(1)
    back = x[:, 0] - cfg.dt * v[:, 0]
    assert np.all(x[:, 0] > q["qx"][0]) and np.all(back > q["qx"][0] - q["dx_grid"][0] - 1e-12)
    assert np.all(back <= q["qx"][0] + 1e-12)
    assert _inside(o, N0 + n)
    assert np.array_equal(o.vp1[N0:N0 + n], v)
    # flux: the mean crossing probability is E[dt*vx/dx] for 0 < dt*vx < dx
    ncy, ncz = cfg.cells[1], cfg.cells[2]
    mean = ppc * ncy * ncz * cfg.dt * ux
    assert abs(n - mean) < 5 * np.sqrt(mean)
    # same step again gives the same ions; another step gives others
    o.ni_tot[0] = N0
    o.inflow_x(2)
    assert int(o.ni_tot[0]) - N0 == n and np.array_equal(o.xp[N0:N0 + n], x)
    o.ni_tot[0] = N0
    o.inflow_x(3)
    assert not np.array_equal(o.xp[N0:N0 + 5], x[:5])


def test_cloud_ionization_counts_are_exact():
    h, o = _setup(extra=4000)
    N0 = int(o.ni_tot[0])
    cfg = h.cfg
    q = o.coords()
    src = dict(seed=9, cloud_N0=2.0, cloud_r0=2.0, cloud_x=float(q["qx"][4]), cloud_y=float(q["qy"][3]),
               cloud_z=float(q["qz"][3]), nu_ion=0.7, mrat_heavy=1.0 / 16, beta_heavy=1.0)
    o.set_sources(abi.make_sources(**src))
    o.ionize_cloud(5)
    n = int(o.ni_tot[0]) - N0
    # per cell: floor(lam) + [u < frac], in the restatement's operation order
    ncx, ncy, ncz = cfg.cells
    want = 0
    for ck in range(ncz):
        for cj in range(ncy):
            for ci in range(ncx):
                xc = 0.5 * (q["qx"][ci] + q["qx"][ci + 1])
                yc = 0.5 * (q["qy"][cj] + q["qy"][cj + 1])
                zc = 0.5 * (q["qz"][ck] + q["qz"][ck + 1])
                vol = q["dx_grid"][ci] * q["dy_grid"][cj] * q["dz_grid"][ck]
                dx, dy, dz = xc - src["cloud_x"], yc - src["cloud_y"], zc - src["cloud_z"]
                r2 = (dx * dx + dy * dy + dz * dz) / (src["cloud_r0"] * src["cloud_r0"])
                lam = vol * cfg.beta * src["beta_heavy"] * (src["cloud_N0"] / (1.0 + r2)) * src["nu_ion"] * cfg.dt
                k = int(np.floor(lam))
                cell = (ck * ncy + cj) * ncx + ci
                want += k + (1 if uniforms(9, RNG_CLOUD, 5, cell, 0)[0] < lam - k else 0)
    assert n == want and n > 0
    assert np.all(o.vp[N0:N0 + n] == 0) and np.all(o.vp1[N0:N0 + n] == 0)
    assert np.all(o.mrat[N0:N0 + n] == 1.0 / 16)
    assert _inside(o, N0 + n)


def test_res_chex_probability_zero_and_one():
    h, o = _setup(extra=0)
    N = int(o.ni_tot[0])
    o.mrat[:10] = 1.0 / 16  # already heavy: never exchanged
    vp10 = o.vp[:10].copy()
    o.set_sources(abi.make_sources(seed=1, cloud_N0=1.0, cloud_r0=1e6, cx_a=1e-30, mrat_heavy=1.0 / 16))
    assert o.res_chex(o.xp, o.vp, 0) == 0
    o.set_sources(abi.make_sources(seed=1, cloud_N0=1.0, cloud_r0=1e6, cx_a=1e6, mrat_heavy=1.0 / 16))
    assert o.res_chex(o.xp, o.vp, 0) == N - 10
    assert np.all(o.vp[10:N] == 0) and np.all(o.vp1[10:N] == 0) and np.all(o.mrat[:N] == 1.0 / 16)
    assert np.array_equal(o.vp[:10], vp10)


def test_fused_step_with_every_source():
    h, o = _setup(extra=6000, u=(2.0, 0.0, 0.0))
    cfg = h.cfg
    q = o.coords()
    o.set_sources(abi.make_sources(
        seed=21, ndot=10.0 / (cfg.dt * cfg.beta * cfg.nodes[2]), vsw=2.0, beta_pu=1.0, mrat_pu=0.5, delz_ref=1.0,
        x_open=1, inflow_ppc=4, inflow_vth=0.5, inflow_ux=2.0,
        cloud_N0=0.5, cloud_r0=2.0, cloud_x=float(q["qx"][4]), cloud_y=float(q["qy"][3]), cloud_z=float(q["qz"][3]),
        nu_ion=0.2, mrat_heavy=1.0 / 16, beta_heavy=1.0, cx_a=2.0, cx_b=0.1))
    counts = [int(o.ni_tot[0])]
    for _ in range(3):
        o.ion_step()
        counts.append(int(o.ni_tot[0]))
        assert _inside(o, counts[-1])
    assert len(set(counts)) > 1
    assert o.chex_count() > 0
