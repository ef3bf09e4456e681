"""The FP32 form (int32 cell + FP32 offset particles, FP32 moments, B
accumulated in double-float) through the C-ABI, against the FP64 oracle and against the
stable counting sort it must reproduce.

Bars:
  * conversion in and out: cells bit-exact, positions/velocities within one
    FP32 rounding, particle order equal to a stable counting sort by key;
  * incremental sort after displacements: the permutation equals the
    oracle's stable counting sort of the same keys (bit-exact) and per-cell
    counts equal;
  * one ion step: B within rel-L2 1e-5 of the FP64 oracle (its perturbation
    B-b0 within 1e-2), density and flow within rel-L2 1e-4;
  * 20 steps: relative energy drift below 1e-3 and max|div B| below 1e-5.
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for

pytestmark = pytest.mark.gpu


def brick_key(h, xp):
    """Brick-major cell key of each particle (4x4x4 bricks), from FP64 positions."""
    ncx, ncy, ncz = h.cfg.cells
    c = h.coords
    ci = np.ceil((xp[:, 0] - c.qx[0]) / (c.qx[1] - c.qx[0])).astype(np.int64) - 1
    cj = np.floor((xp[:, 1] - c.qy[0]) / (c.qy[1] - c.qy[0])).astype(np.int64)
    ck = np.ceil((xp[:, 2] - c.qz[0]) / (c.qz[1] - c.qz[0])).astype(np.int64) - 1
    nbx, nby = ncx // 4, ncy // 4
    b = (ci >> 2) + nbx * ((cj >> 2) + nby * (ck >> 2))
    return b * 64 + (ci & 3) + 4 * (cj & 3) + 16 * (ck & 3), (ci, cj, ck)


def stable_sort(keys, nkeys):
    import ctypes as C

    import pyoracle

    lib = pyoracle.load()
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    perm = np.zeros(len(keys), dtype=np.int64)
    counts = np.zeros(nkeys, dtype=np.int64)
    r = lib.oracle_stable_counting_sort(keys.ctypes.data_as(C.c_void_p), C.c_int64(len(keys)), C.c_int64(nkeys),
                                        perm.ctypes.data_as(C.c_void_p), counts.ctypes.data_as(C.c_void_p))
    assert r == 0
    return perm, counts


def tagged_hybrid(cells=(16, 8, 12), ppc=6, seed=5, shuffle=True):
    h = make_hybrid(cells=cells, ppc=ppc, seed=seed, db=0.0)
    n = int(h.ni_tot[0])
    if shuffle:  # start from an unsorted order
        p = np.random.default_rng(seed).permutation(n)
        for a in (h.xp, h.vp, h.vp1):
            a[:n] = a[p]
    h.vp[:n, 0] = np.arange(n, dtype=np.float64)  # tag: exact in FP32 below 2**24
    h.mark_host_dirty()
    return h, n


def test_f32_conversion_and_initial_sort():
    h, n = tagged_hybrid()
    xp0 = h.xp[:n].copy()
    vp0 = h.vp[:n].copy()
    keys, _ = brick_key(h, xp0)
    nkeys = int(np.prod(h.cfg.cells))
    perm, counts = stable_sort(keys, nkeys)
    h.f32_begin()
    h.f32_end()
    h.sync_to_host()
    got_perm = h.vp[:n, 0].astype(np.int64)
    assert np.array_equal(got_perm, perm)
    assert np.max(np.abs(h.xp[:n] - xp0[perm])) <= 2e-6 * np.max(np.abs(xp0))
    assert np.max(np.abs(h.vp[:n, 1:] - vp0[perm, 1:])) <= 1e-6 * np.max(np.abs(vp0[:, 1:]))
    k2, _ = brick_key(h, h.xp[:n])
    assert np.array_equal(k2, keys[perm])  # cells survive the round trip exactly
    assert np.array_equal(np.bincount(k2, minlength=nkeys), counts)


@pytest.mark.parametrize("cells", [(12, 8, 8), (16, 12, 12)])  # second: most keys take the order-table path
def test_f32_incremental_sort_is_the_stable_counting_sort(cells):
    h, n = tagged_hybrid(cells=cells, ppc=5, seed=9)
    h.f32_begin()
    h.f32_end()
    h.sync_to_host()
    order0 = h.vp[:n, 0].astype(np.int64).copy()  # tags in the sorted order
    keys0, (ci, cj, ck) = brick_key(h, h.xp[:n])
    rng = np.random.default_rng(1)
    sel = np.sort(rng.choice(n, size=n // 3, replace=False))
    d = rng.integers(-1, 2, size=(len(sel), 3))
    dcell = (d[:, 0] + 1) | ((d[:, 1] + 1) << 10) | ((d[:, 2] + 1) << 20)
    # the FP32 state is still live after f32_end: displace and re-sort it
    h.f32_displace_resort(sel, dcell)
    ncx, ncy, ncz = h.cfg.cells
    ci2, cj2, ck2 = ci.copy(), cj.copy(), ck.copy()
    ci2[sel] = (ci2[sel] + d[:, 0]) % ncx
    cj2[sel] = (cj2[sel] + d[:, 1]) % ncy
    ck2[sel] = (ck2[sel] + d[:, 2]) % ncz
    nbx, nby = ncx // 4, ncy // 4
    keys1 = ((ci2 >> 2) + nbx * ((cj2 >> 2) + nby * (ck2 >> 2))) * 64 + (ci2 & 3) + 4 * (cj2 & 3) + 16 * (ck2 & 3)
    perm, counts = stable_sort(keys1, ncx * ncy * ncz)
    h.f32_end()
    h.sync_to_host()
    got = h.vp[:n, 0].astype(np.int64)
    assert np.array_equal(got, order0[perm])
    k3, _ = brick_key(h, h.xp[:n])
    assert np.array_equal(np.bincount(k3, minlength=counts.size), counts)


def _one_step_pair(cells=(16, 8, 8), ppc=16, seed=7, steps=1):
    h = make_hybrid(cells=cells, ppc=ppc, seed=seed, db=0.0)
    o = oracle_for(h)
    h.f32_begin()
    h.f32_run(steps)
    h.f32_end()
    h.sync_to_host()
    for _ in range(steps):
        o.ion_step()
    return h, o


def test_f32_one_step_matches_fp64_oracle():
    h, o = _one_step_pair()
    assert rel_l2(h.b1, o.b1) < 1e-5
    assert rel_l2(h.b1 - h.b0, o.b1 - o.b0) < 1e-2
    assert rel_l2(h.np, o.np) < 1e-4
    assert rel_l2(h.up, o.up) < 1e-4
    assert rel_l2(h.E, o.E) < 1e-3


def test_f32_energy_and_divB_over_20_steps():
    h = make_hybrid(cells=(16, 8, 8), ppc=16, seed=3, db=0.0)
    h.f32_begin()
    e0 = h.f32_energy()
    h.f32_run(20)
    e1 = h.f32_energy()
    h.f32_end()
    h.sync_to_host()
    drift = abs((e1[0] + e1[1]) - (e0[0] + e0[1])) / (e0[0] + e0[1])
    assert drift < 1e-3, drift
    assert h.max_abs_divB(h.b1) < 1e-5
    assert np.all(np.isfinite(h.b1)) and np.all(np.isfinite(h.xp[: int(h.ni_tot[0])]))
