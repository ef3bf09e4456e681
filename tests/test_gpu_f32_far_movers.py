"""Ions that move more than one cell per axis in one step (|v| dt > dx) in the
FP32 form.  The reference moves an ion any distance below the grid's extent
(move_ion_half, gutsp.f:454-570) and finds its cell again (get_interp_weights,
gutsp.f:1378-1435); the FP32 form's sort only follows moves to a neighbour
cell, so pass 3 lists the farther movers, their moments go into the brick
partials from that list, and the sort places them after the near arrivals of
their new cell in array order.

On a box where one ion in 37 moves 2.6 or 5.5 cells per step along each axis
(half moves of 1.3 and 2.75 cells, so some deposit outside their brick's
tile window too), three steps agree with the FP64 oracle on the same start to
the FP32 form's rounding, and two runs give the same bits.
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for

pytestmark = pytest.mark.gpu


def _fast_box(seed=21, every=37, speeds=(2.6, 5.5)):
    h = make_hybrid(cells=(16, 8, 8), ppc=8, seed=seed, db=0.0, extra=64)
    n = int(h.ni_tot[0])
    rng = np.random.default_rng(seed)
    idx = np.arange(0, n, every)
    cells_per_step = rng.choice(speeds, size=(idx.size, 3)) * rng.choice([-1.0, 1.0], size=(idx.size, 3))
    v = cells_per_step * np.array([h.coords.dx, h.coords.dy, h.coords.delz]) / h.cfg.dt
    h.vp[idx] = v
    h.vp1[idx] = v
    h.mark_host_dirty()
    return h, idx.size


def _run_f32(h, steps):
    h.f32_begin()
    h.f32_run(steps)
    far = h.f32_far_movers()
    h.f32_end()
    h.sync_to_host()
    return far


def test_far_movers_match_the_fp64_oracle():
    h, nfast = _fast_box()
    o = oracle_for(h)
    steps = 3
    far = _run_f32(h, steps)
    for _ in range(steps):
        o.ion_step()
    # every fast ion takes the far path at every step
    assert far == steps * nfast, (far, nfast)
    n = int(h.ni_tot[0])
    assert n == int(o.ni_tot[0])
    assert rel_l2(h.b1, o.b1) < 1e-5
    assert rel_l2(h.b1 - h.b0, o.b1 - o.b0) < 1e-2
    assert rel_l2(h.np, o.np) < 1e-4
    assert rel_l2(h.up, o.up) < 1e-4
    # the same ions: each coordinate and the speeds as multisets (the FP32
    # form writes them back in its sorted order)
    for ax in range(3):
        assert np.max(np.abs(np.sort(h.xp[:n, ax]) - np.sort(o.xp[:n, ax]))) < 1e-4, ax
    sh = np.sort(np.linalg.norm(h.vp[:n], axis=1))
    so = np.sort(np.linalg.norm(o.vp[:n], axis=1))
    assert np.max(np.abs(sh - so)) < 1e-3 * np.max(so)
    h.close()


def test_far_movers_are_deterministic():
    runs = []
    for _ in range(2):
        h, _ = _fast_box(seed=5)
        _run_f32(h, 4)
        runs.append({k: getattr(h, k).copy() for k in ("b1", "np", "up", "xp", "vp")})
        h.close()
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


def test_a_move_across_the_grid_is_refused():
    from swap_gb300 import abi

    h, _ = _fast_box(speeds=(2.6,))
    h.vp[0] = (0.0, 14.0 * h.coords.dy / h.cfg.dt, 0.0)  # a half move of 7 cells on an 8-cell axis
    h.vp1[0] = h.vp[0]
    h.mark_host_dirty()
    h.f32_begin()
    with pytest.raises(abi.SwapError) as ei:
        h.f32_run(1)
    assert ei.value.code == 7  # SWAP_EMOVE
    h.close()
