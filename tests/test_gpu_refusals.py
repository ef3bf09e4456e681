"""Inputs the library refuses, and the context after each refusal.

Every refusal comes back as a SWAP_E* code with a message, before or in place
of the work it refuses; the context then runs the next call as if the refused
one had not been made (the FP64 step after it still equals the oracle's).
"""
import numpy as np
import pytest

from helpers import make_hybrid, oracle_for
from swap_gb300.abi import SwapError

pytestmark = pytest.mark.gpu

SWAP_EINVAL, SWAP_EDOMAIN, SWAP_ECAPACITY = 1, 3, 4


def _step_matches_oracle(h):
    o = oracle_for(h)
    h.ion_step()
    o.ion_step()
    h.sync_to_host()
    n = int(h.ni_tot[0])
    assert n == int(o.ni_tot[0])
    for name in ("xp", "vp"):
        a, b = getattr(h, name)[:n], getattr(o, name)[:n]
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    for name in ("b1", "np", "up"):
        a, b = getattr(h, name), getattr(o, name)
        assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(b)


def test_a_particle_outside_the_grid_is_refused_and_the_next_step_runs():
    h = make_hybrid(cells=(8, 8, 8), ppc=2, seed=21)
    y = float(h.xp[5, 1])
    h.xp[5, 1] = -3.0 * h.coords.dy  # below the first cell in y (gutsp.f:1398)
    h.mark_host_dirty()
    with pytest.raises(SwapError) as e:
        h.get_interp_weights(h.xp)
    assert e.value.code == SWAP_EDOMAIN and "outside the grid" in str(e.value)
    h.xp[5, 1] = y
    h.mark_host_dirty()
    h.get_interp_weights(h.xp)  # the error word was cleared with the report
    _step_matches_oracle(h)
    h.close()


def test_more_ions_than_the_capacity_are_refused_before_any_work():
    h = make_hybrid(cells=(8, 8, 8), ppc=2, seed=22)
    n = int(h.ni_tot[0])
    b1 = h.b1.copy()
    h.ni_tot[0] = h.ni_max + 1
    with pytest.raises(SwapError) as e:
        h.ion_step()
    assert e.value.code == SWAP_ECAPACITY and "Ni_max" in str(e.value)
    h.ni_tot[0] = n
    h.sync_to_host()
    assert np.array_equal(h.b1, b1)  # nothing ran
    _step_matches_oracle(h)
    h.close()


def test_the_fp32_form_refuses_grids_it_does_not_tile():
    # 10 cells in x: not a whole number of 4-cell bricks
    h = make_hybrid(cells=(10, 8, 8), ppc=2, seed=23)
    with pytest.raises(SwapError) as e:
        h.f32_begin()
    assert e.value.code == SWAP_EINVAL and "multiples of 4" in str(e.value)
    with pytest.raises(SwapError) as e:
        h.f32_run(1)
    assert e.value.code == SWAP_EINVAL and "swap_f32_begin has not been called" in str(e.value)
    _step_matches_oracle(h)  # the FP64 drop-in on the same context
    h.close()

