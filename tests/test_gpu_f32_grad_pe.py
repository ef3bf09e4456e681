"""The isothermal electron-pressure term in the FP32 form (grad_pe != 0; the
reference keeps it as a commented "- gradP", gutsf.f:1083,1283, and the FP64
path and the oracle carry it as an extension): E at every face subtracts
grad_pe * grad(n_p) / n_face, and the particles' gathered E subtracts the
same gradient centred per node (get_Ep's extension).

Against the FP64 oracle with the same term: one step to the FP32 form's
rounding, 20 steps within its accumulated rounding, and the term changes the
run.  It runs with the exact moment sums only.
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for

pytestmark = pytest.mark.gpu

GP = 0.3


def _pair(steps, grad_pe=GP):
    h = make_hybrid(cells=(16, 8, 8), ppc=16, seed=7, db=0.0, grad_pe=grad_pe)
    o = oracle_for(h)
    h.f32_begin()
    h.f32_run(steps)
    h.f32_end()
    h.sync_to_host()
    for _ in range(steps):
        o.ion_step()
    return h, o


def test_f32_grad_pe_one_step_matches_fp64_oracle():
    h, o = _pair(1)
    assert rel_l2(h.b1, o.b1) < 1e-5
    assert rel_l2(h.b1 - h.b0, o.b1 - o.b0) < 1e-2
    assert rel_l2(h.np, o.np) < 1e-4
    assert rel_l2(h.up, o.up) < 1e-4
    assert rel_l2(h.E, o.E) < 1e-3
    h.close()


def test_f32_grad_pe_20_steps_and_the_term_is_live():
    h, o = _pair(20)
    assert rel_l2(h.b1, o.b1) < 1e-4
    assert rel_l2(h.b1 - h.b0, o.b1 - o.b0) < 3e-2
    assert rel_l2(h.np, o.np) < 1e-3
    assert np.all(np.isfinite(h.b1))
    assert h.max_abs_divB(h.b1) < 1e-5
    h0, _ = _pair(20, grad_pe=0.0)
    # without the term the run differs by far more than the FP32 form's error
    assert rel_l2(h0.b1 - h0.b0, h.b1 - h.b0) > 10 * rel_l2(h.b1 - h.b0, o.b1 - o.b0)
    h.close()
    h0.close()


def test_f32_grad_pe_needs_the_exact_sums():
    h = make_hybrid(cells=(8, 8, 8), ppc=2, seed=3, grad_pe=GP)
    h.f32_begin()
    assert h.lib.swap_f32_set_moment_sums(h.ctx, 0) == 1  # SWAP_EINVAL
    h.f32_run(1)  # still usable with the exact sums
    h.f32_end()
    h.close()
