"""Compensated FP32 moment sums (the FP32 form's precision: FP32 moments with
compensated per-block partial sums) against plain FP32 sums.

One step of the FP32 form from the same load, with the moment sums
compensated (the default) and plain, each against the FP64 oracle's step:
the compensated density and velocity moments must sit much closer to the
FP64 ones (the rounding of the deposit sums is what the FP32 form adds to
the moments after one step; the positions' own rounding is far smaller).
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for

pytestmark = pytest.mark.gpu

KW = dict(cells=(16, 8, 8), ppc=64, seed=31, db=0.0)


def _f32_step(compensated):
    h = make_hybrid(**KW)
    h.f32_begin()
    h._check(h.lib.swap_f32_set_compensated(h.ctx, 1 if compensated else 0))
    h.f32_run(1)
    h.f32_end()
    h.sync_to_host()
    return h


def test_compensated_moments_are_closer_to_fp64():
    ref = make_hybrid(**KW)
    o = oracle_for(ref)
    o.ion_step()
    on, off = _f32_step(True), _f32_step(False)
    err = {}
    for name in ("np", "up"):
        err[name] = (rel_l2(getattr(on, name), getattr(o, name)), rel_l2(getattr(off, name), getattr(o, name)))
    print("compensated vs plain FP32, rel-L2 against FP64 after one step:", err)
    assert err["np"][0] < err["np"][1] / 3, err
    assert err["up"][0] < err["up"][1] / 1.5, err
    assert err["np"][0] < 1e-7 and err["up"][0] < 1e-5, err
    # B moves by the moments: the compensated run stays at least as close
    assert rel_l2(on.b1, o.b1) <= 1.05 * rel_l2(off.b1, o.b1)
    for h in (on, off, ref):
        h.close()
