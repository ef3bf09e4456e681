"""The FP32 form's moment sums: FP32 per warp, then exact 64-bit fixed-point
accumulation per brick and over the bricks, one rounding per node.

- Against plain FP32 atomics, one step from the same load is closer to the
  FP64 oracle's step (the sums' rounding is what the FP32 form adds to the
  moments after one step; the positions' own rounding is far smaller).
- The sums do not depend on the order of the GPU's adds, so the FP32 form is
  reproducible: two runs from one state agree bit for bit, and a run resumed
  from a checkpoint equals the uninterrupted run bit for bit (maind.f:588-607
  writes the reference's restart files).
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for
from swap_gb300 import abi

pytestmark = pytest.mark.gpu

KW = dict(cells=(16, 8, 8), ppc=64, seed=31, db=0.0)
STATE = ("xp", "vp", "vp1", "b1", "b12", "np", "up", "E")


def _f32(exact, steps=1, kw=KW, sources=None):
    h = make_hybrid(**kw)
    if sources is not None:
        h.set_sources(sources, 0)
    h.f32_begin()
    h._check(h.lib.swap_f32_set_moment_sums(h.ctx, 1 if exact else 0))
    h.f32_run(steps)
    h.f32_end()
    h.sync_to_host()
    return h


def test_exact_sums_are_closer_to_fp64_than_plain_atomics():
    ref = make_hybrid(**KW)
    o = oracle_for(ref)
    o.ion_step()
    ex, pl = _f32(True), _f32(False)
    err = {n: (rel_l2(getattr(ex, n), getattr(o, n)), rel_l2(getattr(pl, n), getattr(o, n))) for n in ("np", "up")}
    print("exact vs plain FP32 sums, rel-L2 against FP64 after one step:", err)
    assert err["np"][0] < err["np"][1] / 1.5 and err["np"][0] < 6e-8, err
    assert err["up"][0] < err["up"][1], err
    for h in (ex, pl, ref):
        h.close()


def test_fp32_form_is_reproducible_bit_for_bit():
    src = abi.make_sources(seed=8, x_open=1, inflow_ppc=16, inflow_vth=0.5, inflow_ux=2.0)
    kw = dict(cells=(16, 8, 8), ppc=16, seed=4, db=0.02, extra=40000)
    a, b = _f32(True, 6, kw, src), _f32(True, 6, kw, src)
    n = int(a.ni_tot[0])
    assert n == int(b.ni_tot[0])
    for name in STATE:
        x, y = getattr(a, name), getattr(b, name)
        if x.shape[0] == a.ni_max:
            x, y = x[:n], y[:n]
        assert np.array_equal(x, y), name
    a.close()
    b.close()


def test_resume_from_a_checkpoint_is_bit_exact():
    kw = dict(cells=(16, 8, 8), ppc=16, seed=6, db=0.02, extra=40000)
    src = abi.make_sources(seed=9, x_open=1, inflow_ppc=16, inflow_vth=0.5, inflow_ux=2.0)
    whole = _f32(True, 6, kw, src)
    h = make_hybrid(**kw)
    h.set_sources(src, 0)
    h.f32_begin()
    h.f32_run(3)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ck.bin")
        h.checkpoint_write(path)  # the running FP32 state goes into the file
        h.close()
        r = make_hybrid(**kw)
        r.checkpoint_read(path)  # restores the sources, the step counter and the FP32 state
    r.f32_run(3)
    r.f32_end()
    r.sync_to_host()
    n = int(whole.ni_tot[0])
    assert n == int(r.ni_tot[0])
    for name in STATE:
        x, y = getattr(whole, name), getattr(r, name)
        if x.shape[0] == whole.ni_max:
            x, y = x[:n], y[:n]
        assert np.array_equal(x, y), name
    whole.close()
    r.close()
