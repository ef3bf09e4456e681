"""Deterministic FP64 deposits (swap_set_deterministic): the FP64 drop-in's
moment sums in 128-bit fixed point, rounded once per node, instead of FP64
atomics whose result depends on the order of the GPU's adds.

Bars: update_np and update_up against the oracle within the deposit
tolerance of the atomic form; two runs of the fused step give the same bits;
a run resumed from a checkpoint equals the uninterrupted run bit for bit
(maind.f:208-226,588-607 restart, resumed exactly).
"""
import numpy as np
import pytest

from conftest import relerr
from helpers import copy_state, make_hybrid, oracle_for

pytestmark = pytest.mark.gpu

DEPOSIT_TOL = 1e-12
NAMES = ("xp", "vp", "vp1", "b1", "b12", "bt", "np", "up", "E")


def _state(h):
    h.sync_to_host()
    N = int(h.ni_tot[0])
    return {n: getattr(h, n)[:N].copy() if n in ("xp", "vp", "vp1") else getattr(h, n).copy() for n in NAMES}


def test_deterministic_deposits_match_the_oracle():
    h = make_hybrid()
    h.set_deterministic(True)
    o = oracle_for(h)
    for name, args in (("update_np", ("np",)), ("update_up", ("vp", "np", "up"))):
        copy_state(h, o)
        h.get_interp_weights(h.xp)
        o.get_interp_weights(o.xp)
        getattr(o, name)(*[getattr(o, a) for a in args])
        getattr(h, name)(*[getattr(h, a) for a in args])
        h.sync_to_host()
        out = args[-1]
        assert relerr(getattr(h, out), getattr(o, out)) < DEPOSIT_TOL, name
    h.close()


def test_deterministic_fp64_runs_repeat_bit_for_bit():
    runs = []
    for _ in range(2):
        h = make_hybrid(cells=(16, 8, 8), ppc=8, seed=21, extra=0)
        h.set_deterministic(True)
        h.run(3)
        runs.append(_state(h))
        h.close()
    for k in NAMES:
        assert np.array_equal(runs[0][k], runs[1][k]), k


def test_deterministic_fp64_resume_is_bit_exact(tmp_path):
    h = make_hybrid(extra=0)
    h.set_deterministic(True)
    h.run(2)
    path = str(tmp_path / "ck.bin")
    h.checkpoint_write(path)
    h.run(3)
    a = _state(h)
    g = make_hybrid(extra=0, seed=99)  # a different load, overwritten by the restart
    g.set_deterministic(True)
    g.checkpoint_read(path)
    g.run(3)
    b = _state(g)
    for k in NAMES:
        assert np.array_equal(a[k], b[k]), k
    h.close()
    g.close()
