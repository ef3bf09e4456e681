"""Failure detection without a GPU fault: each failure is made on the host
or by a device wait that runs out, and comes back as a status code with the
context still usable.

- A device wait of the FP32 passes set to give up at once returns SWAP_EWAIT;
  with the limit restored, a new swap_f32_begin runs the step normally.
- A NaN written into a bound host array is caught by swap_check_finite.
- A truncated or altered checkpoint is refused by its checksum.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid
from swap_gb300 import abi

pytestmark = pytest.mark.gpu

KW = dict(cells=(16, 8, 8), ppc=8, seed=23, db=0.0)


def _f32_steps(h, n):
    h.f32_begin()
    h.f32_run(n)
    h.f32_end()
    h.sync_to_host()


def test_stage_wait_that_runs_out_returns_ewait_and_the_context_recovers():
    ref = make_hybrid(**KW)
    _f32_steps(ref, 2)
    h = make_hybrid(**KW)
    h.f32_begin()
    h._check(h.lib.swap_set_wait_limit(h.ctx, 0))  # every chunk wait gives up at once
    with pytest.raises(abi.SwapError) as ei:
        h.f32_run(1)
    assert ei.value.code == 8  # SWAP_EWAIT
    h._check(h.lib.swap_set_wait_limit(h.ctx, 1 << 22))
    _f32_steps(h, 2)  # begins again from the bound arrays
    assert int(h.ni_tot[0]) == int(ref.ni_tot[0])
    assert rel_l2(h.b1, ref.b1) < 1e-6 and rel_l2(h.np, ref.np) < 1e-5
    h.close()
    ref.close()


def test_nan_injected_on_the_host_is_caught():
    h = make_hybrid(**KW)
    h.check_finite()
    h.vp[5, 1] = np.nan
    h.mark_host_dirty(h.vp)
    with pytest.raises(abi.SwapError) as ei:
        h.check_finite()
    assert ei.value.code == 5  # SWAP_ENONFINITE
    h.b1[3, 2, 1, 0] = np.inf
    h.vp[5, 1] = 0.1
    h.mark_host_dirty()
    with pytest.raises(abi.SwapError):
        h.check_finite()
    h.b1[3, 2, 1, 0] = h.b0[3, 2, 1, 0]
    h.mark_host_dirty()
    h.check_finite()
    h.close()


@pytest.mark.parametrize("damage", ["truncate", "flip", "trailer"])
def test_damaged_checkpoint_is_refused(damage):
    h = make_hybrid(**KW)
    h.run(1)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ck.bin")
        h.checkpoint_write(path)
        h.checkpoint_read(path)  # the intact file reads back
        size = os.path.getsize(path)
        with open(path, "r+b") as f:
            if damage == "truncate":
                f.truncate(size - 4096)
            elif damage == "flip":
                f.seek(size // 2)
                b = f.read(1)
                f.seek(size // 2)
                f.write(bytes([b[0] ^ 0x10]))
            else:
                f.seek(size - 3)
                f.write(b"\x00\x00\x00")
        xp = h.xp.copy()
        with pytest.raises(abi.SwapError) as ei:
            h.checkpoint_read(path)
        assert ei.value.code == 1 and "checksum" in str(ei.value)
        assert np.array_equal(h.xp, xp)  # nothing was read into the arrays
    h.run(1)  # the context stays usable
    h.close()
