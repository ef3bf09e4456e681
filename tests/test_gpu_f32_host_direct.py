"""Host-direct conversions of the FP32 form against the staged ones.

In host-direct mode swap_f32_begin reads the FP64 particle arrays in the
caller's (here pageable) memory and swap_f32_end writes xp, vp, vp1, mrat and
beta_p straight back; staged mode copies them through the device mirrors.  The
arithmetic is the same, so a round trip (begin, end) must come back bit for
bit; steps in between agree to the rounding of the deposits' shared-memory
sums.  The transfer counters must count exactly the bytes each mode moves,
and an FP64 entry after swap_f32_end must pick the written-back arrays up.
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid
from swap_gb300 import abi

pytestmark = pytest.mark.gpu

PARTS = ("xp", "vp", "vp1", "mrat", "beta_p")
OUT_FIELDS = ("b1", "b12", "b1p2", "bt", "np", "up", "aj", "E")


def _run(direct, sources, steps=3):
    h = make_hybrid(cells=(16, 8, 8), ppc=8, seed=11, db=0.02, extra=20000)
    if direct:
        try:
            h.set_host_direct(True)
        except RuntimeError:
            pytest.skip("this device does not address host memory directly")
    else:
        h.set_host_direct(False)
    if sources:
        cfg = h.cfg
        h.set_sources(abi.make_sources(seed=5, x_open=1, inflow_ppc=8, inflow_vth=cfg.vth,
                                       inflow_ux=cfg.u[0]), 0)
    n0 = int(h.ni_tot[0])
    h.transfer_bytes(reset=True)
    h.f32_begin()
    up = h.transfer_bytes(reset=True)
    h.f32_run(steps)
    h.f32_end()
    h.sync_to_host()
    down = h.transfer_bytes(reset=True)
    return h, n0, up, down


def _expected_bytes(h, n_in, n_out):
    grid = h.b1.nbytes // 3
    # f32_begin reads xp, vp, vp1, mrat, beta_p and b0, b1, b12, np, nu;
    # f32_end writes the particles and the fields of OUT_FIELDS
    up = n_in * (3 * 24 + 2 * 8) + 3 * 3 * grid + 2 * grid
    down = n_out * (3 * 24 + 2 * 8) + sum(getattr(h, a).nbytes for a in OUT_FIELDS)
    return up, down


@pytest.mark.parametrize("sources", [False, True], ids=["periodic", "open_x"])
def test_host_direct_round_trip_matches_staged_bit_for_bit(sources):
    # begin and end with no step between: conversions only, no deposit order
    hs, n0, up_s, down_s = _run(False, sources, steps=0)
    hd, n0d, up_d, down_d = _run(True, sources, steps=0)
    assert n0 == n0d
    N = int(hs.ni_tot[0])
    assert int(hd.ni_tot[0]) == N == n0
    for a in PARTS:
        np.testing.assert_array_equal(getattr(hd, a)[:N], getattr(hs, a)[:N], err_msg=a)
    for a in OUT_FIELDS:
        np.testing.assert_array_equal(getattr(hd, a), getattr(hs, a), err_msg=a)
    # the same bytes cross the link either way: the particle vectors by copy
    # or by the conversion kernels' own loads and stores
    exp = _expected_bytes(hs, n0, N)
    assert (up_s[0], down_s[1]) == exp
    assert (up_d[0], down_d[1]) == exp


def test_host_direct_steps_track_staged():
    # the deposits add in shared memory in warp order, so three steps agree
    # to float rounding, not bit for bit
    hs, n0, up_s, down_s = _run(False, True, steps=3)
    hd, _, up_d, down_d = _run(True, True, steps=3)
    N, Nd = int(hs.ni_tot[0]), int(hd.ni_tot[0])
    assert abs(N - Nd) <= 2
    assert (up_d[0], down_d[1]) == _expected_bytes(hd, n0, Nd)
    assert (up_s[0], down_s[1]) == _expected_bytes(hs, n0, N)
    assert rel_l2(hd.b1, hs.b1) < 1e-6
    assert rel_l2(hd.np, hs.np) < 1e-4


def test_fp64_entry_after_host_direct_end_reads_the_written_arrays():
    hs, _, _, _ = _run(False, False, steps=2)
    hd, _, _, _ = _run(True, False, steps=2)
    # one FP64 step from the written-back state: the direct context uploads
    # the host copies the FP32 form wrote (stale mirrors would hold the state
    # from before the FP32 steps), the staged one reuses its mirrors
    hs.run(1)
    hd.run(1)
    hs.sync_to_host()
    hd.sync_to_host()
    N = int(hs.ni_tot[0])
    assert int(hd.ni_tot[0]) == N
    for a in ("xp", "vp", "vp1"):
        assert rel_l2(getattr(hd, a)[:N], getattr(hs, a)[:N]) < 1e-6, a
    assert rel_l2(hd.b1, hs.b1) < 1e-6
