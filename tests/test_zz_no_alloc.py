"""swap_update_up_noalloc: the moment deposit for callers that cannot call
cudaMalloc (a host whose device memory another allocator owns, or one that
cannot let an allocation synchronize the device in its step).

It must give the same up as the context entries swap_get_interp_weights +
swap_update_up (gutsp.f:1378-1435, 1649-1842), within the deposit tolerance
of the other parity tests, on two calls in a row -- the second call reuses the
shared static scratch that the first call left behind.  Collected last, so a
run that stops at the first failure has run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import relerr
from helpers import make_hybrid

pytestmark = pytest.mark.gpu

DEPOSIT_TOL = 1e-13  # same bar as the atomic deposits in test_gpu_parity.py


def _to_device(a):
    """A Fortran-ordered float64 array as a flat CUDA tensor with the same layout."""
    import torch

    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def _noalloc(h, n, stream=None, expect=0):
    import torch

    xp_d, vp_d, bp_d, np_d = (_to_device(a) for a in (h.xp, h.vp, h.beta_p, h.np))
    up_d = torch.full((h.up.size,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    rc = h.lib.swap_update_up_noalloc(C.byref(h.dims), C.byref(h.params), C.byref(h._coords_c), ptr(xp_d),
                                      ptr(vp_d), ptr(bp_d), n, ptr(np_d), ptr(up_d),
                                      None if stream is None else C.c_void_p(stream.cuda_stream))
    assert rc == expect, rc
    return up_d.cpu().numpy().reshape(h.up.shape, order="F")


def _context_up(h):
    h.get_interp_weights(h.xp)
    h.update_np(h.np)
    h.update_up(h.vp, h.np, h.up)
    h.sync_to_host()
    return h.up.copy(order="F")


def test_noalloc_matches_context_entry_on_two_calls():
    h = make_hybrid(cells=(14, 6, 9), ppc=5, seed=21)
    n = int(h.ni_tot[0])
    rng = np.random.default_rng(4)
    for call in range(2):
        if call == 1:  # other velocities and positions for the second call
            h.vp[:n] += 0.2 * rng.standard_normal((n, 3))
            h.xp[:n, 0] = 1.0 + np.mod(h.xp[:n, 0] - 1.0 + 0.37, h.cfg.cells[0])
            h.mark_host_dirty()
        h.get_interp_weights(h.xp)
        h.update_np(h.np)
        h.update_up(h.vp, h.np, h.up)
        h.sync_to_host()
        want = h.up.copy(order="F")
        got = _noalloc(h, n)
        assert np.all(np.isfinite(got))
        assert relerr(got, want) < DEPOSIT_TOL, (call, relerr(got, want))
    h.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from swap_gb300 import abi

    lib = abi.load()
    big = abi.Dims(4097, 3, 3, 0, 1)  # more nodes on x than SWAP_NOALLOC_MAX_AXIS
    h = make_hybrid(cells=(4, 3, 3), ppc=1, seed=2)
    rc = lib.swap_update_up_noalloc(C.byref(big), C.byref(h.params), C.byref(h._coords_c), None, None, None, 0,
                                    C.c_void_p(1), C.c_void_p(1), None)
    assert rc == 4  # SWAP_ECAPACITY, before any device work
    h.close()


def test_noalloc_larger_grid_then_smaller_grid_on_a_stream():
    # the second call runs on a smaller grid: the geometry and sums it finds
    # in the shared scratch are the first call's, and it must replace them
    import torch

    stream = torch.cuda.Stream()
    for cells, seed in (((16, 10, 12), 5), ((6, 4, 5), 6)):
        h = make_hybrid(cells=cells, ppc=3, seed=seed)
        n = int(h.ni_tot[0])
        want = _context_up(h)
        got = _noalloc(h, n, stream=stream)
        assert relerr(got, want) < DEPOSIT_TOL, (cells, relerr(got, want))
        h.close()


def test_noalloc_reports_a_particle_outside_the_grid():
    h = make_hybrid(cells=(6, 4, 5), ppc=2, seed=8)
    n = int(h.ni_tot[0])
    _context_up(h)
    h.xp[3, 2] = h.coords.qz[-1] + 5.0  # beyond the last node in z
    _noalloc(h, n, expect=3)  # SWAP_EDOMAIN
    h.xp[3, 2] = 0.5 * (h.coords.qz[1] + h.coords.qz[2])
    h.mark_host_dirty()  # the entry works again on the next call
    want = _context_up(h)
    got = _noalloc(h, n)
    assert relerr(got, want) < DEPOSIT_TOL
    h.close()
