"""The C-ABI at the reference's own precision: SWAP as its makefile builds it
(makefile:1, -real-size 32) binds float32 arrays (swap_dims.real_bytes = 4).

The device computes in FP64 and rounds its outputs back to float, so the
result must equal the FP64 oracle run on the widened float inputs, rounded to
float (a few ulp for the atomic deposits' order), and must agree with the
FP32 oracle (oracle32_, the reference's own arithmetic) to FP32 rounding.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import rel_l2
from helpers import periodic_np
from swap_gb300.hybrid import Hybrid, config

pytestmark = pytest.mark.gpu

FIELDS = ("b0", "b1", "b12", "b1p2", "bt", "btc", "np", "up", "aj", "E", "nu")


def _hybrid4(cells=(12, 6, 8), ppc=4, seed=13, db=0.05, **over):
    cfg = config(0, cells=cells, ppc=ppc, seed=seed, **over)
    h = Hybrid(cfg, ni_max=cfg.n_particles + 5, real_bytes=4)
    h.load_maxwellian()
    rng = np.random.default_rng(seed + 7)
    b = (h.b0.astype(np.float64) + db * rng.standard_normal(h.b1.shape)).astype(np.float32)
    periodic_np(b)
    for n in ("b1", "b12", "b1p2", "bt"):
        getattr(h, n)[...] = b
    h.mark_host_dirty()
    return h


def _ulps(a, b):
    """max |a - b| in units of float32 spacing at |b| (b the reference)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    sp = np.spacing(np.abs(b).astype(np.float32)).astype(np.float64)
    scale = np.maximum(sp, np.spacing(np.float32(np.max(np.abs(b)) * 1e-6)))
    return float(np.max(np.abs(a - b) / scale)) if a.size else 0.0


def test_real4_arrays_are_float32_and_round_trip(oracle_mod):
    # move_ion_half in FP64 on the widened positions, rounded back to float:
    # exactly the FP64 oracle's move of the same floats, rounded
    h = _hybrid4()
    assert h.xp.dtype == np.float32 and h.b1.dtype == np.float32 and h.real_bytes == 4
    o64 = oracle_mod.from_hybrid_arrays(h, precision="f64")
    n = int(h.ni_tot[0])
    h.move_ion_half(h.xp, h.vp, h.vp1, h.input_p)
    h.sync_to_host()
    o64.move_ion_half(o64.xp, o64.vp, o64.vp1, o64.input_p)
    assert np.array_equal(h.xp[:n], o64.xp[:n].astype(np.float32))
    h0, d0 = h.transfer_bytes()
    assert h0 > 0 and d0 > 0
    h.close()


def test_real4_fused_step_against_the_oracles(oracle_mod):
    h = _hybrid4()
    o64 = oracle_mod.from_hybrid_arrays(h, precision="f64")  # the float inputs, widened
    o32 = oracle_mod.from_hybrid_arrays(h, precision="f32")  # the reference's own arithmetic
    h.ion_step()
    h.sync_to_host()
    o64.ion_step()
    o32.ion_step()
    n = int(h.ni_tot[0])
    assert n == int(o64.ni_tot[0]) == int(o32.ni_tot[0])
    for name in ("xp", "vp", "vp1"):
        got = getattr(h, name)[:n]
        assert got.dtype == np.float32
        # FP64 arithmetic then one rounding: the FP64 oracle rounded to float
        assert _ulps(got, getattr(o64, name)[:n].astype(np.float32)) <= 2.0, name
        assert rel_l2(got, getattr(o32, name)[:n]) < 1e-5, name
    for name in ("b1", "np", "up", "E"):
        got = getattr(h, name)
        assert _ulps(got, getattr(o64, name).astype(np.float32)) <= 4.0, name
        assert rel_l2(got, getattr(o32, name)) < 2e-4, name
    h.close()


def test_real4_subroutine_entries_against_oracle32(oracle_mod):
    h = _hybrid4(seed=29)
    o32 = oracle_mod.from_hybrid_arrays(h, precision="f32")
    h.get_interp_weights(h.xp)
    h.update_np(h.np)
    h.update_up(h.vp, h.np, h.up)
    h.curlB(h.bt, h.np, h.aj)
    h.get_E(h.E, h.b0, h.bt, h.aj, h.up, h.np, h.nu)
    h.sync_to_host()
    o32.get_interp_weights(o32.xp)
    o32.update_np(o32.np)
    o32.update_up(o32.vp, o32.np, o32.up)
    o32.curlB(o32.bt, o32.np, o32.aj)
    o32.get_E(o32.E, o32.b0, o32.bt, o32.aj, o32.up, o32.np, o32.nu)
    for name, tol in (("np", 1e-5), ("up", 1e-5), ("aj", 1e-4), ("E", 1e-4)):
        assert rel_l2(getattr(h, name), getattr(o32, name)) < tol, name
    h.close()


def test_real4_fp32_form_and_checkpoint(oracle_mod):
    # the FP32 form stages through the device mirrors with 4-byte reals; a
    # checkpoint of a 4-byte context restores the float arrays exactly
    h = _hybrid4(cells=(16, 8, 8), ppc=8, seed=3, db=0.0)
    o64 = oracle_mod.from_hybrid_arrays(h, precision="f64")
    h.f32_begin()
    h.f32_run(1)
    h.f32_end()
    h.sync_to_host()
    o64.ion_step()
    for name, tol in (("b1", 1e-5), ("np", 1e-4), ("up", 1e-4)):
        assert rel_l2(getattr(h, name), getattr(o64, name)) < tol, name
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ck.bin")
        h.checkpoint_write(path)
        saved = {k: getattr(h, k).copy() for k in ("xp", "vp", "b1", "np")}
        n = int(h.ni_tot[0])
        for k in saved:
            getattr(h, k)[...] = 0
        h.checkpoint_read(path)
        h.sync_to_host()
        assert int(h.ni_tot[0]) == n
        for k, v in saved.items():
            a = getattr(h, k)
            assert np.array_equal(a[:n] if k in ("xp", "vp") else a, v[:n] if k in ("xp", "vp") else v), k
    h.close()
