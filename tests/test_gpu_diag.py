"""Diagnostic moments, the Fortran-unformatted output files and checkpoints.

Bars: update_rho and get_temperature within the atomic-deposit tolerance of
the oracle; every output record in the reference's layout (maind.f:240-254,
502-571) holding the state it names; a checkpoint restores the bound state
and the FP32 form's state bit for bit, and a resumed run continues as the
uninterrupted one (within the run-to-run spread of atomic deposits).
"""
import ctypes
import struct

import numpy as np
import pytest

from conftest import rel_l2, relerr
from helpers import fortran_records, make_hybrid, oracle_for

pytestmark = pytest.mark.gpu

DEPOSIT_TOL = 1e-12


def test_update_rho_and_get_temperature_match_oracle():
    h = make_hybrid()
    o = oracle_for(h)
    N = int(h.ni_tot[0])
    h.mrat[: N // 3] = 0.5  # two species, so mrat matters
    o.mrat[: N // 3] = 0.5
    h.mark_host_dirty()
    for x in (h, o):
        x.get_interp_weights(x.xp)
        x.update_np(x.np)
    mh, mo = np.zeros_like(h.np), np.zeros_like(o.np)
    th, to = np.zeros_like(h.np), np.zeros_like(o.np)
    for a in (mh, th):
        h.lib.swap_bind_array(h.ctx, a.ctypes.data_as(ctypes.c_void_p), a.nbytes)
    h.update_rho(mh)
    h.get_temperature(h.xp, h.vp, h.np, th)
    o.update_rho(mo)
    o.get_temperature(o.xp, o.vp, o.np, to)
    h.sync_to_host()
    assert relerr(mh, mo) < DEPOSIT_TOL
    assert relerr(th, to) < 1e-9  # a difference of two deposited moments


def test_output_files_hold_the_reference_records(tmp_path):
    h = make_hybrid(extra=0)
    d = str(tmp_path) + "/"
    h.diag_open(d, nt=4, nout=2)
    for m in (1, 2):
        h.ion_step()
        h.diag_step(m)
    h.diag_close()
    h.sync_to_host()
    nx, ny, nz = h.cfg.nodes
    C, NM = nx * ny * nz, h.ni_max
    para = fortran_records(d + "para.dat")
    assert len(para) == 10
    assert struct.unpack("<3i3f", para[0])[:3] == (nx, ny, nz)
    nt, dtsub, ntsub, dt, nout = struct.unpack("<ififi", para[1])
    assert (nt, ntsub, nout) == (4, h.cfg.ntsub, 2) and abs(dt - h.cfg.dt) < 1e-7
    assert len(para[2]) == 50 and para[2].decode().rstrip() == d[:50].rstrip()  # character(50) out_dir
    assert struct.unpack("<i", para[4])[0] == NM
    energy = fortran_records(d + "c.energy.dat")
    assert [struct.unpack("<i", r)[0] for r in energy[0::2]] == [1, 2] and all(len(r) == 48 for r in energy[1::2])
    e = h.energy()
    assert abs(struct.unpack("<12f", energy[3])[2] - e[0]) <= 1e-6 * e[0]  # Evp of the last step
    npr = fortran_records(d + "c.np.dat")
    assert len(npr) == 2 and struct.unpack("<i", npr[0])[0] == 2
    assert np.array_equal(np.frombuffer(npr[1], "<f4"), h.np.ravel(order="F").astype(np.float32))
    xr = fortran_records(d + "c.xp_0.dat")
    assert np.array_equal(np.frombuffer(xr[1], "<f4"), h.xp.ravel(order="F").astype(np.float32))
    for name, n in (("c.b1.dat", 3 * C), ("c.E.dat", 3 * C), ("c.up.dat", 3 * C), ("c.temp_p.dat", C),
                    ("c.mnp.dat", C), ("c.vp_0.dat", 3 * NM), ("c.mrat_0.dat", NM), ("c.aj.dat", 3 * C)):
        r = fortran_records(d + name)
        assert len(r) == 2 and len(r[1]) == 4 * n, name
    b1 = np.frombuffer(fortran_records(d + "c.b1.dat")[1], "<f4")
    assert np.array_equal(b1, h.bt.ravel(order="F").astype(np.float32))


def _state(h):
    h.sync_to_host()
    N = int(h.ni_tot[0])
    return {n: getattr(h, n)[:N].copy() if n in ("xp", "vp", "vp1", "mrat", "beta_p") else getattr(h, n).copy()
            for n in ("xp", "vp", "vp1", "mrat", "beta_p", "b1", "b12", "bt", "np", "up", "E")}


def test_checkpoint_fp64_round_trip_and_resume(tmp_path):
    h = make_hybrid(extra=0)
    h.run(2)
    path = str(tmp_path / "ck.bin")
    h.checkpoint_write(path)
    saved = _state(h)
    h.run(2)
    a = _state(h)
    g = make_hybrid(extra=0, seed=99)  # a different load, overwritten by the restart
    g.checkpoint_read(path)
    r = _state(g)
    for k in saved:
        assert np.array_equal(r[k], saved[k]), k
    g.run(2)
    b = _state(g)
    for k in ("xp", "vp", "b1", "np"):
        assert relerr(b[k], a[k]) < 1e-10, k


def test_checkpoint_fp32_state_is_exact_and_resumes(tmp_path):
    cells = (16, 8, 8)
    h = make_hybrid(cells=cells, ppc=8, db=0.0, extra=0)
    h.f32_begin()
    h.f32_run(2)
    path = str(tmp_path / "ck32.bin")
    h.checkpoint_write(path)
    g = make_hybrid(cells=cells, ppc=8, db=0.0, extra=0, seed=42)
    g.checkpoint_read(path)
    h.f32_end()
    g.f32_end()
    a, b = _state(h), _state(g)
    for k in a:
        assert np.array_equal(a[k], b[k]), k  # the restored FP32 state is the saved one
    for x in (h, g):
        x.f32_begin()
        x.f32_run(3)
        x.f32_end()
    a, b = _state(h), _state(g)
    assert rel_l2(b["b1"] - h.b0, a["b1"] - h.b0) < 1e-4
    assert rel_l2(b["np"], a["np"]) < 1e-5
