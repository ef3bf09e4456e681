"""Pin the oracle against the reference's only golden vector, b0.dat.

b0.dat is written by grd6_setup (initial.f:136-139) from the scalars that
initparameters (inputs.f:125-172) derives from inputs.dat, all in FP32
(-real-size 32, makefile:1).  The FP32 restatement must rebuild the file
byte for byte.
"""
import hashlib
import json
import struct
from pathlib import Path

import numpy as np

FIX = json.loads((Path(__file__).parent / "golden" / "b0_dat.json").read_text())


def _fortran_unformatted(*records: bytes) -> bytes:
    out = b""
    for r in records:
        out += struct.pack("<i", len(r)) + r + struct.pack("<i", len(r))
    return out


def test_initparameters_fp32_reproduces_b0z(oracle_mod):
    inp = FIX["inputs"]
    d = oracle_mod.initparameters(inp["b0_init"], int(inp["ion_amu"]), inp["nf_init"], inp["dt_frac"],
                                  inp["dx_frac"], inp["nu_init_frac"], FIX["ntsub"], precision="f32")
    q = np.float32(1.6e-19)
    eoverm = np.float32(q / np.float32(d["mion"]))
    b0z = np.float32(np.float32(inp["b0_init"]) * eoverm)
    assert "0x%08x" % int(b0z.view(np.uint32)) == FIX["b0z_float32_hex"]


def test_grd6_setup_fp32_rebuilds_b0_dat_bytes(oracle_mod):
    inp = FIX["inputs"]
    nx, ny, nz, _ = FIX["shape"]
    d = oracle_mod.initparameters(inp["b0_init"], int(inp["ion_amu"]), inp["nf_init"], inp["dt_frac"],
                                  inp["dx_frac"], inp["nu_init_frac"], FIX["ntsub"], precision="f32")
    o = oracle_mod.Oracle(nx, ny, nz, 1, d["dt"], FIX["ntsub"], d["alpha"], 1.0, dx=d["dx"], dy=d["dy"],
                          delz=d["delz"], precision="f32")
    f = lambda n: np.zeros((nx, ny, nz, n), dtype=np.float32, order="F")
    b0, b1, b12, b1p2, bt, btc, up, aj, E = (f(3) for _ in range(9))
    np_ = np.zeros((nx, ny, nz), dtype=np.float32, order="F")
    nu = np.zeros((nx, ny, nz), dtype=np.float32, order="F")
    o.bind_fields(b0, b1, b12, b1p2, bt, btc, np_, up, aj, E, nu)
    o.grd6_setup(inp["b0_init"], d["mion"], d["nu_init"])
    raw = _fortran_unformatted(struct.pack("<i", nz), b0.tobytes(order="F"))
    assert len(raw) == FIX["file_bytes"]
    assert hashlib.sha256(raw).hexdigest() == FIX["sha256"]
    # the other time levels start equal to b0 (initial.f:82-85)
    for a in (b1, b12, b1p2, bt):
        assert np.array_equal(a, b0)


def test_grd7_uniform_grid_fp32(oracle_mod):
    # the coordinate arrays of the golden run (dx = lambda_i*dx_frac)
    inp = FIX["inputs"]
    d = oracle_mod.initparameters(inp["b0_init"], int(inp["ion_amu"]), inp["nf_init"], inp["dt_frac"],
                                  inp["dx_frac"], inp["nu_init_frac"], FIX["ntsub"], precision="f32")
    nx, ny, nz, _ = FIX["shape"]
    o = oracle_mod.Oracle(nx, ny, nz, 1, d["dt"], 10, d["alpha"], 1.0, dx=d["dx"], dy=d["dy"], delz=d["delz"],
                          precision="f32")
    c = o.coords()
    dz = np.float32(d["delz"])
    qz = np.cumsum(np.full(nz, dz, dtype=np.float32), dtype=np.float32)
    assert np.array_equal(c["qz"], qz)  # q(k) = q(k-1) + dz_grid(k), initial.f:233-237
    assert np.array_equal(c["qy"], (np.arange(1, ny + 1) * np.float32(d["dy"])).astype(np.float32))
    # ends are set to 0.5 (initial.f:262-263); interior ratios are 0.5 only up
    # to FP32 rounding of the cumulative node sums in physical units
    # (xrat(2) = 0.4999999; zrat deviates up to ~1.4e-6 over 401 nodes)
    for r in (c["xrat"], c["yrat"], c["zrat"]):
        assert r[0] == np.float32(0.5) and r[-1] == np.float32(0.5)
        assert np.max(np.abs(r - np.float32(0.5))) <= 1e-4  # ulp(q)/dz at q ~ 1.4e5 km
