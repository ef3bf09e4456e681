"""Generate the fixtures of tests/golden from the reference's source tree.

b0_dat.json -- the reference's own golden vector.
The reference ships one golden vector, b0.dat, written by grd6_setup
(initial.f:136-139) as a Fortran unformatted sequential file with two
records: nz (int32) and b0(nx,ny,nz,3) (float32).  This script decodes it and
the run-time inputs it was made from (inputs.dat, read by inputs.f:84-119)
into a small JSON fixture, so that tests need nothing from the reference at
run time.

reference_interfaces.json -- the argument lists of the reference subroutines
that the Fortran wrappers replace, with the file and line of each header,
so that a test can hold the wrappers to the reference's interfaces.

Usage: python tests/golden/make_fixtures.py REFERENCE_DIR
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def read_records(raw: bytes):
    recs, off = [], 0
    while off < len(raw):
        (n,) = struct.unpack_from("<i", raw, off)
        body = raw[off + 4: off + 4 + n]
        (n2,) = struct.unpack_from("<i", raw, off + 4 + n)
        assert n == n2, "bad record markers"
        recs.append(body)
        off += 8 + n
    return recs


def parse_inputs(text: str):
    keys = ["b0_init", "ion_amu", "m_pu", "nf_init", "dt_frac", "nt", "nout", "vsw", "vth", "Ni_tot_frac",
            "dx_frac", "nu_init_frac", "ppc", "out_dir"]
    vals = {}
    for k, line in zip(keys, text.splitlines()):
        tok = line.split("!")[0].strip().split()[0]
        vals[k] = tok.strip("'") if k == "out_dir" else float(tok)
    return vals


def main(ref: Path):
    raw = (ref / "b0.dat").read_bytes()
    recs = read_records(raw)
    (nz,) = struct.unpack("<i", recs[0])
    b0 = np.frombuffer(recs[1], dtype="<f4")
    nxy = b0.size // (3 * nz)
    nx = ny = int(round(nxy ** 0.5))
    b0 = b0.reshape((nx, ny, nz, 3), order="F")
    bz = np.unique(b0[..., 2])
    assert bz.size == 1 and not np.any(b0[..., :2])
    inputs = parse_inputs((ref / "inputs.dat").read_text())
    fx = {
        "source": "b0.dat (grd6_setup, initial.f:136-139) and inputs.dat (inputs.f:84-119) of pdelamere/SWAP",
        "file_bytes": len(raw),
        "sha256": hashlib.sha256(raw).hexdigest(),
        "records": [len(r) for r in recs],
        "nz": nz,
        "shape": [nx, ny, nz, 3],
        "b0_xy_all_zero": True,
        "b0z_float32_hex": "0x%08x" % int(np.asarray(bz[0], dtype="<f4").view("<u4")),
        "b0z": float(bz[0]),
        "inputs": inputs,
        "ntsub": 10,
    }
    out = HERE / "b0_dat.json"
    out.write_text(json.dumps(fx, indent=1) + "\n")
    print("wrote", out)
    interfaces(ref)


# The subroutines of the ion step that the Fortran wrappers stand in for.
WRAPPED = ["get_interp_weights", "update_np", "update_up", "extrapol_up", "get_Ep", "get_vplus_vminus",
           "improve_up", "get_vp_final", "move_ion_half", "curlB", "edge_to_center", "face_to_center", "get_E",
           "predict_B", "correct_B", "f_update_tlev", "check_time_step", "periodic", "periodic_scalar",
           "Ionize_sw_mp", "remove_ion", "res_chex", "update_rho", "get_temperature"]


def interfaces(ref: Path):
    """Each wrapped subroutine's header line in the fixed-form sources:
    its dummy arguments in order, and where it stands."""
    found = {}
    for f in sorted(ref.glob("*.f")):
        if f.name == "old_routines.f":  # superseded copies, not compiled by the makefile
            continue
        for ln, line in enumerate(f.read_text(errors="replace").splitlines(), 1):
            if line[:1] in "cC*!":
                continue
            m = re.match(r"^\s+subroutine\s+(\w+)\s*\(([^)]*)\)", line, re.I)
            if m and m.group(1) in WRAPPED:
                assert m.group(1) not in found, ("defined twice", m.group(1))
                found[m.group(1)] = {"args": [a.strip() for a in m.group(2).split(",")], "at": f"{f.name}:{ln}"}
    missing = sorted(set(WRAPPED) - set(found))
    assert not missing, missing
    out = HERE / "reference_interfaces.json"
    out.write_text(json.dumps({"source": "SUBROUTINE headers of pdelamere/SWAP", "subroutines": found},
                              indent=1, sort_keys=True) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SWAP_REFERENCE")
    if not src:
        sys.exit("usage: make_fixtures.py REFERENCE_DIR (or set SWAP_REFERENCE): the SWAP source tree holding b0.dat")
    main(Path(src))
