"""Python face of the CPU oracle (TEST INFRASTRUCTURE ONLY).

``Oracle`` mirrors ``swap_gb300.hybrid.Hybrid`` method for method (same
names and arguments as the reference subroutines) but computes on the host
with the C++ restatement in swap_oracle.hpp, in place on the numpy arrays it
is handed.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        for p in ("oracle_", "oracle32_"):
            getattr(_lib, p + "create").restype = C.c_void_p
            getattr(_lib, p + "create").argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int64, C.c_double, C.c_int,
                                                                                        C.c_double, C.c_double,
                                                                                        C.c_double, C.c_int]
            getattr(_lib, p + "last_error").restype = C.c_char_p
            getattr(_lib, p + "max_abs_divB").restype = C.c_double
    return _lib


class Oracle:
    """CPU restatement with the reference's subroutine interface."""

    def __init__(self, nx, ny, nz, ni_max, dt, ntsub, alpha, beta, dx=1.0, dy=1.0, delz=1.0, grad_pe=0.0,
                 precision="f64", nthreads=1):
        self.lib = load()
        self.p = "oracle_" if precision == "f64" else "oracle32_"
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.nx, self.ny, self.nz, self.ni_max = nx, ny, nz, int(ni_max)
        self.h = self._fn("create")(nx, ny, nz, dx, dy, delz, int(ni_max), dt, ntsub, alpha, beta, grad_pe,
                                    nthreads)
        if not self.h:
            raise RuntimeError("oracle create failed")
        self.h = C.c_void_p(self.h)

    def _fn(self, name):
        return getattr(self.lib, self.p + name)

    def _ptr(self, a):
        if a is None:
            return None
        assert a.dtype in (self.dtype, np.int32), (a.dtype, self.dtype)
        return a.ctypes.data_as(C.c_void_p)

    def _call(self, name, *arrays, extra=()):
        r = self._fn(name)(self.h, *[self._ptr(a) for a in arrays], *extra)
        if r:
            raise RuntimeError(f"oracle {name}: " + self._fn("last_error")(self.h).decode())

    def close(self):
        if self.h:
            self._fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # geometry ---------------------------------------------------------
    def coords(self):
        out = {}
        names = ("qx", "qy", "qz", "dx_grid", "dy_grid", "dz_grid", "dx_cell", "dy_cell", "dz_cell", "xrat",
                 "yrat", "zrat")
        ns = (self.nx, self.ny, self.nz) * 4
        arrs = [np.zeros(n, dtype=self.dtype) for n in ns]
        self._fn("get_coords")(self.h, *[a.ctypes.data_as(C.c_void_p) for a in arrs])
        for n, a in zip(names, arrs):
            out[n] = a
        return out

    def bind_particles(self, xp, vp, vp1, mrat, beta_p, ijkp, ni_tot):
        self._keep_p = (xp, vp, vp1, mrat, beta_p, ijkp, ni_tot)
        self._call("bind_particles", xp, vp, vp1, mrat, beta_p, ijkp, ni_tot)

    def bind_fields(self, b0, b1, b12, b1p2, bt, btc, np_, up, aj, E, nu):
        self._keep_f = (b0, b1, b12, b1p2, bt, btc, np_, up, aj, E, nu)
        self._call("bind_fields", b0, b1, b12, b1p2, bt, btc, np_, up, aj, E, nu)

    def ijkp(self):
        out = np.zeros((self.ni_max, 3), dtype=np.int32, order="F")
        self._fn("get_ijkp")(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def wght(self):
        out = np.zeros((self.ni_max, 8), dtype=self.dtype, order="F")
        self._fn("get_wght")(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def set_nthreads(self, n):
        self._fn("set_nthreads")(self.h, int(n))

    def load_maxwellian(self, seed, ppc, vth, u, stream=0, mrat=1.0, beta_p=1.0, first=0):
        """The workloads' stratified Maxwellian load into the bound particle
        arrays (oracle_capi.cpp load_maxwellian); sets Ni_tot = first + count."""
        cnt = C.c_int64()
        self._call("load_maxwellian", extra=(C.c_uint64(int(seed)), C.c_uint32(int(stream)), C.c_int(int(ppc)),
                                             C.c_double(vth), C.c_double(u[0]), C.c_double(u[1]),
                                             C.c_double(u[2]), C.c_double(mrat), C.c_double(beta_p),
                                             C.c_int64(int(first)), C.byref(cnt)))
        return cnt.value

    # gutsp.f ----------------------------------------------------------
    def get_interp_weights(self, xp):
        self._call("get_interp_weights", xp)

    def update_np(self, np_):
        self._call("update_np", np_)

    def update_np_local(self, np_):
        self._call("update_np_local", np_)

    def update_up(self, vp, np_, up):
        self._call("update_up", vp, np_, up)

    def extrapol_up(self, up, vp, vp1, np_):
        self._call("extrapol_up", up, vp, vp1, np_)

    def get_Ep(self, Ep, aj, np_, up, btc, nu):
        self._call("get_Ep", Ep, aj, np_, up, btc, nu)

    def get_vplus_vminus(self, Ep, btc, vp, vplus, vminus):
        self._call("get_vplus_vminus", Ep, btc, vp, vplus, vminus)

    def improve_up(self, vp1, vplus, vminus, up, np_):
        self._call("improve_up", vp1, vplus, vminus, up, np_)

    def get_vp_final(self, Ep, vp, vp1, vplus):
        self._call("get_vp_final", Ep, vp, vp1, vplus)

    def move_ion_half(self, xp, vp, vp1, input_p):
        self._call("move_ion_half", xp, vp, vp1, input_p)

    # gutsf.f ----------------------------------------------------------
    def curlB(self, bt, np_, aj):
        self._call("curlB", bt, np_, aj)

    def edge_to_center(self, bt, btc):
        self._call("edge_to_center", bt, btc)

    def face_to_center(self, v, vc):
        self._call("face_to_center", v, vc)

    def get_E(self, E, b0, bt, aj, up, np_, nu):
        self._call("get_E", E, b0, bt, aj, up, np_, nu)

    def predict_B(self, b0, b1, b12, b1p2, bt, E, aj, up, np_, nu, dtsub):
        self._call("predict_B", b0, b1, b12, b1p2, bt, E, aj, up, np_, nu, extra=(C.c_double(dtsub),))

    def correct_B(self, b0, b1, b1p2, E, aj, up, np_, nu, dtsub):
        self._call("correct_B", b0, b1, b1p2, E, aj, up, np_, nu, extra=(C.c_double(dtsub),))

    def f_update_tlev(self, b1, b12, b1p2, bt, b0):
        self._call("f_update_tlev", b1, b12, b1p2, bt, b0)

    def check_time_step(self, bt, np_, dtsub, ntf):
        d, n = C.c_double(dtsub), C.c_double(ntf)
        self._call("check_time_step", bt, np_, extra=(C.byref(d), C.byref(n)))
        return d.value, n.value

    def max_abs_divB(self, b):
        return self._fn("max_abs_divB")(self.h, self._ptr(b))

    def energy(self):
        out = np.zeros(4)
        self._fn("energy")(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def ion_step(self):
        self._call("ion_step")

    def run(self, n):
        for _ in range(n):
            self.ion_step()

    def sort_perm(self, ni_tot):
        perm = np.zeros(ni_tot, dtype=np.int64)
        counts = np.zeros(self.nx * self.ny * self.nz, dtype=np.int64)
        r = self._fn("sort_perm")(self.h, perm.ctypes.data_as(C.c_void_p), counts.ctypes.data_as(C.c_void_p))
        if r:
            raise RuntimeError("oracle sort_perm failed")
        return perm, counts

    def update_rho(self, mnp, mion=1.0):
        self._call("update_rho", mnp, extra=(C.c_double(mion),))

    def get_temperature(self, xp, vp, np_, temp_p, mion=1.0):
        self._call("get_temperature", xp, vp, np_, temp_p, extra=(C.c_double(mion),))

    # sources and sinks ----------------------------------------------
    def set_sources(self, src, step0=0):
        """src: a swap_gb300.abi.Sources (the same struct layout)."""
        self._src = src
        r = self._fn("set_sources")(self.h, C.byref(src), C.c_int64(int(step0)))
        if r:
            raise RuntimeError("oracle set_sources failed")

    def chex_count(self):
        f = self._fn("chex_count")
        f.restype = C.c_int64
        return int(f(self.h))

    def Ionize_sw_mp(self, np_, vp, vp1, xp, m_tstep, input_p, up):
        r = self._fn("Ionize_sw_mp")(self.h, self._ptr(np_), self._ptr(vp), self._ptr(vp1), self._ptr(xp),
                                     C.c_int32(int(m_tstep)), self._ptr(input_p), self._ptr(up))
        if r:
            raise RuntimeError("oracle Ionize_sw_mp: " + self._fn("last_error")(self.h).decode())

    def inflow_x(self, m_tstep):
        self._call("inflow_x", extra=(C.c_int32(int(m_tstep)),))

    def ionize_cloud(self, m_tstep):
        self._call("ionize_cloud", extra=(C.c_int32(int(m_tstep)),))

    def remove_outflow_x(self):
        self._call("remove_outflow_x")

    def remove_ion(self, xp, vp, vp1, ion_l):
        self._call("remove_ion", xp, vp, vp1, extra=(C.c_int32(int(ion_l)),))

    def res_chex(self, xp, vp, m_tstep):
        n = C.c_int64()
        self._call("res_chex", xp, vp, extra=(C.c_int32(int(m_tstep)), C.byref(n)))
        return n.value

    def move_ion_half_open(self, xp, vp):
        self._call("move_ion_half_open", xp, vp)

    def grd6_setup(self, b0_init, mion, nu_init):
        self._fn("grd6_setup")(self.h, C.c_double(b0_init), C.c_double(mion), C.c_double(nu_init))


def initparameters(b0_init, ion_amu, nf_init, dt_frac, dx_frac, nu_init_frac, ntsub=10, precision="f32"):
    """inputs.f:125-172 restated; returns mion, omega_p, lambda_i, dx, dy, delz, dt, dtsub_init, nu_init, alpha."""
    lib = load()
    out = (C.c_double * 10)()
    fn = lib.oracle32_initparameters if precision == "f32" else lib.oracle_initparameters
    fn(C.c_double(b0_init), int(ion_amu), C.c_double(nf_init), C.c_double(dt_frac), C.c_double(dx_frac),
       C.c_double(nu_init_frac), int(ntsub), out)
    keys = ("mion", "omega_p", "lambda_i", "dx", "dy", "delz", "dt", "dtsub_init", "nu_init", "alpha")
    return dict(zip(keys, list(out)))


def standalone(cfg, ni_max=None, precision="f64", nthreads=1):
    """An Oracle for a workload (a swap_gb300.hybrid.RunConfig) with its own
    arrays of maind.f:38-70: the uniform grid of grd7, b0 = (0,0,cfg.b0) and
    the time levels equal to it, nu = cfg.nu (grd6_setup, initial.f:54-85),
    particles loaded by the oracle's own load_maxwellian with cfg's seed and
    the workload's sources set.  Nothing of the product is loaded."""
    nx, ny, nz = cfg.nodes
    NM = int(ni_max if ni_max is not None else cfg.ni_max_hint())
    o = Oracle(nx, ny, nz, NM, cfg.dt, cfg.ntsub, cfg.alpha, cfg.beta, grad_pe=cfg.grad_pe, precision=precision,
               nthreads=nthreads)
    dt = o.dtype
    f3 = lambda: np.zeros((NM, 3), dtype=dt, order="F")
    o.xp, o.vp, o.vp1 = f3(), f3(), f3()
    o.mrat, o.beta_p = np.ones(NM, dtype=dt), np.ones(NM, dtype=dt)
    o.ijkp_arr = np.zeros((1, 3), dtype=np.int32, order="F")
    o.ni_tot = np.zeros(1, dtype=np.int32)
    grid = lambda *c: np.zeros((nx, ny, nz) + c, dtype=dt, order="F")
    o.b0 = grid(3)
    o.b0[..., 2] = cfg.b0
    for n in ("b1", "b12", "b1p2", "bt"):
        setattr(o, n, o.b0.copy(order="F"))
    for n in ("btc", "up", "aj", "E"):
        setattr(o, n, grid(3))
    o.np = grid()
    o.nu = grid()
    o.nu[...] = cfg.nu
    o.input_p = np.zeros(3, dtype=dt)
    o.bind_particles(o.xp, o.vp, o.vp1, o.mrat, o.beta_p, o.ijkp_arr, o.ni_tot)
    o.bind_fields(o.b0, o.b1, o.b12, o.b1p2, o.bt, o.btc, o.np, o.up, o.aj, o.E, o.nu)
    o.load_maxwellian(cfg.seed, cfg.ppc, cfg.vth, cfg.u)
    src = cfg.make_sources()
    if src is not None:
        o.set_sources(src, 0)
    o.cfg = cfg
    return o


def from_hybrid_arrays(h, precision="f64", nthreads=1):
    """An Oracle with the same geometry/parameters as a Hybrid-like object and
    its own copies of that object's host arrays (bound like the Fortran's)."""
    cfg = h.cfg
    nx, ny, nz = cfg.nodes
    co = getattr(h, "coords", None)
    o = Oracle(nx, ny, nz, h.ni_max, cfg.dt, cfg.ntsub, cfg.alpha, cfg.beta, dx=getattr(co, "dx", 1.0),
               dy=getattr(co, "dy", 1.0), delz=getattr(co, "delz", 1.0), grad_pe=cfg.grad_pe,
               precision=precision, nthreads=nthreads)
    dt = o.dtype
    cp = lambda a: np.array(a, dtype=dt, order="F", copy=True)
    o.xp, o.vp, o.vp1 = cp(h.xp), cp(h.vp), cp(h.vp1)
    o.Ep, o.vplus, o.vminus = cp(h.Ep), cp(h.vplus), cp(h.vminus)
    o.mrat, o.beta_p = cp(h.mrat), cp(h.beta_p)
    o.ijkp_arr = np.zeros((h.ni_max, 3), dtype=np.int32, order="F")
    o.ni_tot = np.array(h.ni_tot, dtype=np.int32, copy=True)
    for n in ("b0", "b1", "b12", "b1p2", "bt", "btc", "np", "up", "aj", "E", "nu"):
        setattr(o, n, cp(getattr(h, n)))
    o.input_p = np.zeros(3, dtype=dt)
    o.bind_particles(o.xp, o.vp, o.vp1, o.mrat, o.beta_p, o.ijkp_arr, o.ni_tot)
    o.bind_fields(o.b0, o.b1, o.b12, o.b1p2, o.bt, o.btc, o.np, o.up, o.aj, o.E, o.nu)
    o.cfg = cfg
    return o
