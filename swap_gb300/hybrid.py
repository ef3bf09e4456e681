"""Host-side mirror of the reference's hot-path interface.

``Hybrid`` owns the arrays that maind.f declares (maind.f:38-70) in Fortran
layout, registers them with the C-ABI context, and exposes one method per
reference subroutine with the same name and arguments (gutsp.f, gutsf.f,
grid_interp.f, boundary.f), so a replay of maind.f reads like the Fortran.
All computation runs in the sm_103a library; there is no CPU path here.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .grid import Coords, grd6_setup, grd7


@dataclass
class RunConfig:
    """A workload in normalized units: d_i = 1, Omega_i = 1, v_A = 1, n0 = 1
    (alpha*n0 = 1, B0 = 1 as a gyrofrequency)."""

    name: str
    cells: tuple  # physical cells (x, y, z); nodes = cells + 2 ghosts
    ppc: int
    vth: float = 0.5
    u: tuple = (2.0, 0.0, 0.0)
    b0: float = 1.0
    n0: float = 1.0
    dt: float = 0.05
    ntsub: int = 10
    nu: float = 0.002  # nu_init_frac of inputs.dat, in units of Omega_i
    steps: int = 100
    seed: int = 1
    grad_pe: float = 0.0
    sources: dict = field(default_factory=dict)  # swap_sources fields; empty = periodic box, no sources
    extra: dict = field(default_factory=dict)

    @property
    def nodes(self):
        return tuple(c + 2 for c in self.cells)

    @property
    def n_particles(self) -> int:
        return int(np.prod(self.cells)) * self.ppc

    @property
    def alpha(self) -> float:
        return 1.0 / self.n0

    @property
    def beta(self) -> float:
        # one macro-particle per cell of volume 1 carries n0/ppc
        return self.ppc / self.n0

    def make_sources(self):
        """The workload's sources and sinks as an abi.Sources (None when it has none)."""
        return abi.make_sources(**self.sources) if self.sources else None

    def cloud_ions_per_step(self) -> float:
        """Expected ions the cloud ionization creates per step: the sum over
        cell centres of beta*beta_heavy*n_n*nu_ion*dt (unit cells)."""
        q = self.sources
        if not q.get("nu_ion"):
            return 0.0
        cx, cy, cz = (np.arange(c) + 1.5 for c in self.cells)
        r2 = ((cx[:, None, None] - q["cloud_x"]) ** 2 + (cy[None, :, None] - q["cloud_y"]) ** 2
              + (cz[None, None, :] - q["cloud_z"]) ** 2) / q["cloud_r0"] ** 2
        dens = float(np.sum(q["cloud_N0"] / (1.0 + r2)))
        return self.beta * q.get("beta_heavy", 1.0) * dens * q["nu_ion"] * self.dt

    def inflow_ions_per_step(self) -> float:
        """Ions entering through the open x face per step, at most: the
        face's cells times inflow_ppc times (u_x + vth) dt (unit cells)."""
        q = self.sources
        if not q.get("x_open"):
            return 0.0
        face = self.cells[1] * self.cells[2] * q.get("inflow_ppc", 0)
        return face * (abs(q.get("inflow_ux", 0.0)) + q.get("inflow_vth", 0.0)) * self.dt

    def ni_max_hint(self, steps: int | None = None) -> int:
        """Particle capacity with headroom for a workload whose count varies:
        10% for inflow and outflow, plus the cloud's new ions over `steps`
        (default: the workload's step count), plus, with charge exchange, every
        ion that enters in that time: an exchanged ion is heavy and at rest,
        and stays in the box far longer than the step count."""
        n = self.n_particles
        if not self.sources:
            return n
        per_step = self.cloud_ions_per_step()
        if self.sources.get("cx_a"):
            per_step += self.inflow_ions_per_step()
        return int(n * 1.10 + 1.1 * per_step * (self.steps if steps is None else steps)) + 4096


def config(n: int, **over) -> RunConfig:
    """The named workloads.

    0: periodic box of 64x32x32 cells, 16 ppc (1,048,576 ions; the stated
       524,288 is 8 ppc), u = (2,0,0), 100 steps, seed 1.
    1: 256x128x128 cells, 32 ppc (134,217,728 ions), 200 steps, seed 2, with
       the x axis open: a drifting Maxwellian (u = (2,0,0), vth 0.5) enters
       through x = q(1) from a one-cell slab of 32 ions per face cell and ions
       leaving in x are removed; periodic in y and z.
    2: 256x128x128 cells, 16 ppc solar-wind H+ at u = (4,0,0) through an open
       x axis, a neutral cloud N0/(1+(r/5)^2) at the box centre (N0 = 1000)
       ionized at 1e-3 Omega_i into mass-16 ions at rest, charge exchange
       sigma = 1 - 0.1 ln v_rel; 300 steps, seed 3.
    3: the physics of 2 on 512x256x256 cells at 16 ppc (536,870,912 ions),
       1000 steps, seed 4 (the FP32 form against an FP64 run).
    4: 3 with a stronger B0 (2: Omega_i = 2, v_A = 2), the ion step kept at
       0.05 / Omega_i (dt = 0.025) and 20 field subcycles per ion step,
       seed 5 (the learned field surrogate's workload).
    """
    base = {
        0: dict(name="uniform H+ 64x32x32, 16 ppc", cells=(64, 32, 32), ppc=16, steps=100, seed=1),
        1: dict(name="H+ 256x128x128, 32 ppc, x inflow/outflow", cells=(256, 128, 128), ppc=32, steps=200,
                seed=2),
        2: dict(name="pickup ions 256x128x128, 16 ppc, cloud + charge exchange", cells=(256, 128, 128), ppc=16,
                u=(4.0, 0.0, 0.0), steps=300, seed=3),
        3: dict(name="pickup ions 512x256x256, 16 ppc, cloud + charge exchange", cells=(512, 256, 256), ppc=16,
                u=(4.0, 0.0, 0.0), steps=1000, seed=4),
        4: dict(name="pickup ions 512x256x256, 16 ppc, strong B0, 20 subcycles", cells=(512, 256, 256), ppc=16,
                u=(8.0, 0.0, 0.0), b0=2.0, dt=0.025, ntsub=20, steps=1000, seed=5),
    }[n]
    base.update(over)
    cfg = RunConfig(**base)
    if n in (1, 2, 3, 4) and "sources" not in over:
        src = dict(seed=cfg.seed, x_open=1, inflow_ppc=cfg.ppc, inflow_vth=cfg.vth, inflow_ux=cfg.u[0],
                   inflow_uy=cfg.u[1], inflow_uz=cfg.u[2])
        if n >= 2:
            cx, cy, cz = (c / 2.0 + 1.0 for c in cfg.cells)  # box centre (q(1) = 1 with unit spacing)
            src.update(cloud_N0=1000.0, cloud_r0=5.0, cloud_x=cx, cloud_y=cy, cloud_z=cz, nu_ion=1e-3,
                       mrat_heavy=1.0 / 16.0, beta_heavy=1.0, cx_a=1.0, cx_b=0.1)
        cfg.sources = src
    return cfg


class Hybrid:
    """One context on the current GPU with the reference's arrays bound."""

    def __init__(self, cfg: RunConfig, ni_max: int | None = None, coords: Coords | None = None,
                 pinned: bool = False, work_arrays: bool = True, real_bytes: int = 8):
        """work_arrays=False leaves out the arrays only the per-subroutine
        entries take (Ep, vplus, vminus, ijkp) and their device mirrors: the
        fused steps keep their own, which saves 84 B per particle on each side.
        real_bytes=4 holds every real array in float32, as SWAP built with
        -real-size 32 (makefile:1) does; the context converts at the boundary."""
        self.cfg = cfg
        self.lib = abi.load()
        nx, ny, nz = cfg.nodes
        self.coords = coords or grd7(nx, ny, nz)
        self.ni_max = int(ni_max if ni_max is not None else cfg.n_particles)
        NM = self.ni_max
        self.real_bytes = int(real_bytes)
        self.rdtype = np.float32 if self.real_bytes == 4 else np.float64
        self.dims = abi.Dims(nx, ny, nz, self.real_bytes, NM)
        self.params = abi.Params(cfg.dt, cfg.alpha, cfg.beta, self.coords.dx, self.coords.dy, cfg.grad_pe, cfg.ntsub, 0)
        self._coords_c = abi.Coords(*[abi.dptr(getattr(self.coords, n)) for n in Coords.ARRAYS])
        self._pins = []
        # particle arrays (maind.f:54-59, global.f:44,96,100)
        f = (lambda: self._pinned((NM, 3))) if pinned else (lambda: np.zeros((NM, 3), dtype=self.rdtype, order="F"))
        self.xp, self.vp, self.vp1 = f(), f(), f()
        if work_arrays:
            self.Ep, self.vplus, self.vminus = f(), f(), f()
        self.mrat = self._pinned((NM,)) if pinned else np.zeros(NM, dtype=self.rdtype)
        self.beta_p = self._pinned((NM,)) if pinned else np.zeros(NM, dtype=self.rdtype)
        self.mrat[:] = 1.0
        self.beta_p[:] = 1.0
        self.ijkp = np.zeros((NM, 3) if work_arrays else (1, 3), dtype=np.int32, order="F")
        self.ni_tot = np.zeros(1, dtype=np.int32)
        # fields (maind.f:38-70)
        flds = grd6_setup(self.coords, cfg.b0, cfg.nu)
        for k, v in flds.items():
            if pinned:
                pv = self._pinned(v.shape)
                pv[...] = v
                v = pv
            elif v.dtype != self.rdtype:
                v = np.asarray(v, dtype=self.rdtype, order="F")
            setattr(self, k, v)
        self.input_p = np.zeros(3, dtype=self.rdtype)
        ctx = C.c_void_p()
        abi.check(self.lib, None, self.lib.swap_init(C.byref(ctx), C.byref(self.dims), C.byref(self.params),
                                                       C.byref(self._coords_c)))
        self.ctx = ctx
        self._check(self.lib.swap_bind_particles(ctx, abi.rptr(self.xp), abi.rptr(self.vp), abi.rptr(self.vp1),
                                                 abi.rptr(self.mrat), abi.rptr(self.beta_p),
                                                 abi.iptr(self.ijkp) if work_arrays else None,
                                                 abi.iptr(self.ni_tot)))
        self._check(self.lib.swap_bind_fields(ctx, *[abi.rptr(getattr(self, n)) for n in (
            "b0", "b1", "b12", "b1p2", "bt", "btc", "np", "up", "aj", "E", "nu")]))
        for a in ((self.Ep, self.vplus, self.vminus) if work_arrays else ()) + (self.input_p,):
            self._check(self.lib.swap_bind_array(ctx, a.ctypes.data_as(C.c_void_p), a.nbytes))

    # ---- plumbing ----
    def _pinned(self, shape):
        """A zeroed real Fortran-ordered array in page-locked host memory."""
        import torch

        t = torch.zeros(int(np.prod(shape)), dtype=torch.float32 if self.real_bytes == 4 else torch.float64,
                        pin_memory=True)
        self._pins.append(t)
        return np.ndarray(shape, dtype=self.rdtype, buffer=t.numpy(), order="F")

    def _check(self, code):
        abi.check(self.lib, self.ctx if hasattr(self, "ctx") else None, code)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.swap_finalize(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_maxwellian(self, vth=None, u=None, ppc=None, seed=None, stream=0, mrat=1.0, beta_p=1.0, first=0):
        """Stratified Maxwellian load on the host (replaces part_init.f:146-232)."""
        cfg = self.cfg
        ux, uy, uz = cfg.u if u is None else u
        spec = abi.LoadSpec(cfg.seed if seed is None else seed, stream, cfg.ppc if ppc is None else ppc,
                            cfg.vth if vth is None else vth, ux, uy, uz, mrat, beta_p)
        cnt = C.c_int64()
        if self.real_bytes == 4:  # the loader writes doubles: load into FP64 arrays and round
            NM = self.ni_max
            tmp = [np.zeros((NM, 3), order="F") for _ in range(3)] + [np.zeros(NM), np.zeros(NM)]
            arrs = [abi.dptr(a) for a in tmp]
        else:
            arrs = [abi.dptr(a) for a in (self.xp, self.vp, self.vp1, self.mrat, self.beta_p)]
        abi.check(self.lib, None, self.lib.swap_load_maxwellian_host(
            C.byref(self.dims), C.byref(self._coords_c), C.byref(spec), *arrs, first, C.byref(cnt)))
        if self.real_bytes == 4:
            for dst, src in zip((self.xp, self.vp, self.vp1, self.mrat, self.beta_p), tmp):
                dst[first:first + cnt.value] = src[first:first + cnt.value]
        self.ni_tot[0] = first + cnt.value
        self.mark_host_dirty()
        return cnt.value

    def sync_to_host(self, arr=None):
        self._check(self.lib.swap_sync_to_host(self.ctx, None if arr is None else arr.ctypes.data_as(C.c_void_p)))

    def sync_to_device(self, arr=None):
        self._check(self.lib.swap_sync_to_device(self.ctx, None if arr is None else arr.ctypes.data_as(C.c_void_p)))

    def mark_host_dirty(self, arr=None):
        self._check(self.lib.swap_mark_host_dirty(self.ctx, None if arr is None else arr.ctypes.data_as(C.c_void_p)))

    def set_host_direct(self, on: bool):
        """Let the FP32 form's conversions read and write the FP64 particle arrays in host memory."""
        self._check(self.lib.swap_set_host_direct(self.ctx, int(bool(on))))

    def set_exchange(self, fn):
        """fn(data_ptr, count, kind, stream_ptr) -> int replaces the rank's raw
        deposit sums at data_ptr (device, `count` reals of `kind` bytes) by
        their sum over the ranks (swap_set_exchange); None switches it off."""
        if fn is None:
            self._xfn = None
            self._check(self.lib.swap_set_exchange(self.ctx, abi.EXCHANGE_FN(), None))
            return
        self._xfn = abi.EXCHANGE_FN(lambda user, data, count, kind, stream: fn(data, count, kind, stream))
        self._check(self.lib.swap_set_exchange(self.ctx, self._xfn, None))

    def transfer_bytes(self, reset=False):
        """(h2d, d2h) bytes moved between the bound host arrays and the device since the last reset."""
        h2d, d2h = C.c_int64(), C.c_int64()
        self._check(self.lib.swap_transfer_bytes(self.ctx, C.byref(h2d), C.byref(d2h), int(bool(reset))))
        return h2d.value, d2h.value

    # ---- gutsp.f ----
    def get_interp_weights(self, xp):
        self._check(self.lib.swap_get_interp_weights(self.ctx, abi.rptr(xp)))

    def update_np(self, np_):
        self._check(self.lib.swap_update_np(self.ctx, abi.rptr(np_)))

    def update_up(self, vp, np_, up):
        self._check(self.lib.swap_update_up(self.ctx, abi.rptr(vp), abi.rptr(np_), abi.rptr(up)))

    def extrapol_up(self, up, vp, vp1, np_):
        self._check(self.lib.swap_extrapol_up(self.ctx, abi.rptr(up), abi.rptr(vp), abi.rptr(vp1), abi.rptr(np_)))

    def get_Ep(self, Ep, aj, np_, up, btc, nu):
        self._check(self.lib.swap_get_Ep(self.ctx, *map(abi.rptr, (Ep, aj, np_, up, btc, nu))))

    def get_vplus_vminus(self, Ep, btc, vp, vplus, vminus):
        self._check(self.lib.swap_get_vplus_vminus(self.ctx, *map(abi.rptr, (Ep, btc, vp, vplus, vminus))))

    def improve_up(self, vp1, vplus, vminus, up, np_):
        self._check(self.lib.swap_improve_up(self.ctx, *map(abi.rptr, (vp1, vplus, vminus, up, np_))))

    def get_vp_final(self, Ep, vp, vp1, vplus):
        self._check(self.lib.swap_get_vp_final(self.ctx, *map(abi.rptr, (Ep, vp, vp1, vplus))))

    def move_ion_half(self, xp, vp, vp1, input_p):
        self._check(self.lib.swap_move_ion_half(self.ctx, *map(abi.rptr, (xp, vp, vp1, input_p))))

    # ---- gutsf.f / grid_interp.f / boundary.f ----
    def curlB(self, b1, np_, aj):
        self._check(self.lib.swap_curlB(self.ctx, *map(abi.rptr, (b1, np_, aj))))

    def edge_to_center(self, bt, btc):
        self._check(self.lib.swap_edge_to_center(self.ctx, abi.rptr(bt), abi.rptr(btc)))

    def face_to_center(self, v, vc):
        self._check(self.lib.swap_face_to_center(self.ctx, abi.rptr(v), abi.rptr(vc)))

    def get_E(self, E, b0, bt, aj, up, np_, nu):
        self._check(self.lib.swap_get_E(self.ctx, *map(abi.rptr, (E, b0, bt, aj, up, np_, nu))))

    def predict_B(self, b0, b1, b12, b1p2, bt, E, aj, up, np_, nu, dtsub):
        self._check(self.lib.swap_predict_B(self.ctx, *map(abi.rptr, (b0, b1, b12, b1p2, bt, E, aj, up, np_, nu)),
                                            float(dtsub)))

    def correct_B(self, b0, b1, b1p2, E, aj, up, np_, nu, dtsub):
        self._check(self.lib.swap_correct_B(self.ctx, *map(abi.rptr, (b0, b1, b1p2, E, aj, up, np_, nu)),
                                            float(dtsub)))

    def f_update_tlev(self, b1, b12, b1p2, bt, b0):
        self._check(self.lib.swap_f_update_tlev(self.ctx, *map(abi.rptr, (b1, b12, b1p2, bt, b0))))

    def check_time_step(self, bt, np_, dtsub, ntf):
        d = C.c_double(dtsub)
        n = C.c_double(ntf)
        self._check(self.lib.swap_check_time_step(self.ctx, abi.rptr(bt), abi.rptr(np_), C.byref(d), C.byref(n)))
        return d.value, n.value

    def update_rho(self, mnp):
        self._check(self.lib.swap_update_rho(self.ctx, abi.rptr(mnp)))

    def get_temperature(self, xp, vp, np_, temp_p):
        self._check(self.lib.swap_get_temperature(self.ctx, *map(abi.rptr, (xp, vp, np_, temp_p))))

    def set_mion(self, mion: float):
        self._check(self.lib.swap_set_mion(self.ctx, float(mion)))

    def periodic(self, b):
        self._check(self.lib.swap_periodic(self.ctx, abi.rptr(b)))

    def periodic_scalar(self, b):
        self._check(self.lib.swap_periodic_scalar(self.ctx, abi.rptr(b)))

    # ---- sources and sinks (chem_rates.f, gutsp.f:12-46) ----
    def set_sources(self, src: "abi.Sources", step0: int = 0):
        self._sources = src
        self._check(self.lib.swap_set_sources(self.ctx, C.byref(src), int(step0)))

    def Ionize_sw_mp(self, np_, vp, vp1, xp, m_tstep, input_p, up):
        self._check(self.lib.swap_Ionize_sw_mp(self.ctx, abi.rptr(np_), abi.rptr(vp), abi.rptr(vp1), abi.rptr(xp),
                                               int(m_tstep), abi.rptr(input_p), abi.rptr(up)))

    def remove_ion(self, xp, vp, vp1, ion_l):
        self._check(self.lib.swap_remove_ion(self.ctx, abi.rptr(xp), abi.rptr(vp), abi.rptr(vp1), int(ion_l)))

    def res_chex(self, xp, vp, m_tstep) -> int:
        n = C.c_int64()
        self._check(self.lib.swap_res_chex(self.ctx, abi.rptr(xp), abi.rptr(vp), int(m_tstep), C.byref(n)))
        return n.value

    def inflow_x(self, m_tstep):
        self._check(self.lib.swap_inflow_x(self.ctx, int(m_tstep)))

    def ionize_cloud(self, m_tstep):
        self._check(self.lib.swap_ionize_cloud(self.ctx, int(m_tstep)))

    def remove_outflow_x(self):
        self._check(self.lib.swap_remove_outflow_x(self.ctx))

    def chex_count(self) -> int:
        n = C.c_int64()
        self._check(self.lib.swap_chex_count(self.ctx, C.byref(n)))
        return n.value

    # ---- fused step ----
    def ion_step(self):
        self._check(self.lib.swap_ion_step(self.ctx))

    def run(self, nsteps: int):
        self._check(self.lib.swap_run(self.ctx, int(nsteps)))

    def energy(self):
        out = np.zeros(4)
        self._check(self.lib.swap_energy(self.ctx, abi.dptr(out)))
        return out

    def max_abs_divB(self, b):
        out = C.c_double()
        self._check(self.lib.swap_max_abs_divB(self.ctx, abi.rptr(b), C.byref(out)))
        return out.value

    def check_finite(self):
        self._check(self.lib.swap_check_finite(self.ctx))

    # ---- diagnostic output and checkpoints ----
    def diag_open(self, out_dir: str, nt: int, nout: int, real_bytes: int = 4, rank: int = 0, **scalars):
        """Open the reference's output files in out_dir (para.dat written now)."""
        spec = abi.DiagSpec(nt, nout, real_bytes, rank)
        spec.dtsub_init = self.cfg.dt / self.cfg.ntsub
        spec.mion = 1.0
        for k, v in scalars.items():
            setattr(spec, k, v)
        d = out_dir if out_dir.endswith("/") else out_dir + "/"
        self._check(self.lib.swap_diag_open(self.ctx, d.encode(), C.byref(spec)))

    def diag_step(self, m: int):
        self._check(self.lib.swap_diag_step(self.ctx, int(m)))

    def diag_close(self):
        self._check(self.lib.swap_diag_close(self.ctx))

    def checkpoint_write(self, path: str):
        self._check(self.lib.swap_checkpoint_write(self.ctx, str(path).encode()))

    def checkpoint_read(self, path: str):
        self._check(self.lib.swap_checkpoint_read(self.ctx, str(path).encode()))

    # ---- the FP32 form ----
    def f32_begin(self):
        """Convert the bound FP64 state into the FP32 form (particles sorted by cell)."""
        self._check(self.lib.swap_f32_begin(self.ctx))

    def f32_run(self, nsteps: int):
        self._check(self.lib.swap_f32_run(self.ctx, int(nsteps)))

    def f32_end(self):
        """Write the FP32 state back into the bound arrays; then sync_to_host.

        The particle arrays go straight into host memory when the device addresses
        it (host-direct mode); the fields go to the device copies."""
        self._check(self.lib.swap_f32_end(self.ctx))

    def f32_count(self) -> int:
        """Ions in the FP32 form's state (the count changes with sources and sinks)."""
        n = C.c_int64()
        self._check(self.lib.swap_f32_count(self.ctx, C.byref(n)))
        return n.value

    def f32_key_starts(self) -> np.ndarray:
        """starts[0..nkeys] of the FP32 state's sort keys (brick * 64 + cell in the brick)."""
        nk = int(np.prod([c // 4 for c in self.cfg.cells])) * 64
        out = np.zeros(nk + 1, dtype=np.int64)
        self._check(self.lib.swap_f32_key_starts(self.ctx, out.ctypes.data_as(abi.c_int64_p), nk + 1))
        return out

    def set_deterministic(self, on: bool = True):
        """FP64 deposits in fixed point: order-independent, bit-reproducible."""
        self._check(self.lib.swap_set_deterministic(self.ctx, 1 if on else 0))

    def f32_far_movers(self) -> int:
        """Ions that moved more than one cell per axis in a step since f32_begin."""
        n = C.c_int64()
        self._check(self.lib.swap_f32_far_movers(self.ctx, C.byref(n)))
        return n.value

    def f32_energy(self):
        out = np.zeros(4)
        self._check(self.lib.swap_f32_energy(self.ctx, abi.dptr(out)))
        return out

    def f32_displace_resort(self, idx, dcell):
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        dcell = np.ascontiguousarray(dcell, dtype=np.int32)
        self._check(self.lib.swap_f32_displace_resort(self.ctx, len(idx), idx.ctypes.data_as(abi.c_int64_p),
                                                      dcell.ctypes.data_as(abi.c_int32_p)))


class Surrogate:
    """The learned field-subcycle surrogate (a handle of the C-ABI)."""

    # inputs per voxel: B (3), u_p (3), n_p, p_e, E0 (3), the plain E at the
    # start of the field step, and B - b12 (3), the change over the last
    # subcycle; the output is the mean corrector E minus E0
    NIN = 14

    def __init__(self, seed: int = 1, max_samples: int = 4096, curl_weight: float = 0.0, per_pair: bool = False):
        self.lib = abi.load()
        n, w = C.c_int32(), C.c_int32()
        abi.check(self.lib, None, self.lib.swap_surrogate_layers(C.byref(n)))
        abi.check(self.lib, None, self.lib.swap_surrogate_width(C.byref(w)))
        # (cin, cout) of the conv layers, padded
        W = w.value
        self.layers = tuple([(16, W)] + [(W, W)] * (n.value - 2) + [(W, 16)])
        h = C.c_void_p()
        abi.check(self.lib, None, self.lib.swap_surrogate_create(C.byref(h), int(seed), int(max_samples)))
        self.h = h
        if curl_weight:
            self.set_curl_weight(curl_weight)
        if per_pair:
            self._check(self.lib.swap_surrogate_set_pair_weighting(self.h, 1))

    def set_weight_grad_cores(self, cuda_cores: bool):
        """Weight gradients on the CUDA cores (True) or the tensor cores (False, the default)."""
        self._check(self.lib.swap_surrogate_set_weight_grad_cores(self.h, 1 if cuda_cores else 0))

    def set_curl_weight(self, w: float, kref2: float = 0.0):
        """Add w * mean |curl e|^2 / kref2 to the loss (e the E error: curl e is
        the B error per unit dt); kref2 = 0: mean |curl target|^2 of the pairs."""
        self._check(self.lib.swap_surrogate_set_curl_weight(self.h, float(w), float(kref2)))

    def _check(self, code):
        if code:
            raise abi.SwapError(code, self.lib.swap_surrogate_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.swap_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def collect(self, hybrid: "Hybrid", nsteps: int):
        """nsteps plain FP32 steps of `hybrid` (after f32_begin), each a training pair."""
        r = self.lib.swap_surrogate_collect(self.h, hybrid.ctx, int(nsteps))
        if r:
            raise abi.SwapError(r, self.lib.swap_last_error(hybrid.ctx).decode())

    def samples(self) -> int:
        n = C.c_int32()
        self._check(self.lib.swap_surrogate_samples(self.h, C.byref(n)))
        return n.value

    def train(self, epochs: int, lr: float = 1e-3) -> float:
        loss = C.c_double()
        self._check(self.lib.swap_surrogate_train(self.h, int(epochs), float(lr), C.byref(loss)))
        return loss.value

    def loss(self) -> float:
        loss = C.c_double()
        self._check(self.lib.swap_surrogate_loss(self.h, C.byref(loss)))
        return loss.value

    def norm(self, mean=None, std=None, out_mean=None, out_std=None):
        """Get (mean, std, out_mean, out_std) or set them: inputs are fed as
        (x - mean)/std, the network predicts (E - E0 - out_mean)/out_std."""
        a = [np.zeros(self.NIN, np.float32), np.ones(self.NIN, np.float32), np.zeros(3, np.float32),
             np.ones(3, np.float32)]
        if mean is None:
            self._check(self.lib.swap_surrogate_norm(self.h, *(x.ctypes.data for x in a), 0))
            return tuple(a)
        for x, v in zip(a, (mean, std, out_mean, out_std)):
            x[:] = v
        self._check(self.lib.swap_surrogate_norm(self.h, *(x.ctypes.data for x in a), 1))
        return None

    def weights(self, layer: int, w=None, b=None):
        cin, cout = self.layers[layer]
        if w is None:
            w = np.zeros((27, cout, cin), dtype=np.float32)
            b = np.zeros(cout, dtype=np.float32)
            self._check(self.lib.swap_surrogate_weights(self.h, layer, w.ctypes.data, b.ctypes.data, 0))
            return w, b
        w = np.ascontiguousarray(w, dtype=np.float32)
        b = np.ascontiguousarray(b, dtype=np.float32)
        self._check(self.lib.swap_surrogate_weights(self.h, layer, w.ctypes.data, b.ctypes.data, 1))
        return None

    def grads(self, dims, vin_dev_ptr: int, tgt_dev_ptr: int):
        """Loss and per-layer (gW, gb) for device inputs [V][NIN] and targets [V][3]."""
        n = sum(27 * ci * co + co for ci, co in self.layers)
        g = np.zeros(n, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.swap_surrogate_grads(self.h, *dims, vin_dev_ptr, tgt_dev_ptr, C.byref(loss), g.ctypes.data))
        out, o = [], 0
        for ci, co in self.layers:
            gw = g[o:o + 27 * ci * co].reshape(27, co, ci)
            o += 27 * ci * co
            out.append((gw, g[o:o + co].copy()))
            o += co
        return loss.value, out


def attach_surrogate(h: "Hybrid", net, judge_every: int = 8, bound: float = 1e-3, bound_db: float = 0.0):
    """Use `net` for the field subcycles of h's FP32 steps (None detaches).

    A judged step falls back when the network's B is more than `bound` from
    the subcycles' relative to B, or, with bound_db > 0, more than bound_db
    relative to the plain B - b0."""
    h._check(h.lib.swap_surrogate_attach(h.ctx, None if net is None else net.h, int(judge_every), float(bound)))
    h._check(h.lib.swap_surrogate_set_db_bound(h.ctx, float(bound_db)))


def surrogate_stats(h: "Hybrid") -> dict:
    out = np.zeros(5)
    h._check(h.lib.swap_surrogate_stats(h.ctx, abi.dptr(out)))
    return {"net_steps": int(out[0]), "judged": int(out[1]), "fallbacks": int(out[2]), "err_b": out[3],
            "err_db": out[4]}
