"""ctypes binding of the C-ABI library (include/swap_gpu.h).

There is no CPU fallback: if the sm_103a library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)

SWAP_ERRORS = {
    0: "SWAP_OK",
    1: "SWAP_EINVAL",
    2: "SWAP_ECUDA",
    3: "SWAP_EDOMAIN",
    4: "SWAP_ECAPACITY",
    5: "SWAP_ENONFINITE",
    6: "SWAP_ESUBCYCLE",
    7: "SWAP_EMOVE",
    8: "SWAP_EWAIT",
    9: "SWAP_EEXCHANGE",
}


class SwapError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{SWAP_ERRORS.get(code, code)}: {msg}")
        self.code = code


class Dims(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("real_bytes", C.c_int32),
                ("ni_max", C.c_int64)]


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("alpha", C.c_double),
        ("beta", C.c_double),
        ("dx", C.c_double),
        ("dy", C.c_double),
        ("grad_pe", C.c_double),
        ("ntsub", C.c_int32),
        ("flags", C.c_int32),
    ]


class Coords(C.Structure):
    _fields_ = [(n, c_double_p) for n in (
        "qx", "qy", "qz", "dx_grid", "dy_grid", "dz_grid", "dx_cell", "dy_cell", "dz_cell", "xrat", "yrat", "zrat")]


class LoadSpec(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("stream", C.c_uint32),
        ("ppc", C.c_int32),
        ("vth", C.c_double),
        ("ux", C.c_double),
        ("uy", C.c_double),
        ("uz", C.c_double),
        ("mrat", C.c_double),
        ("beta_p", C.c_double),
    ]


class Sources(C.Structure):
    """swap_sources: particle sources and sinks of the ion step."""

    _fields_ = [
        ("seed", C.c_uint64),
        ("ndot", C.c_double), ("vsw", C.c_double), ("beta_pu", C.c_double), ("mrat_pu", C.c_double),
        ("delz_ref", C.c_double),
        ("x_open", C.c_int32), ("inflow_ppc", C.c_int32),
        ("inflow_vth", C.c_double), ("inflow_ux", C.c_double), ("inflow_uy", C.c_double), ("inflow_uz", C.c_double),
        ("cloud_N0", C.c_double), ("cloud_r0", C.c_double), ("cloud_x", C.c_double), ("cloud_y", C.c_double),
        ("cloud_z", C.c_double), ("nu_ion", C.c_double), ("mrat_heavy", C.c_double), ("beta_heavy", C.c_double),
        ("cx_a", C.c_double), ("cx_b", C.c_double),
    ]


class DiagSpec(C.Structure):
    """swap_diag_spec: diagnostic output settings and para.dat scalars."""

    _fields_ = [("nt", C.c_int32), ("nout", C.c_int32), ("real_bytes", C.c_int32), ("rank", C.c_int32)] + [
        (n, C.c_double) for n in ("dtsub_init", "vtop", "vbottom", "mion", "m_pu", "m_heavy", "np_top",
                                  "np_bottom", "b0_top", "b0_bottom", "vth_top", "vth_bottom")]


def make_sources(**kw) -> Sources:
    """A Sources with every rule off (all zero) except the fields given."""
    s = Sources()
    for k, v in kw.items():
        setattr(s, k, v)
    return s


# Every exported symbol declared in include/swap_gpu.h, with its argument types.
P = C.c_void_p
# swap_exchange_fn: int fn(void* user, void* data, int64 count, int32 kind, void* stream)
EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p)
SIGNATURES: dict[str, tuple] = {
    "swap_init": (C.c_int, [C.POINTER(P), C.POINTER(Dims), C.POINTER(Params), C.POINTER(Coords)]),
    "swap_finalize": (C.c_int, [P]),
    "swap_last_error": (C.c_char_p, [P]),
    "swap_abi_version": (C.c_int, []),
    "swap_bind_particles": (C.c_int, [P] + [c_double_p] * 5 + [c_int32_p, c_int32_p]),
    "swap_bind_fields": (C.c_int, [P] + [c_double_p] * 11),
    "swap_bind_array": (C.c_int, [P, P, C.c_int64]),
    "swap_sync_to_device": (C.c_int, [P, P]),
    "swap_sync_to_host": (C.c_int, [P, P]),
    "swap_mark_host_dirty": (C.c_int, [P, P]),
    "swap_set_host_direct": (C.c_int, [P, C.c_int]),
    "swap_transfer_bytes": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int]),
    "swap_set_exchange": (C.c_int, [P, EXCHANGE_FN, P]),
    "swap_set_wait_limit": (C.c_int, [P, C.c_uint32]),
    "swap_get_interp_weights": (C.c_int, [P, c_double_p]),
    "swap_update_np": (C.c_int, [P, c_double_p]),
    "swap_update_up": (C.c_int, [P] + [c_double_p] * 3),
    "swap_extrapol_up": (C.c_int, [P] + [c_double_p] * 4),
    "swap_get_Ep": (C.c_int, [P] + [c_double_p] * 6),
    "swap_get_vplus_vminus": (C.c_int, [P] + [c_double_p] * 5),
    "swap_improve_up": (C.c_int, [P] + [c_double_p] * 5),
    "swap_get_vp_final": (C.c_int, [P] + [c_double_p] * 4),
    "swap_move_ion_half": (C.c_int, [P] + [c_double_p] * 4),
    "swap_curlB": (C.c_int, [P] + [c_double_p] * 3),
    "swap_edge_to_center": (C.c_int, [P] + [c_double_p] * 2),
    "swap_face_to_center": (C.c_int, [P] + [c_double_p] * 2),
    "swap_get_E": (C.c_int, [P] + [c_double_p] * 7),
    "swap_predict_B": (C.c_int, [P] + [c_double_p] * 10 + [C.c_double]),
    "swap_correct_B": (C.c_int, [P] + [c_double_p] * 8 + [C.c_double]),
    "swap_f_update_tlev": (C.c_int, [P] + [c_double_p] * 5),
    "swap_check_time_step": (C.c_int, [P] + [c_double_p] * 4),
    "swap_periodic": (C.c_int, [P, c_double_p]),
    "swap_periodic_scalar": (C.c_int, [P, c_double_p]),
    "swap_update_rho": (C.c_int, [P, c_double_p]),
    "swap_get_temperature": (C.c_int, [P] + [c_double_p] * 4),
    "swap_set_mion": (C.c_int, [P, C.c_double]),
    "swap_ion_step_pre": (C.c_int, [P]),
    "swap_field_subcycles": (C.c_int, [P]),
    "swap_ion_step_post": (C.c_int, [P]),
    "swap_ion_step": (C.c_int, [P]),
    "swap_run": (C.c_int, [P, C.c_int32]),
    "swap_set_sources": (C.c_int, [P, C.POINTER(Sources), C.c_int64]),
    "swap_chex_count": (C.c_int, [P, c_int64_p]),
    "swap_Ionize_sw_mp": (C.c_int, [P] + [c_double_p] * 4 + [C.c_int32] + [c_double_p] * 2),
    "swap_remove_ion": (C.c_int, [P] + [c_double_p] * 3 + [C.c_int32]),
    "swap_res_chex": (C.c_int, [P, c_double_p, c_double_p, C.c_int32, c_int64_p]),
    "swap_inflow_x": (C.c_int, [P, C.c_int32]),
    "swap_ionize_cloud": (C.c_int, [P, C.c_int32]),
    "swap_remove_outflow_x": (C.c_int, [P]),
    "swap_diag_open": (C.c_int, [P, C.c_char_p, C.POINTER(DiagSpec)]),
    "swap_diag_step": (C.c_int, [P, C.c_int32]),
    "swap_diag_close": (C.c_int, [P]),
    "swap_checkpoint_write": (C.c_int, [P, C.c_char_p]),
    "swap_checkpoint_read": (C.c_int, [P, C.c_char_p]),
    "swap_f32_begin": (C.c_int, [P]),
    "swap_f32_run": (C.c_int, [P, C.c_int32]),
    "swap_f32_end": (C.c_int, [P]),
    "swap_f32_energy": (C.c_int, [P, c_double_p]),
    "swap_f32_count": (C.c_int, [P, c_int64_p]),
    "swap_f32_far_movers": (C.c_int, [P, c_int64_p]),
    "swap_set_deterministic": (C.c_int, [P, C.c_int32]),
    "swap_surrogate_layers": (C.c_int, [c_int32_p]),
    "swap_surrogate_width": (C.c_int, [c_int32_p]),
    "swap_surrogate_set_curl_weight": (C.c_int, [P, C.c_double, C.c_double]),
    "swap_surrogate_set_pair_weighting": (C.c_int, [P, C.c_int32]),
    "swap_surrogate_set_weight_grad_cores": (C.c_int, [P, C.c_int32]),
    "swap_f32_key_starts": (C.c_int, [P, c_int64_p, C.c_int64]),
    "swap_f32_set_moment_sums": (C.c_int, [P, C.c_int]),
    "swap_f32_displace_resort": (C.c_int, [P, C.c_int64, c_int64_p, c_int32_p]),
    "swap_energy": (C.c_int, [P, c_double_p]),
    "swap_max_abs_divB": (C.c_int, [P, c_double_p, c_double_p]),
    "swap_check_finite": (C.c_int, [P]),
    "swap_load_maxwellian_host": (C.c_int, [C.POINTER(Dims), C.POINTER(Coords), C.POINTER(LoadSpec)]
                                  + [c_double_p] * 5 + [C.c_int64, c_int64_p]),
    "swap_update_up_noalloc": (C.c_int, [C.POINTER(Dims), C.POINTER(Params), C.POINTER(Coords)]
                               + [P] * 3 + [C.c_int64, P, P, P]),
    "swap_tc_gemm_check": (C.c_int, [P, P, P, C.c_int32]),
    "swap_conv3_check": (C.c_int, [C.c_int32] * 5 + [P, P, P, P, P, C.c_int32]),
    "swap_surrogate_create": (C.c_int, [C.POINTER(P), C.c_uint64, C.c_int32]),
    "swap_surrogate_destroy": (C.c_int, [P]),
    "swap_surrogate_last_error": (C.c_char_p, [P]),
    "swap_surrogate_collect": (C.c_int, [P, P, C.c_int32]),
    "swap_surrogate_samples": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "swap_surrogate_train": (C.c_int, [P, C.c_int32, C.c_double, c_double_p]),
    "swap_surrogate_loss": (C.c_int, [P, c_double_p]),
    "swap_surrogate_attach": (C.c_int, [P, P, C.c_int32, C.c_double]),
    "swap_surrogate_set_db_bound": (C.c_int, [P, C.c_double]),
    "swap_surrogate_stats": (C.c_int, [P, c_double_p]),
    "swap_surrogate_norm": (C.c_int, [P, P, P, P, P, C.c_int32]),
    "swap_surrogate_weights": (C.c_int, [P, C.c_int32, P, P, C.c_int32]),
    "swap_surrogate_grads": (C.c_int, [P] + [C.c_int32] * 3 + [P, P, c_double_p, P]),
    "swap_timer_start": (C.c_int, [P]),
    "swap_timer_stop": (C.c_int, [P, c_double_p]),
    "swap_profile_enable": (C.c_int, [P, C.c_int]),
    "swap_profile_read": (C.c_int, [P, C.c_int32, C.POINTER(C.c_char_p), c_double_p, c_int64_p, c_int32_p]),
    "swap_profile_reset": (C.c_int, [P]),
}

_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libswap_gpu.so (building it in-tree if absent).  Raises if it can't."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run swap_gb300.build.build()")
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1), "need a float64 Fortran-ordered array"
    return a.ctypes.data_as(c_double_p)


def rptr(a: np.ndarray):
    """A bound real array as the ABI's double*: float64, or float32 for a
    context created with real_bytes = 4 (the reference's -real-size 32)."""
    assert a.dtype in (np.float64, np.float32) and (a.flags.f_contiguous or a.ndim == 1), \
        "need a float64/float32 Fortran-ordered array"
    return a.ctypes.data_as(c_double_p)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32
    return a.ctypes.data_as(c_int32_p)


def check(lib, ctx, code: int) -> None:
    if code != 0:
        msg = lib.swap_last_error(ctx) if ctx else b""
        raise SwapError(code, (msg or b"").decode())
