"""Loader of the sm_103a library (wumingpic2d_gb300/_lib/libwmpic2d.so) through ctypes.

There is no fallback: if the library is missing or cannot be loaded, every
call raises.  Argument types follow include/wumingpic2d.h.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libwmpic2d.so"

STATUS = {
    0: "WM_OK", 1: "WM_ERR_CG_MAXITER", 2: "WM_ERR_OVERFLOW", 3: "WM_ERR_BAD_ARG", 4: "WM_ERR_CELL",
    5: "WM_ERR_CUDA", 6: "WM_ERR_NOT_INIT", 7: "WM_ERR_UNSUPPORTED", 8: "WM_ERR_IO",
}
WM_PREC_FP64, WM_PREC_MIXED = 0, 1


class WmError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}")


class SimConfig(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nsp", ctypes.c_int), ("np", ctypes.c_int),
        ("delx", ctypes.c_double), ("delt", ctypes.c_double), ("c", ctypes.c_double), ("gfac", ctypes.c_double),
        ("q", ctypes.c_double * 4), ("r", ctypes.c_double * 4),
        ("cg_err", ctypes.c_double), ("cg_itemax", ctypes.c_int),
        ("precision", ctypes.c_int), ("capacity", ctypes.c_int64),
        ("bc", ctypes.c_int), ("u0", ctypes.c_double),
    ]


_I, _D, _P = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
# name -> argtypes (all return int unless listed in _RESTYPE)
SIGNATURES = {
    "wm_particle_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _P, _P],
    "wm_particle_solv": [_P, _P, _P, _P, _I, _I],
    "wm_field_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _P, _P, _D],
    "wm_field_fdtd_i": [_P, _P, _P, _P, _I, _I],
    "wm_sort_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I],
    "wm_sort_bucket": [_P, _P, _P, _P, _I, _I],
    "wm_mom_calc_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _P, _P],
    "wm_mom_calc_accl": [_P, _P, _P, _P, _I, _I],
    "wm_mom_calc_nvt": [_P, _P, _P],
    "wm_bc_periodic_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P, _I, _D, _D, _D],
    "wm_bc_periodic_particle_x": [_P, _P],
    "wm_bc_periodic_particle_y": [_P, _P],
    "wm_bc_periodic_dfield": [_P, _I, _I, _I, _I, _I, _I],
    "wm_bc_periodic_curre": [_P, _I, _I, _I, _I, _I, _I],
    "wm_bc_periodic_phi": [_P, _I, _I, _I, _I, _I],
    "wm_bc_periodic_mom": [_P],
    "wm_bc_reconnection_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P, _I, _D, _D, _D],
    "wm_bc_reconnection_particle_x": [_P, _P, _I, _I],
    "wm_bc_reconnection_particle_y": [_P, _P],
    "wm_bc_reconnection_dfield": [_P, _I, _I, _I, _I, _I, _I],
    "wm_bc_reconnection_curre": [_P, _I, _I, _I, _I, _I, _I],
    "wm_bc_reconnection_phi": [_P, _I, _I, _I, _I, _I],
    "wm_bc_reconnection_mom": [_P],
    "wm_bc_shock_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P, _I, _D, _D, _D],
    "wm_bc_shock_particle_x": [_P, _P, _I, _I],
    "wm_bc_shock_particle_y": [_P, _P],
    "wm_bc_shock_injection": [_P, _P, _I, _I, _D],
    "wm_bc_shock_dfield": [_P, _I, _I, _I, _I, _I, _I],
    "wm_bc_shock_curre": [_P, _I, _I, _I, _I, _I, _I],
    "wm_bc_shock_phi": [_P, _I, _I, _I, _I, _I],
    "wm_bc_shock_mom": [_P],
    "wm_energy_sums": [_P, _P, _P, _P],
    "wm_field_cg_iters": [_P],
    "wm_field_get_work": [_P, _P],
    "wm_field_set_work": [_P],
    "wm_finalize": [],
    "wm_status_string": [_I],
    "wm_build_info": [],
    "wm_sim_create": [ctypes.POINTER(SimConfig), ctypes.POINTER(_P)],
    "wm_sim_destroy": [_P],
    "wm_sim_load": [_P, _P, _P, _P],
    "wm_sim_store": [_P, _P, _P, _P, _P],
    "wm_sim_step": [_P, _I],
    "wm_sim_step_host": [_P, _P, _P, _P, _P, _I],
    "wm_sim_energy": [_P, _P],
    "wm_sim_moments": [_P, _P],
    "wm_sim_cg_iters": [_P, _P],
    "wm_sim_kernel_times": [_P, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_D), ctypes.POINTER(_I)],
    "wm_sim_set_timing": [_P, _I],
    "wm_sim_launches": [_P, ctypes.POINTER(ctypes.c_int64)],
    "wm_sim_info": [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
    "wm_sim_sync": [_P],
    "wm_sim_set_rebin": [_P, _I],
    "wm_sim_get_work": [_P, _P, _P],
    "wm_sim_set_work": [_P, _P],
    "wm_sim_step_timed": [_P, _I, ctypes.POINTER(_D)],
    "wm_sim_set_guess": [_P, _P, ctypes.c_longlong],
    "wm_sim_guess_stats": [_P, _P],
    "wm_set_device": [_I],
    "wm_deposit_current_noalloc": [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _P, _P],
    "wm_fp64_fma_rate": [ctypes.POINTER(_D), ctypes.POINTER(_D)],
    "wm_host_register": [_P, ctypes.c_size_t],
    "wm_host_unregister": [_P],
    "wm_host_alloc": [_P, ctypes.c_size_t],
    "wm_host_free": [_P],
    "wm_sim_write_snapshot": [_P, ctypes.c_char_p, ctypes.c_char_p, _I],
    "wm_sim_read_snapshot": [_P, ctypes.c_char_p, ctypes.c_char_p, _P],
    "wm_sim_write_moments": [_P, ctypes.c_char_p, _I],
    "wm_sim_init_weibel": [_P, _I, _D, _D, _D, ctypes.c_uint64],
    "wm_sim_init_harris": [_P, _I, _I, _D, _D, _D, _D, _D, _D, ctypes.c_uint64],
    "wm_sim_init_shock": [_P, _I, _D, _D, _D, _D, _D, _D, _D, _D, _D, ctypes.c_uint64],
    "wm_sim_set_injection": [_P, _I, _I, _D, _D, _D, _D, _D, _D, ctypes.c_uint64],
    "wm_sim_set_expansion": [_P, _I, _I],
    "wm_sim_get_nxe": [_P, _P],
    "wm_sim_set_step": [_P, ctypes.c_int64],
    "wm_sim_get_step": [_P, _P],
    "wm_sim_write_particles": [_P, ctypes.c_char_p, _I, _I],
    "wm_paraio_init": [_I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _P, _P, ctypes.c_char_p],
    "wm_paraio_finalize": [],
    "wm_paraio_output": [_P, _P, _P, _I, _I, _I, ctypes.c_char_p],
    "wm_paraio_input": [_P, _P, _P, _P, _P, _P, ctypes.c_char_p],
    "wm_paraio_param": [_I, _D, _D, _D, _D, _D, _D, ctypes.c_char_p],
    "wm_paraio_mom": [_P, _P, _I],
    "wm_paraio_ptcl": [_P, _P, _P, _I],
    "wm_paraio_orb": [_P, _P, _P, _I],
    "wm_cnn_conv3x3": [_P, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _P, _P],
    "wm_cnn_status": [_I],
    "wm_cnn_conv3x3_wgrad": [_P, _P, _I, _I, _I, _I, _I, _I, _I, _P, _P, _P, ctypes.c_int64, _P],
    "wm_cnn_mse": [_P, _P, ctypes.c_int64, _P, _P, _I, _P, _P],
    "wm_cnn_mse_interior": [_P, _P, _I, _I, _I, _I, _P, _P, _I, _P, _P],
    "wm_cnn_adam": [_P, _P, _P, _P, _P, ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _I, _P],
    "wm_cnn_prep_weights": [_P, _I, _I, _I, _P, _P, _P],
}
_RESTYPE = {"wm_status_string": ctypes.c_char_p, "wm_build_info": ctypes.c_char_p}

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded library; raises if it was not built (run __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"CUDA library not built: {LIB_PATH} is missing (run __graft_entry__.build())")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != 0:
        raise WmError(status, where)
