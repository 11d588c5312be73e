"""ctypes front end of the C restatement in wm_oracle.c.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
the cpu_baseline / reference legs of bench.py, as the checker.  The product
(wumingpic2d_gb300) never imports it.

Every function takes the reference-layout numpy arrays described in
wumingpic2d_gb300/layout.py and mirrors one reference routine; the C file
cites the Fortran lines.  The library is compiled by ``build()`` (called from
__graft_entry__.build()) into oracle/_build/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "liboracle.so"
SRC = HERE / "wm_oracle.c"

OK, ERR_CG_MAXITER, ERR_OVERFLOW, ERR_BAD_ARG, ERR_CELL = 0, 1, 2, 3, 4


def build(force: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB_PATH.with_suffix(f".so.tmp{os.getpid()}")
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-frounding-math", "-fopenmp", "-fPIC", "-shared",
               "-o", str(tmp), str(SRC), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Par(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int), ("np", ctypes.c_int), ("nsp", ctypes.c_int),
        ("nxgs", ctypes.c_int), ("nxge", ctypes.c_int), ("nygs", ctypes.c_int), ("nyge", ctypes.c_int),
        ("nys", ctypes.c_int), ("nye", ctypes.c_int),
        ("delx", ctypes.c_double), ("delt", ctypes.c_double), ("c", ctypes.c_double), ("gfac", ctypes.c_double),
        ("q", ctypes.c_double * 8), ("r", ctypes.c_double * 8),
        ("cg_err", ctypes.c_double), ("cg_itemax", ctypes.c_int),
        ("bc", ctypes.c_int), ("u0", ctypes.c_double),
    ]


BC = {"periodic": 0, "reconnection": 1, "shock": 2}


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.POINTER(Par)
        dp = ctypes.c_void_p
        i = ctypes.c_int
        sig = {
            "wmo_particle_solv": (None, [P, dp, dp, dp, dp, i, i]),
            "wmo_mom_accl": (None, [P, dp, dp, dp, dp, i, i]),
            "wmo_ele_cur": (None, [P, dp, dp, dp, dp, i, i]),
            "wmo_bc_curre": (None, [P, dp, i, i]),
            "wmo_bc_dfield": (None, [P, dp, i, i]),
            "wmo_bc_phi": (None, [P, dp, i, i, i]),
            "wmo_bc_particle_x_walls": (None, [P, dp, dp, i, i]),
            "wmo_bc_injection": (None, [P, dp, dp, i, i, ctypes.c_double]),
            "wmo_cgm": (i, [P, dp, dp, i, i, dp]),
            "wmo_field_fdtd_i": (i, [P, dp, dp, dp, dp, i, i, dp, dp, dp, dp]),
            "wmo_bc_particle_x": (None, [P, dp, dp]),
            "wmo_bc_particle_y": (i, [P, dp, dp]),
            "wmo_sort_bucket": (i, [P, dp, dp, dp, dp, i, i]),
            "wmo_mom_nvt": (None, [P, dp, dp, dp]),
            "wmo_bc_mom": (None, [P, dp]),
            "wmo_energy": (None, [P, dp, dp, dp, dp]),
            "wmo_step": (i, [P, dp, dp, dp, dp, dp, i, i, dp, dp, dp, dp]),
            "wmo_num_threads": (i, []),
            "wmo_set_num_threads": (None, [i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags.f_contiguous or a.ndim <= 1
    return a.ctypes.data


def make_par(dims, delt, q, r, c=1.0, delx=1.0, gfac=0.501, cg_err=1e-6, cg_itemax=100, bc="periodic", u0=0.0) -> Par:
    p = Par()
    p.ndim, p.np, p.nsp = dims.ndim, dims.np, dims.nsp
    p.nxgs, p.nxge, p.nygs, p.nyge = dims.nxgs, dims.nxge, dims.nygs, dims.nyge
    p.nys, p.nye = dims.nys, dims.nye
    p.delx, p.delt, p.c, p.gfac = delx, delt, c, gfac
    for k in range(dims.nsp):
        p.q[k] = float(q[k])
        p.r[k] = float(r[k])
    p.cg_err, p.cg_itemax = cg_err, cg_itemax
    p.bc, p.u0 = BC[bc], u0
    return p


def set_threads(n: int) -> None:
    lib().wmo_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().wmo_num_threads())


class OracleState:
    """The SAVE'd work arrays of field__fdtd_i (field.f90:98) for one simulation."""

    def __init__(self, dims):
        self.df = np.zeros((6, dims.nx + 4, dims.ny + 4), order="F")
        self.gkl = np.zeros((3, dims.nx, dims.ny), order="F")
        self.uj = np.zeros((3, dims.nx + 4, dims.ny + 4), order="F")


def particle_solv(par, dims, gp, up, uf, cumcnt):
    lib().wmo_particle_solv(ctypes.byref(par), _p(gp), _p(up), _p(uf), _p(cumcnt), dims.nxs, dims.nxe)


def mom_accl(par, dims, gp, up, uf, cumcnt):
    lib().wmo_mom_accl(ctypes.byref(par), _p(gp), _p(up), _p(uf), _p(cumcnt), dims.nxs, dims.nxe)


def ele_cur(par, dims, uj, up, gp, cumcnt):
    lib().wmo_ele_cur(ctypes.byref(par), _p(uj), _p(up), _p(gp), _p(cumcnt), dims.nxs, dims.nxe)


def bc_curre(par, dims, uj):
    lib().wmo_bc_curre(ctypes.byref(par), _p(uj), dims.nxs, dims.nxe)


def bc_dfield(par, dims, df):
    lib().wmo_bc_dfield(ctypes.byref(par), _p(df), dims.nxs, dims.nxe)


def bc_phi(par, dims, phi, l=1):
    lib().wmo_bc_phi(ctypes.byref(par), _p(phi), dims.nxs, dims.nxe, l)


def cgm(par, dims, db, gkl):
    iters = np.zeros(3, dtype=np.int32)
    st = lib().wmo_cgm(ctypes.byref(par), _p(db), _p(gkl), dims.nxs, dims.nxe, _p(iters))
    return st, iters


def field_fdtd_i(par, dims, uf, up, gp, cumcnt, state: OracleState):
    iters = np.zeros(3, dtype=np.int32)
    st = lib().wmo_field_fdtd_i(ctypes.byref(par), _p(uf), _p(up), _p(gp), _p(cumcnt), dims.nxs, dims.nxe,
                                _p(state.df), _p(state.gkl), _p(state.uj), _p(iters))
    return st, iters


def bc_particle_x(par, dims, up, np2):
    lib().wmo_bc_particle_x(ctypes.byref(par), _p(up), _p(np2))


def bc_particle_x_walls(par, dims, up, np2):
    lib().wmo_bc_particle_x_walls(ctypes.byref(par), _p(up), _p(np2), dims.nxs, dims.nxe)


def bc_injection(par, dims, up, np2, u0):
    lib().wmo_bc_injection(ctypes.byref(par), _p(up), _p(np2), dims.nxs, dims.nxe, u0)


def bc_particle_y(par, dims, up, np2):
    return lib().wmo_bc_particle_y(ctypes.byref(par), _p(up), _p(np2))


def sort_bucket(par, dims, gp, up, cumcnt, np2):
    return lib().wmo_sort_bucket(ctypes.byref(par), _p(gp), _p(up), _p(cumcnt), _p(np2), dims.nxs, dims.nxe)


def mom_nvt(par, dims, mom, up, np2):
    lib().wmo_mom_nvt(ctypes.byref(par), _p(mom), _p(up), _p(np2))


def bc_mom(par, dims, mom):
    lib().wmo_bc_mom(ctypes.byref(par), _p(mom))


def energy(par, dims, up, uf, np2):
    out = np.zeros(dims.nsp + 2)
    lib().wmo_energy(ctypes.byref(par), _p(out), _p(up), _p(uf), _p(np2))
    return out


def step(par, dims, up, gp, uf, cumcnt, np2, state: OracleState):
    iters = np.zeros(3, dtype=np.int32)
    st = lib().wmo_step(ctypes.byref(par), _p(up), _p(gp), _p(uf), _p(cumcnt), _p(np2), dims.nxs, dims.nxe,
                        _p(state.df), _p(state.gkl), _p(state.uj), _p(iters))
    return st, iters
