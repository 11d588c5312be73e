"""The reference's common/ module procedures, on the GPU.

Same names and argument lists as the Fortran module procedures used through
common/wuming2d.f90; arrays are numpy arrays in the reference layout (see
layout.py).  Each call runs the sm_103a kernels of libwmpic2d.so; errors where
the reference calls `stop` raise WmError.

    particle__init / particle__solv         common/particle.f90:18-177
    field__init / field__fdtd_i             common/field.f90:22-186
    sort__init / sort__bucket               common/sort.f90:16-82
    mom_calc__init / __accl / __nvt         common/mom_calc.f90:18-249
    boundary_periodic__init / __particle_x / __particle_y / __dfield /
        __curre / __phi / __mom             common/boundary_periodic.f90:26-636
    boundary_reconnection__*                proj/reconnection/boundary_reconnection.f90:26-647
    boundary_shock__* (with __injection)    proj/shock/boundary_shock.f90:27-693
    paraio__init / __output / __input / __param / __mom / __ptcl / __orb
                                            common/paraio.f90:37-849 (host file I/O)

field__fdtd_i takes the three boundary procedures as arguments in the
reference; here the boundary module whose *__init ran last supplies them (pass
them for symmetry, they are checked to belong to one module).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._native import check, lib

_MPI_DUMMY = 0


def _p(a: np.ndarray):
    return a.ctypes.data


def _f64(a, name):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not (a.flags.f_contiguous or a.ndim == 1):
        raise TypeError(f"{name} must be a Fortran-ordered float64 array")
    return a


def _i32(a, name):
    if not isinstance(a, np.ndarray) or a.dtype != np.int32 or not (a.flags.f_contiguous or a.ndim == 1):
        raise TypeError(f"{name} must be a Fortran-ordered int32 array")
    return a


def _qr(a, nsp):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if a.size != nsp:
        raise ValueError("q and r need one value per species")
    return a


# ---------------------------------------------------------------- particle.f90
def particle__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c, q, r):
    q = _qr(q, nsp)
    r = _qr(r, nsp)
    check(lib().wm_particle_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c, _p(q), _p(r)),
          "particle__init")


def particle__solv(gp, up, uf, cumcnt, nxs, nxe):
    check(lib().wm_particle_solv(_p(_f64(gp, "gp")), _p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(cumcnt, "cumcnt")),
                                 nxs, nxe), "particle__solv")


# ------------------------------------------------------------------- field.f90
def field__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, mnpr, ncomw, opsum, nerr, delx, delt, c, q, r, gfac):
    q = _qr(q, nsp)
    r = _qr(r, nsp)
    check(lib().wm_field_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, mnpr, ncomw, opsum, nerr, delx, delt, c,
                              _p(q), _p(r), gfac), "field__init")


def field__fdtd_i(uf, up, gp, cumcnt, nxs, nxe, set_boundary_dfield=None, set_boundary_curre=None,
                  set_boundary_phi=None):
    kinds = {"periodic": (boundary_periodic__dfield, boundary_periodic__curre, boundary_periodic__phi),
             "reconnection": (boundary_reconnection__dfield, boundary_reconnection__curre, boundary_reconnection__phi),
             "shock": (boundary_shock__dfield, boundary_shock__curre, boundary_shock__phi)}
    given = (set_boundary_dfield, set_boundary_curre, set_boundary_phi)
    if any(f is not None for f in given) and not any(all(f is None or f is w for f, w in zip(given, want))
                                                   for want in kinds.values()):
        raise NotImplementedError("the boundary procedures must be those of one boundary module")
    check(lib().wm_field_fdtd_i(_p(_f64(uf, "uf")), _p(_f64(up, "up")), _p(_f64(gp, "gp")), _p(_i32(cumcnt, "cumcnt")),
                                nxs, nxe), "field__fdtd_i")


def field__cg_iters() -> np.ndarray:
    out = np.zeros(3, dtype=np.int32)
    check(lib().wm_field_cg_iters(_p(out)), "field cg iters")
    return out


def field__get_work(df=None, uj=None):
    check(lib().wm_field_get_work(_p(df) if df is not None else None, _p(uj) if uj is not None else None),
          "field work")


def field__set_work(df):
    check(lib().wm_field_set_work(_p(_f64(df, "df"))), "field work")


# -------------------------------------------------------------------- sort.f90
def sort__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye):
    check(lib().wm_sort_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye), "sort__init")


def sort__bucket(gp, up, cumcnt, np2, nxs, nxe):
    check(lib().wm_sort_bucket(_p(_f64(gp, "gp")), _p(_f64(up, "up")), _p(_i32(cumcnt, "cumcnt")), _p(_i32(np2, "np2")),
                               nxs, nxe), "sort__bucket")


# ---------------------------------------------------------------- mom_calc.f90
def mom_calc__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c, q, r):
    q = _qr(q, nsp)
    r = _qr(r, nsp)
    check(lib().wm_mom_calc_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c, _p(q), _p(r)),
          "mom_calc__init")


def mom_calc__accl(gp, up, uf, cumcnt, nxs, nxe):
    check(lib().wm_mom_calc_accl(_p(_f64(gp, "gp")), _p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(cumcnt, "cumcnt")),
                                 nxs, nxe), "mom_calc__accl")


def mom_calc__nvt(mom, up, np2):
    check(lib().wm_mom_calc_nvt(_p(_f64(mom, "mom")), _p(_f64(up, "up")), _p(_i32(np2, "np2"))), "mom_calc__nvt")


# ------------------------------------------------------- boundary_periodic.f90
def boundary_periodic__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nup, ndown, mnpi, mnpr, ncomw, nerr,
                            nstat, delx, delt, c):
    st = np.ascontiguousarray(np.asarray(nstat if nstat is not None else [0], dtype=np.int32))
    check(lib().wm_bc_periodic_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nup, ndown, mnpi, mnpr, ncomw, nerr,
                                    _p(st), st.size, delx, delt, c), "boundary_periodic__init")


def boundary_periodic__particle_x(up, np2):
    check(lib().wm_bc_periodic_particle_x(_p(_f64(up, "up")), _p(_i32(np2, "np2"))), "boundary_periodic__particle_x")


def boundary_periodic__particle_y(up, np2):
    check(lib().wm_bc_periodic_particle_y(_p(_f64(up, "up")), _p(_i32(np2, "np2"))), "boundary_periodic__particle_y")


def boundary_periodic__dfield(df, nxs, nxe, nys, nye, nxgs, nxge):
    check(lib().wm_bc_periodic_dfield(_p(_f64(df, "df")), nxs, nxe, nys, nye, nxgs, nxge), "boundary_periodic__dfield")


def boundary_periodic__curre(uj, nxs, nxe, nys, nye, nxgs, nxge):
    check(lib().wm_bc_periodic_curre(_p(_f64(uj, "uj")), nxs, nxe, nys, nye, nxgs, nxge), "boundary_periodic__curre")


def boundary_periodic__phi(phi, nxs, nxe, nys, nye, l):
    check(lib().wm_bc_periodic_phi(_p(_f64(phi, "phi")), nxs, nxe, nys, nye, l), "boundary_periodic__phi")


def boundary_periodic__mom(mom):
    check(lib().wm_bc_periodic_mom(_p(_f64(mom, "mom"))), "boundary_periodic__mom")


# ---------------------------------------- proj/reconnection/boundary_reconnection.f90
def boundary_reconnection__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nup, ndown, mnpi, mnpr, ncomw, nerr,
                                nstat, delx, delt, c):
    st = np.ascontiguousarray(np.asarray(nstat if nstat is not None else [0], dtype=np.int32))
    check(lib().wm_bc_reconnection_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nup, ndown, mnpi, mnpr, ncomw, nerr,
                                        _p(st), st.size, delx, delt, c), "boundary_reconnection__init")


def boundary_reconnection__particle_x(up, np2, nxs, nxe):
    check(lib().wm_bc_reconnection_particle_x(_p(_f64(up, "up")), _p(_i32(np2, "np2")), nxs, nxe),
          "boundary_reconnection__particle_x")


def boundary_reconnection__particle_y(up, np2):
    check(lib().wm_bc_reconnection_particle_y(_p(_f64(up, "up")), _p(_i32(np2, "np2"))), "boundary_reconnection__particle_y")


def boundary_reconnection__dfield(df, nxs, nxe, nys, nye, nxgs, nxge):
    check(lib().wm_bc_reconnection_dfield(_p(_f64(df, "df")), nxs, nxe, nys, nye, nxgs, nxge), "boundary_reconnection__dfield")


def boundary_reconnection__curre(uj, nxs, nxe, nys, nye, nxgs, nxge):
    check(lib().wm_bc_reconnection_curre(_p(_f64(uj, "uj")), nxs, nxe, nys, nye, nxgs, nxge), "boundary_reconnection__curre")


def boundary_reconnection__phi(phi, nxs, nxe, nys, nye, l):
    check(lib().wm_bc_reconnection_phi(_p(_f64(phi, "phi")), nxs, nxe, nys, nye, l), "boundary_reconnection__phi")


def boundary_reconnection__mom(mom):
    check(lib().wm_bc_reconnection_mom(_p(_f64(mom, "mom"))), "boundary_reconnection__mom")


# ------------------------------------------------------ proj/shock/boundary_shock.f90
def boundary_shock__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nup, ndown, mnpi, mnpr, ncomw, nerr, nstat, delx, delt,
                         c):
    st = np.ascontiguousarray(np.asarray(nstat if nstat is not None else [0], dtype=np.int32))
    check(lib().wm_bc_shock_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nup, ndown, mnpi, mnpr, ncomw, nerr, _p(st),
                                 st.size, delx, delt, c), "boundary_shock__init")


def boundary_shock__particle_x(up, np2, nxs, nxe):
    check(lib().wm_bc_shock_particle_x(_p(_f64(up, "up")), _p(_i32(np2, "np2")), nxs, nxe), "boundary_shock__particle_x")


def boundary_shock__particle_y(up, np2):
    check(lib().wm_bc_shock_particle_y(_p(_f64(up, "up")), _p(_i32(np2, "np2"))), "boundary_shock__particle_y")


def boundary_shock__injection(up, np2, nxs, nxe, u0):
    check(lib().wm_bc_shock_injection(_p(_f64(up, "up")), _p(_i32(np2, "np2")), nxs, nxe, u0), "boundary_shock__injection")


def boundary_shock__dfield(df, nxs, nxe, nys, nye, nxgs, nxge):
    check(lib().wm_bc_shock_dfield(_p(_f64(df, "df")), nxs, nxe, nys, nye, nxgs, nxge), "boundary_shock__dfield")


def boundary_shock__curre(uj, nxs, nxe, nys, nye, nxgs, nxge):
    check(lib().wm_bc_shock_curre(_p(_f64(uj, "uj")), nxs, nxe, nys, nye, nxgs, nxge), "boundary_shock__curre")


def boundary_shock__phi(phi, nxs, nxe, nys, nye, l):
    check(lib().wm_bc_shock_phi(_p(_f64(phi, "phi")), nxs, nxe, nys, nye, l), "boundary_shock__phi")


def boundary_shock__mom(mom):
    check(lib().wm_bc_shock_mom(_p(_f64(mom, "mom"))), "boundary_shock__mom")


# ---------------------------------------------------------------- paraio.f90
def _name(s: str) -> bytes:
    return s.encode()


def paraio__init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nproc, nrank, delx, delt, c, q, r, dir):
    """dir is a prefix joined to the file names, as in the Fortran (end it with '/')."""
    q = _qr(q, nsp)
    r = _qr(r, nsp)
    check(lib().wm_paraio_init(ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, nproc, nrank, delx, delt, c, _p(q), _p(r),
                               _name(dir)), "paraio__init")


def paraio__finalize():
    check(lib().wm_paraio_finalize(), "paraio__finalize")


def paraio__output(up, uf, np2, nxs, nxe, it, filename):
    check(lib().wm_paraio_output(_p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(np2, "np2")), nxs, nxe, it, _name(filename)),
          "paraio__output")


def paraio__input(up, uf, np2, filename):
    """Fills up, uf, np2 in place; returns (nxs, nxe, it), the Fortran's intent(out) scalars."""
    v = (ctypes.c_int * 3)()
    check(lib().wm_paraio_input(_p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(np2, "np2")), ctypes.byref(v, 0),
                                ctypes.byref(v, 4), ctypes.byref(v, 8), _name(filename)), "paraio__input")
    return v[0], v[1], v[2]


def paraio__param(n0, wpe, wpi, wge, wgi, vti, vte, filename):
    check(lib().wm_paraio_param(n0, wpe, wpi, wge, wgi, vti, vte, _name(filename)), "paraio__param")


def paraio__mom(mom, uf, it):
    check(lib().wm_paraio_mom(_p(_f64(mom, "mom")), _p(_f64(uf, "uf")), it), "paraio__mom")


def paraio__ptcl(up, uf, np2, it):
    check(lib().wm_paraio_ptcl(_p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(np2, "np2")), it), "paraio__ptcl")


def paraio__orb(up, uf, np2, it):
    check(lib().wm_paraio_orb(_p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(np2, "np2")), it), "paraio__orb")


# ------------------------------------------------------------- diagnostics
def energy_sums(up, uf, np2, nsp) -> np.ndarray:
    """energy_history's sums (proj/weibel/app.f90:507-534): [KE_1..KE_nsp, E^2/8pi, B^2/8pi]."""
    out = np.zeros(nsp + 2)
    check(lib().wm_energy_sums(_p(_f64(up, "up")), _p(_f64(uf, "uf")), _p(_i32(np2, "np2")), _p(out)), "energy_sums")
    return out


def finalize():
    check(lib().wm_finalize(), "finalize")


def build_info() -> str:
    return lib().wm_build_info().decode()


def init_all(dims, delt, q, r, c=1.0, delx=1.0, gfac=0.501, bc="periodic"):
    """Call every module's *__init the way proj/weibel/app.f90:331-347 does (single rank); bc
    names the boundary module ("periodic", "reconnection" or "shock")."""
    d = dims
    args = (d.ndim, d.np, d.nsp, d.nxgs, d.nxge, d.nygs, d.nyge, d.nys, d.nye)
    init_bc = {"periodic": boundary_periodic__init, "reconnection": boundary_reconnection__init,
               "shock": boundary_shock__init}[bc]
    init_bc(*args, 0, 0, _MPI_DUMMY, _MPI_DUMMY, _MPI_DUMMY, 0, None, delx, delt, c)
    particle__init(*args, delx, delt, c, q, r)
    field__init(*args, _MPI_DUMMY, _MPI_DUMMY, _MPI_DUMMY, 0, delx, delt, c, q, r, gfac)
    sort__init(*args)
    mom_calc__init(*args, delx, delt, c, q, r)
