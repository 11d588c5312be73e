"""Resident simulation: particles and fields stay on the GPU between steps.

Simulation wraps the wm_sim_* entry points.  A state in the reference layout
(up, uf, np2) is loaded once and cell-sorted on the GPU; step(n) runs the
main-loop body of proj/weibel/app.f90:102-107 n times; store() writes the state
back into reference-layout arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._native import WM_PREC_FP64, WM_PREC_MIXED, SimConfig, check, lib
from .layout import Dims

PRECISIONS = {"fp64": WM_PREC_FP64, "mixed": WM_PREC_MIXED}
BOUNDARIES = {"periodic": 0, "reconnection": 1, "shock": 2}


class Simulation:
    def __init__(self, dims: Dims, delt: float, q, r, c: float = 1.0, delx: float = 1.0, gfac: float = 0.501,
                 cg_err: float = 1e-6, cg_itemax: int = 100, precision: str = "fp64", capacity: int = 0, bc: str = "periodic",
                 u0: float = 0.0):
        """bc: the application's boundary module -- "periodic" (Weibel), "reconnection" (walls in x) or
        "shock" (reflecting wall and injection boundary, upstream four-velocity u0)."""
        if dims.nxgs != 2 or dims.nygs != 2:
            raise ValueError("the resident simulation uses nxgs = nygs = 2 like the reference apps")
        self.dims = dims
        cfg = SimConfig()
        cfg.nx, cfg.ny, cfg.nsp, cfg.np = dims.nx, dims.ny, dims.nsp, dims.np
        cfg.delx, cfg.delt, cfg.c, cfg.gfac = delx, delt, c, gfac
        for k in range(dims.nsp):
            cfg.q[k] = float(q[k])
            cfg.r[k] = float(r[k])
        cfg.cg_err, cfg.cg_itemax = cg_err, cg_itemax
        cfg.precision = PRECISIONS[precision]
        cfg.capacity = capacity
        cfg.bc = BOUNDARIES[bc]
        cfg.u0 = u0
        self._h = ctypes.c_void_p()
        check(lib().wm_sim_create(ctypes.byref(cfg), ctypes.byref(self._h)), "wm_sim_create")

    # ------------------------------------------------------------------ state
    def load(self, up: np.ndarray, uf: np.ndarray, np2: np.ndarray) -> None:
        check(lib().wm_sim_load(self._h, up.ctypes.data, uf.ctypes.data, np2.ctypes.data), "wm_sim_load")

    def store(self, up=None, uf=None, np2=None, cumcnt=None):
        d = self.dims
        up = d.alloc_up() if up is None else up
        uf = d.alloc_uf() if uf is None else uf
        np2 = d.alloc_np2() if np2 is None else np2
        cumcnt = d.alloc_cumcnt() if cumcnt is None else cumcnt
        check(lib().wm_sim_store(self._h, up.ctypes.data, uf.ctypes.data, np2.ctypes.data, cumcnt.ctypes.data),
              "wm_sim_store")
        return up, uf, np2, cumcnt

    def fields(self) -> np.ndarray:
        """The current fields uf in the reference layout (6, nx+4, ny+4)."""
        uf = self.dims.alloc_uf()
        check(lib().wm_sim_store(self._h, None, uf.ctypes.data, None, None), "wm_sim_store")
        return uf

    def set_guess(self, params) -> None:
        """Start each step's CG from the learned network's dB where it beats the previous step's
        (params: the network's flat FP32 parameters), or switch that off (None)."""
        if params is None:
            check(lib().wm_sim_set_guess(self._h, None, 0), "wm_sim_set_guess")
            return
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(lib().wm_sim_set_guess(self._h, p.ctypes.data, p.size), "wm_sim_set_guess")

    def guess_stats(self) -> np.ndarray:
        """Last step: |b - A dB_net|^2 (3), |b - A dB_prev|^2 (3), network guess taken (3), |b|^2 (3)."""
        out = np.zeros(12)
        check(lib().wm_sim_guess_stats(self._h, out.ctypes.data), "wm_sim_guess_stats")
        return out

    def step(self, nsteps: int = 1) -> None:
        check(lib().wm_sim_step(self._h, int(nsteps)), "wm_sim_step")

    def step_host(self, up, uf, np2, cumcnt, nsteps: int = 1) -> None:
        """One call with host buffers: copy in, nsteps steps, copy out (the drop-in path)."""
        check(lib().wm_sim_step_host(self._h, up.ctypes.data, uf.ctypes.data, np2.ctypes.data, cumcnt.ctypes.data,
                                     int(nsteps)), "wm_sim_step_host")

    def step_timed(self, nsteps: int) -> float:
        """Run nsteps steps; return their GPU time in ms (CUDA events on the simulation stream)."""
        ms = ctypes.c_double()
        check(lib().wm_sim_step_timed(self._h, int(nsteps), ctypes.byref(ms)), "wm_sim_step_timed")
        return ms.value

    def sync(self) -> None:
        check(lib().wm_sim_sync(self._h), "wm_sim_sync")

    def set_rebin(self, mode: str) -> None:
        """Mixed path: 'permute' (default; the next push reads through the new order) or 'move'
        (the particles are moved into cell order after every step).  Same results bit for bit."""
        check(lib().wm_sim_set_rebin(self._h, {"permute": 0, "move": 1}[mode]), "wm_sim_set_rebin")

    # ------------------------------------------------------------ diagnostics
    def energy(self) -> np.ndarray:
        out = np.zeros(self.dims.nsp + 2)
        check(lib().wm_sim_energy(self._h, out.ctypes.data), "wm_sim_energy")
        return out

    def moments(self) -> np.ndarray:
        mom = self.dims.alloc_mom()
        check(lib().wm_sim_moments(self._h, mom.ctypes.data), "wm_sim_moments")
        return mom

    # ------------------------------------------------ initial conditions generated on the GPU
    def init_weibel(self, ppc: int, v_drift: float, vth_e: float, vth_i: float, seed: int) -> None:
        """The two-beam Weibel state (ppc per cell and species), generated and sorted on the GPU."""
        check(lib().wm_sim_init_weibel(self._h, int(ppc), float(v_drift), float(vth_e), float(vth_i), int(seed)),
              "wm_sim_init_weibel")

    def init_harris(self, cfg) -> None:
        """The reconnection application's Harris sheet for a harris.HarrisConfig."""
        vte, vti, wpe, wpi, q, b0, lcs = cfg.plasma()
        check(lib().wm_sim_init_harris(self._h, cfg.nbg, cfg.ncs, lcs, b0, cfg.e1, vte, vti, cfg.rtemp, int(cfg.seed)),
              "wm_sim_init_harris")

    def init_shock(self, cfg, inject: bool = True) -> None:
        """The shock application's upstream plasma for a shock.ShockConfig, with the application's
        particle injection at the right boundary switched on (inject=True).  cfg.n_x_ini and
        cfg.intvl_expand set the expanding box (proj/shock/app.f90:277, :123-125): the plasma fills
        nxs+1 .. nxe-1 with nxe = nxgs + n_x_ini, and nxe grows by one cell every intvl_expand steps."""
        n_x_ini = cfg.n_x_ini if cfg.n_x_ini else self.dims.nx - 1
        check(lib().wm_sim_set_expansion(self._h, int(n_x_ini), int(cfg.intvl_expand)), "wm_sim_set_expansion")
        check(lib().wm_sim_init_shock(self._h, *cfg.init_args()), "wm_sim_init_shock")
        self.set_injection(cfg if inject else None)

    @property
    def nxe(self) -> int:
        """The active right end of the box (nxge unless the shock's box is expanding)."""
        v = ctypes.c_int()
        check(lib().wm_sim_get_nxe(self._h, ctypes.byref(v)), "wm_sim_get_nxe")
        return v.value

    def set_injection(self, cfg) -> None:
        """Inject the upstream plasma of a shock.ShockConfig every step (None: off)."""
        if cfg is None:
            check(lib().wm_sim_set_injection(self._h, 0, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0), "wm_sim_set_injection")
            return
        a = cfg.init_args()  # n0, u0, vth_e, vth_i, b0, theta, phi, l_damp, xrs, xre, seed
        check(lib().wm_sim_set_injection(self._h, 1, a[0], a[2], a[3], a[4], a[5], a[6], a[7], a[10]), "wm_sim_set_injection")

    @property
    def step_number(self) -> int:
        v = ctypes.c_int64()
        check(lib().wm_sim_get_step(self._h, ctypes.byref(v)), "wm_sim_get_step")
        return v.value

    @step_number.setter
    def step_number(self, it: int) -> None:
        check(lib().wm_sim_set_step(self._h, int(it)), "wm_sim_set_step")

    # ------------------------------------------------------- files (common/paraio.f90 format)
    @staticmethod
    def _dir(d: str) -> bytes:
        return (d if d.endswith("/") else d + "/").encode()

    def write_snapshot(self, dirname: str, filename: str, it: int) -> None:
        """The restart snapshot of paraio__output: <dirname>/<filename>.json + .raw."""
        check(lib().wm_sim_write_snapshot(self._h, self._dir(dirname), filename.encode(), int(it)), "wm_sim_write_snapshot")

    def read_snapshot(self, dirname: str, filename: str) -> int:
        """Load a paraio__output snapshot (this library's or the reference's); returns its step."""
        it = ctypes.c_int()
        check(lib().wm_sim_read_snapshot(self._h, self._dir(dirname), filename.encode(), ctypes.byref(it)), "wm_sim_read_snapshot")
        return it.value

    def write_moments(self, dirname: str, it: int) -> None:
        """paraio__mom of the current moments and fields: <dirname>/<it:07d>_mom.json + .raw."""
        check(lib().wm_sim_write_moments(self._h, self._dir(dirname), int(it)), "wm_sim_write_moments")

    def write_particles(self, dirname: str, it: int, tracers_only: bool = False) -> None:
        """paraio__ptcl (all active particles) or paraio__orb (ids > 0): <it:07d>_ptcl / _orb."""
        check(lib().wm_sim_write_particles(self._h, self._dir(dirname), int(it), int(bool(tracers_only))),
              "wm_sim_write_particles")

    def cg_iters(self) -> np.ndarray:
        out = np.zeros(3, dtype=np.int32)
        check(lib().wm_sim_cg_iters(self._h, out.ctypes.data), "wm_sim_cg_iters")
        return out

    def get_work(self):
        d = self.dims
        df = d.alloc_uf()
        uj = d.alloc_uj()
        check(lib().wm_sim_get_work(self._h, df.ctypes.data, uj.ctypes.data), "wm_sim_get_work")
        return df, uj

    def set_work(self, df: np.ndarray) -> None:
        check(lib().wm_sim_set_work(self._h, df.ctypes.data), "wm_sim_set_work")

    def set_timing(self, on: bool) -> None:
        check(lib().wm_sim_set_timing(self._h, 1 if on else 0), "wm_sim_set_timing")

    def kernel_times(self) -> dict:
        n = ctypes.c_int(64)
        names = (ctypes.c_char_p * 64)()
        ms = (ctypes.c_double * 64)()
        check(lib().wm_sim_kernel_times(self._h, names, ms, ctypes.byref(n)), "wm_sim_kernel_times")
        return {names[i].decode(): ms[i] for i in range(n.value)}

    def launches(self) -> int:
        c = ctypes.c_int64()
        check(lib().wm_sim_launches(self._h, ctypes.byref(c)), "wm_sim_launches")
        return c.value

    def info(self):
        n, b = ctypes.c_int64(), ctypes.c_int64()
        check(lib().wm_sim_info(self._h, ctypes.byref(n), ctypes.byref(b)), "wm_sim_info")
        return n.value, b.value

    def close(self) -> None:
        if self._h:
            lib().wm_sim_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def set_device(device: int) -> None:
    check(lib().wm_set_device(int(device)), "wm_set_device")


def pin(a: np.ndarray) -> None:
    """Page-lock a numpy array in place (cudaHostRegister)."""
    check(lib().wm_host_register(a.ctypes.data, a.nbytes), "wm_host_register")


def unpin(a: np.ndarray) -> None:
    check(lib().wm_host_unregister(a.ctypes.data), "wm_host_unregister")


class _PinnedBlock:
    """Page-locked host bytes from wm_host_alloc, freed when the last array over them goes."""

    def __init__(self, nbytes: int):
        p = ctypes.c_void_p()
        check(lib().wm_host_alloc(ctypes.byref(p), int(nbytes)), "wm_host_alloc")
        self.ptr, self.nbytes = p.value, int(nbytes)
        self.__array_interface__ = {"shape": (self.nbytes,), "typestr": "|u1", "data": (self.ptr, False), "version": 3}

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().wm_host_free(self.ptr)
            self.ptr = None


def pinned_zeros(shape, dtype=np.float64, order: str = "F") -> np.ndarray:
    """A zero-filled array in page-locked host memory (the layout of np.zeros(shape, dtype, order)),
    for the state that wm_sim_step_host copies in and out every call."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    a = np.asarray(_PinnedBlock(max(n, 1)))[:n].view(dtype)
    a = a.reshape(shape, order=order)
    a[...] = 0
    return a
