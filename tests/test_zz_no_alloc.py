"""The allocation-free current deposit, checked against the allocating path through the C ABI.

Callers that cannot call cudaMalloc -- for example an application that hands this library GPU
memory from its own pool and allows no allocation after start-up -- use
wm_deposit_current_noalloc: they pass their own device buffers, and the scratch of the deposit
comes from a fixed static array inside the library.  This test acts as such a caller: it makes its
device buffers itself through the CUDA runtime, calls the entry point several times in a row on
different states (the calls share the library's scratch), and compares each current with the one
field__fdtd_i deposits on the allocating path, to the 1e-12 normwise tolerance of the other GPU
tests.  It also checks that the device's free memory does not change on the calls after the first
(the first may place the static array in device memory under lazy module loading), that a particle
moving more than one cell is reported as WM_ERR_CELL and the next valid call returns WM_OK (the
shared status word is cleared on every call), and that a grid over the size limit is refused.
This file is collected last.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import State, rel_err
from wumingpic2d_gb300 import api
from wumingpic2d_gb300._native import lib

pytestmark = pytest.mark.gpu
TOL = 1e-12
WM_ERR_BAD_ARG = 3
WM_ERR_CELL = 4


class CallerBuffers:
    """Device buffers owned by the caller (allocated here, not by the entry point)."""

    H2D, D2H = 1, 2

    def __init__(self):
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")):
            if name:
                try:
                    rt = ctypes.CDLL(name)
                    break
                except OSError:
                    continue
        assert rt is not None, "CUDA runtime library not found"
        rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        rt.cudaFree.argtypes = [ctypes.c_void_p]
        rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
        self.rt = rt
        self.ptrs = []

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), nbytes) == 0
        self.ptrs.append(p)
        return p

    def put(self, a):
        p = self.alloc(a.nbytes)
        assert self.rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, self.H2D) == 0
        return p

    def get(self, p, out):
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, self.D2H) == 0

    def free_bytes(self):
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        assert self.rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
        return free.value

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []


def allocating_path(st):
    """Pushed particles and the current field__fdtd_i deposits (ele_cur + current fold)."""
    d = st.d
    api.init_all(d, st.cfg.delt, st.cfg.charge, st.cfg.mass)
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, d, gp, st.up, st.uf, st.cumcnt)
    api.field__fdtd_i(st.uf.copy(order="F"), st.up, gp, st.cumcnt, d.nxs, d.nxe)
    uj = d.alloc_uj()
    api.field__get_work(None, uj)
    return gp, uj


def noalloc_call(bufs, st, gp):
    """One call on caller-owned copies of (up, gp, cumcnt); returns (status, uj, the device's free
    bytes just before and just after the call)."""
    d = st.d
    dup, dgp, dcc = bufs.put(st.up), bufs.put(gp), bufs.put(st.cumcnt)
    uj = d.alloc_uj()
    duj = bufs.alloc(uj.nbytes)
    q = np.ascontiguousarray(st.cfg.charge, dtype=np.float64)
    before = bufs.free_bytes()
    status = lib().wm_deposit_current_noalloc(dup, dgp, dcc, duj, d.ndim, d.np, d.nsp, d.nxgs, d.nxge, d.nygs, d.nyge, 1.0,
                                              st.cfg.delt, 1.0, q.ctypes.data, None)
    after = bufs.free_bytes()
    bufs.get(duj, uj)
    return status, uj, (before, after)


def noalloc_path(bufs, st, gp, check_free=False):
    status, uj, (before, after) = noalloc_call(bufs, st, gp)
    assert status == 0, status
    if check_free:  # not the first call on this device: the entry point allocates nothing
        assert before - after < 2 << 20, (before, after)  # an allocation takes at least one 2 MiB page
    return uj


def test_noalloc_deposit_matches_allocating_path_on_consecutive_calls(gpu):
    states = [State(nx=48, ny=40, ppc=8, seed=21, field_amp=0.05),
              State(nx=40, ny=32, ppc=12, seed=22, field_amp=0.08)]
    expected = [allocating_path(st) for st in states]
    bufs = CallerBuffers()
    try:
        for n, (st, (gp, uj_ref)) in enumerate([(states[0], expected[0]), (states[1], expected[1]), (states[0], expected[0])]):
            uj = noalloc_path(bufs, st, gp, check_free=n > 0)
            for k in range(3):
                assert rel_err(uj[k], uj_ref[k]) <= TOL, k
    finally:
        bufs.free()


def test_noalloc_refuses_grids_over_the_limit(gpu):
    bufs = CallerBuffers()
    try:
        p = bufs.alloc(64)  # never read: the size check comes first
        q = np.array([1.0, -1.0])
        status = lib().wm_deposit_current_noalloc(p, p, p, p, 6, 16, 2, 2, 513, 2, 257, 1.0, 0.5, 1.0, q.ctypes.data, None)
        assert status == WM_ERR_BAD_ARG
    finally:
        bufs.free()


def test_noalloc_reports_a_particle_moving_more_than_one_cell(gpu):
    st = State(nx=40, ny=32, ppc=8, seed=23, field_amp=0.05)
    gp, uj_ref = allocating_path(st)
    bad = gp.copy(order="F")
    x = bad[0, 0, 5, 1]  # one electron of row 5 lands three cells away, still inside the grid
    bad[0, 0, 5, 1] = x - 3.0 if x >= st.d.nxgs + 4 else x + 3.0
    assert st.d.nxgs <= bad[0, 0, 5, 1] < st.d.nxge + 1
    bufs = CallerBuffers()
    try:
        status, _, _ = noalloc_call(bufs, st, bad)
        assert status == WM_ERR_CELL
        uj = noalloc_path(bufs, st, gp)  # the status word starts from zero again
        for k in range(3):
            assert rel_err(uj[k], uj_ref[k]) <= TOL, k
    finally:
        bufs.free()
