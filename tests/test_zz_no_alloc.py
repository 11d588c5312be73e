"""The allocation-free current deposit, checked against the allocating path through the C ABI.

Callers that cannot call cudaMalloc -- for example an application that hands this library GPU
memory from its own pool and allows no allocation after start-up -- use
wm_deposit_current_noalloc: they pass their own device buffers, and the scratch of the deposit
comes from a fixed static array inside the library.  This test acts as such a caller: it makes its
device buffers itself through the CUDA runtime, calls the entry point several times in a row on
different states (the calls share the library's scratch), and compares each current with the one
field__fdtd_i deposits on the allocating path, to the 1e-12 normwise tolerance of the other GPU
tests.  It also checks that a grid over the size limit is refused.  This file is collected last.
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


def noalloc_path(bufs, st, gp):
    d = st.d
    dup, dgp, dcc = bufs.put(st.up), bufs.put(gp), bufs.put(st.cumcnt)
    uj = d.alloc_uj()
    duj = bufs.alloc(uj.nbytes)
    q = np.ascontiguousarray(st.cfg.charge, dtype=np.float64)
    status = lib().wm_deposit_current_noalloc(dup, dgp, dcc, duj, d.ndim, d.np, d.nsp, d.nxgs, d.nxge, d.nygs, d.nyge, 1.0,
                                              st.cfg.delt, 1.0, q.ctypes.data, None)
    assert status == 0, status
    bufs.get(duj, uj)
    return uj


def test_noalloc_deposit_matches_allocating_path_on_consecutive_calls(gpu):
    states = [State(nx=48, ny=40, ppc=8, seed=21, field_amp=0.05),
              State(nx=40, ny=32, ppc=12, seed=22, field_amp=0.08)]
    expected = [allocating_path(st) for st in states]
    bufs = CallerBuffers()
    try:
        for st, (gp, uj_ref) in [(states[0], expected[0]), (states[1], expected[1]), (states[0], expected[0])]:
            uj = noalloc_path(bufs, st, gp)
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
