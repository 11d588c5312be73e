"""The host-buffer step with page-locked, device-mapped arrays (wm_host_alloc): the particle rows
move in chunks on a second stream, overlapped with the unpack and pack kernels.  The result must be
bit-identical to the same step through ordinary host arrays (one pitched copy each way)."""
import numpy as np
import pytest

from tests.helpers import State
from wumingpic2d_gb300.sim import Simulation, pinned_zeros

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_host_page_locked_matches_pageable(gpu, precision):
    st = State(nx=64, ny=48, ppc=8, field_amp=0.02, seed=71, slack=1.5)
    d = st.d
    args = (d, st.cfg.delt, st.cfg.charge, st.cfg.mass)
    results = []
    for pinned in (False, True):
        with Simulation(*args, precision=precision) as sim:
            sim.load(st.up, st.uf, st.np2)
            u, f, n, c = sim.store(up=d.alloc_up())  # a cell-sorted state with its cumcnt
            if pinned:
                up, uf = pinned_zeros(u.shape), pinned_zeros(f.shape)
                up[...] = u
                uf[...] = f
            else:
                up, uf = u, f
            for _ in range(3):
                sim.step_host(up, uf, n, c, 1)
            results.append((np.array(up), np.array(uf), n.copy(), c.copy()))
    (ua, fa, na, ca), (ub, fb, nb, cb) = results
    assert np.array_equal(na, nb) and np.array_equal(ca, cb)
    assert np.array_equal(fa, fb)
    assert np.array_equal(ua.view(np.uint64), ub.view(np.uint64))
