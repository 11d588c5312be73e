"""The resident simulation (state kept on the GPU) against the CPU restatement's step loop.

After each step the cell counts (cumcnt, np2) and the slot of every particle
(compared through its id) must match exactly; positions, momenta and fields to
a normwise relative error of TOL = 1e-12 per component.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import State, rel_err
from wumingpic2d_gb300.layout import bits_to_pid
from wumingpic2d_gb300.sim import Simulation

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _sim(st, **kw):
    return Simulation(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, **kw)


def _compare(st, up, uf, np2, cumcnt, ref_up, ref_uf, ref_np2, ref_cc, tol=TOL):
    d = st.d
    assert np.array_equal(np2, ref_np2)
    assert np.array_equal(cumcnt, ref_cc)
    for isp in range(d.nsp):
        for j in range(d.ny):
            n = ref_np2[j, isp]
            assert np.array_equal(bits_to_pid(up[5, :n, j, isp]), bits_to_pid(ref_up[5, :n, j, isp])), (isp, j)
    for k in range(5):
        a = np.concatenate([up[k, :ref_np2[j, s], j, s] for s in range(d.nsp) for j in range(d.ny)])
        b = np.concatenate([ref_up[k, :ref_np2[j, s], j, s] for s in range(d.nsp) for j in range(d.ny)])
        assert rel_err(a, b) <= tol, k
    for k in range(6):
        assert rel_err(uf[k], ref_uf[k]) <= tol, k


def test_load_sorts_like_sort_bucket(gpu):
    st = State(nx=40, ny=20, ppc=8)
    from wumingpic2d_gb300.weibel import weibel_particles

    up0, np2 = weibel_particles(st.cfg)
    with _sim(st) as sim:
        sim.load(up0, st.uf, np2)
        up, uf, np2o, cc = sim.store()
    assert np.array_equal(np2o, st.np2)
    assert np.array_equal(cc, st.cumcnt)
    for isp in range(2):
        for j in range(st.d.ny):
            n = st.np2[j, isp]
            assert np.array_equal(up[:, :n, j, isp].view(np.int64), st.up[:, :n, j, isp].view(np.int64))


@pytest.mark.parametrize("amp,dfamp", [(0.05, 1e-3)])
def test_one_step_from_state(gpu, amp, dfamp):
    st = State(nx=48, ny=32, ppc=10, field_amp=amp, df_amp=dfamp)
    ref = st.copy()
    S = ref.oracle_state()
    stt, it_ref = O.step(ref.par, ref.d, ref.up, ref.gp, ref.uf, ref.cumcnt, ref.np2, S)
    assert stt == 0
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        sim.set_work(st.df)
        sim.step(1)
        assert np.array_equal(sim.cg_iters(), it_ref)
        up, uf, np2, cc = sim.store()
        df, uj = sim.get_work()
    _compare(st, up, uf, np2, cc, ref.up, ref.uf, ref.np2, ref.cumcnt)
    for k in range(6):
        assert rel_err(df[k], S.df[k]) <= TOL
    for k in range(3):
        assert rel_err(uj[k], S.uj[k]) <= TOL


def test_ten_steps_weibel(gpu):
    st = State(nx=64, ny=64, ppc=8, seed=11)
    ref = st.copy()
    S = ref.oracle_state()
    iters = []
    for _ in range(10):
        stt, it = O.step(ref.par, ref.d, ref.up, ref.gp, ref.uf, ref.cumcnt, ref.np2, S)
        assert stt == 0
        iters.append(it.copy())
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        for it in iters:
            sim.step(1)
            assert np.array_equal(sim.cg_iters(), it)
        up, uf, np2, cc = sim.store()
        e_gpu = sim.energy()
        mom_gpu = sim.moments()
    _compare(st, up, uf, np2, cc, ref.up, ref.uf, ref.np2, ref.cumcnt, tol=1e-11)
    e_ref = O.energy(ref.par, ref.d, ref.up, ref.uf, ref.np2)
    assert rel_err(e_gpu, e_ref) <= 1e-11
    gp = ref.gp.copy(order="F")
    O.mom_accl(ref.par, ref.d, gp, ref.up, ref.uf, ref.cumcnt)
    mom_ref = ref.d.alloc_mom()
    O.mom_nvt(ref.par, ref.d, mom_ref, gp, ref.np2)
    O.bc_mom(ref.par, ref.d, mom_ref)
    for k in range(7):
        assert rel_err(mom_gpu[k], mom_ref[k]) <= 1e-11, k


def test_step_host_equals_resident(gpu):
    st = State(nx=32, ny=32, ppc=8, field_amp=0.02)
    a = st.copy()
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        sim.step(2)
        up1, uf1, np21, cc1 = sim.store()
    with _sim(st) as sim:
        up, uf, np2, cc = a.up, a.uf, a.np2, a.cumcnt
        sim.step_host(up, uf, np2, cc, 1)
        sim.step_host(up, uf, np2, cc, 1)
    assert np.array_equal(np2, np21) and np.array_equal(cc, cc1)
    for isp in range(2):
        for j in range(st.d.ny):
            n = np2[j, isp]
            assert np.array_equal(up[:, :n, j, isp].view(np.int64), up1[:, :n, j, isp].view(np.int64))
    assert np.array_equal(uf.view(np.int64), uf1.view(np.int64))
