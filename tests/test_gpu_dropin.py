"""Each common/ module procedure on the GPU against the CPU restatement, same inputs.

Integer and permutation work (sort, particle boundaries, ghost copies) must be
bit-exact; FP64 arithmetic must agree to a normwise relative error of 1e-12
per component (TOL).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import State, periodic_ghosts, rel_err
from wumingpic2d_gb300 import api

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _init(st):
    api.init_all(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass)


def _pid(a):
    return a[5].view(np.int64)


@pytest.mark.parametrize("amp", [0.0, 0.05])
def test_particle_solv(gpu, amp):
    st = State(nx=40, ny=24, ppc=8, field_amp=amp)
    _init(st)
    ref = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, ref, st.up, st.uf, st.cumcnt)
    out = st.gp.copy(order="F")
    api.particle__solv(out, st.up, st.uf, st.cumcnt, st.d.nxs, st.d.nxe)
    for k in range(5):
        assert rel_err(out[k], ref[k]) <= TOL, k
    assert np.array_equal(_pid(out), _pid(ref))


def test_mom_calc_accl(gpu):
    st = State(nx=32, ny=16, ppc=6, field_amp=0.05)
    _init(st)
    ref = st.gp.copy(order="F")
    O.mom_accl(st.par, st.d, ref, st.up, st.uf, st.cumcnt)
    out = st.gp.copy(order="F")
    api.mom_calc__accl(out, st.up, st.uf, st.cumcnt, st.d.nxs, st.d.nxe)
    assert np.array_equal(out[:2], ref[:2])
    for k in range(2, 5):
        assert rel_err(out[k], ref[k]) <= TOL, k
    assert np.array_equal(_pid(out), _pid(ref))


def _pushed(st):
    """gp after the oracle push and particle_x (input of particle_y)."""
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    return gp


def test_particle_x_bit_exact(gpu):
    st = State(nx=32, ny=16, ppc=8, field_amp=0.05)
    _init(st)
    gp = _pushed(st)
    ref = gp.copy(order="F")
    O.bc_particle_x(st.par, st.d, ref, st.np2)
    out = gp.copy(order="F")
    api.boundary_periodic__particle_x(out, st.np2)
    assert np.array_equal(out.view(np.int64), ref.view(np.int64))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_particle_y_bit_exact(gpu, seed):
    st = State(nx=24, ny=20, ppc=10, seed=seed, field_amp=0.08)
    _init(st)
    gp = _pushed(st)
    O.bc_particle_x(st.par, st.d, gp, st.np2)
    ref, np2_ref = gp.copy(order="F"), st.np2.copy(order="F")
    assert O.bc_particle_y(st.par, st.d, ref, np2_ref) == 0
    out, np2_out = gp.copy(order="F"), st.np2.copy(order="F")
    api.boundary_periodic__particle_y(out, np2_out)
    assert np.array_equal(np2_out, np2_ref)
    assert np.array_equal(out.view(np.int64), ref.view(np.int64))


def test_sort_bucket_bit_exact(gpu):
    st = State(nx=48, ny=16, ppc=12, field_amp=0.05)
    _init(st)
    gp = _pushed(st)
    O.bc_particle_x(st.par, st.d, gp, st.np2)
    np2 = st.np2.copy(order="F")
    assert O.bc_particle_y(st.par, st.d, gp, np2) == 0
    init_out = st.d.alloc_up()
    init_out[:] = -1.0
    ref, cc_ref = init_out.copy(order="F"), st.d.alloc_cumcnt()
    assert O.sort_bucket(st.par, st.d, ref, gp, cc_ref, np2) == 0
    out, cc_out = init_out.copy(order="F"), st.d.alloc_cumcnt()
    api.sort__bucket(out, gp, cc_out, np2, st.d.nxs, st.d.nxe)
    assert np.array_equal(cc_out, cc_ref)
    assert np.array_equal(out.view(np.int64), ref.view(np.int64))


def test_ghost_routines_bit_exact(gpu):
    st = State(nx=20, ny=12, ppc=2)
    _init(st)
    d = st.d
    rng = np.random.default_rng(3)
    df = np.asfortranarray(rng.standard_normal((6, d.nx + 4, d.ny + 4)))
    ref = df.copy(order="F")
    O.bc_dfield(st.par, d, ref)
    api.boundary_periodic__dfield(df, d.nxs, d.nxe, d.nys, d.nye, d.nxgs, d.nxge)
    assert np.array_equal(df, ref)
    uj = np.asfortranarray(rng.standard_normal((3, d.nx + 4, d.ny + 4)))
    ref = uj.copy(order="F")
    O.bc_curre(st.par, d, ref)
    api.boundary_periodic__curre(uj, d.nxs, d.nxe, d.nys, d.nye, d.nxgs, d.nxge)
    assert np.array_equal(uj, ref)
    phi = np.asfortranarray(rng.standard_normal((d.nx + 2, d.ny + 2)))
    ref = phi.copy(order="F")
    O.bc_phi(st.par, d, ref)
    api.boundary_periodic__phi(phi, d.nxs, d.nxe, d.nys, d.nye, 1)
    assert np.array_equal(phi, ref)
    mom = np.asfortranarray(rng.standard_normal((7, d.nx + 2, d.ny + 2, d.nsp)))
    ref = mom.copy(order="F")
    O.bc_mom(st.par, d, ref)
    api.boundary_periodic__mom(mom)
    assert np.array_equal(mom, ref)


@pytest.mark.parametrize("amp,dfamp", [(0.0, 0.0), (0.05, 1e-3)])
def test_field_fdtd_i(gpu, amp, dfamp):
    st = State(nx=40, ny=32, ppc=8, field_amp=amp, df_amp=dfamp)
    _init(st)
    gp = _pushed(st)
    S = st.oracle_state()
    uf_ref = st.uf.copy(order="F")
    stt, it_ref = O.field_fdtd_i(st.par, st.d, uf_ref, st.up, gp, st.cumcnt, S)
    assert stt == 0
    api.field__set_work(st.df)
    uf = st.uf.copy(order="F")
    api.field__fdtd_i(uf, st.up, gp, st.cumcnt, st.d.nxs, st.d.nxe)
    assert np.array_equal(api.field__cg_iters(), it_ref)
    for k in range(6):
        assert rel_err(uf[k], uf_ref[k]) <= TOL, k
    df = st.d.alloc_uf()
    uj = st.d.alloc_uj()
    api.field__get_work(df, uj)
    for k in range(3):
        assert rel_err(uj[k], S.uj[k]) <= TOL, k
    for k in range(6):
        assert rel_err(df[k], S.df[k]) <= TOL, k


def test_mom_calc_nvt(gpu):
    st = State(nx=32, ny=16, ppc=8, field_amp=0.05)
    _init(st)
    ref = st.d.alloc_mom()
    O.mom_nvt(st.par, st.d, ref, st.up, st.np2)
    out = st.d.alloc_mom()
    api.mom_calc__nvt(out, st.up, st.np2)
    for k in range(7):
        assert rel_err(out[k], ref[k]) <= TOL, k


def test_energy_sums(gpu):
    st = State(nx=32, ny=16, ppc=8, field_amp=0.05)
    _init(st)
    ref = O.energy(st.par, st.d, st.up, st.uf, st.np2)
    out = api.energy_sums(st.up, st.uf, st.np2, st.d.nsp)
    assert rel_err(out, ref) <= TOL


def test_uninitialised_module_reports_status(gpu):
    api.finalize()
    st = State(nx=8, ny=8, ppc=1)
    with pytest.raises(Exception):
        api.particle__solv(st.gp, st.up, st.uf, st.cumcnt, st.d.nxs, st.d.nxe)
    _init(st)


def test_sort_reports_out_of_grid(gpu):
    st = State(nx=16, ny=8, ppc=2)
    _init(st)
    bad = st.up.copy(order="F")
    bad[0, 0, 0, 0] = st.d.nxge + 5.0  # outside nxs..nxe
    out = st.d.alloc_up()
    with pytest.raises(Exception):
        api.sort__bucket(out, bad, st.d.alloc_cumcnt(), st.np2, st.d.nxs, st.d.nxe)
