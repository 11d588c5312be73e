"""The wall boundary modules of the reconnection and shock applications
(proj/reconnection/boundary_reconnection.f90, proj/shock/boundary_shock.f90): the hand
restatement (oracle/wm_oracle.c with par.bc set) against the reference's own Fortran translated to
C (oracle/f90c.py), bit for bit, routine by routine and over whole steps in each application's
order (proj/reconnection/app.f90:101-106, proj/shock/app.f90:112-117).
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import reference as R
from tests.helpers import State, confine_x

pytestmark = pytest.mark.skipif(not R.available(), reason="reference translation unavailable")

U0 = -0.1 / np.sqrt(1 - 0.01)  # upstream four-velocity of the shock app (u0 = -0.1c)


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.fixture(autouse=True)
def one_thread():
    O.set_threads(1)
    yield


def setup(bc, **kw):
    st = State(**kw)
    st.par = O.make_par(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc, u0=U0)
    ref = R.Reference(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc)
    return st, ref


@pytest.mark.parametrize("bc", ["reconnection", "shock"])
def test_wall_ghost_routines(bc):
    st, ref = setup(bc, nx=12, ny=10, ppc=1)
    rng = np.random.default_rng(6)
    d = st.d
    for shape, fo, fr in (((6, d.nx + 4, d.ny + 4), O.bc_dfield, ref.bc_dfield),
                          ((3, d.nx + 4, d.ny + 4), O.bc_curre, ref.bc_curre)):
        a = np.asfortranarray(rng.standard_normal(shape))
        b = a.copy(order="F")
        fo(st.par, d, a)
        assert fr(b) == 0
        assert np.array_equal(bits(a), bits(b))
    for l in (1, 2, 3):
        a = np.asfortranarray(rng.standard_normal((d.nx + 2, d.ny + 2)))
        b = a.copy(order="F")
        O.bc_phi(st.par, d, a, l)
        assert ref.bc_phi(b, l) == 0
        assert np.array_equal(bits(a), bits(b))
    a = np.asfortranarray(rng.standard_normal((7, d.nx + 2, d.ny + 2, d.nsp)))
    b = a.copy(order="F")
    O.bc_mom(st.par, d, a)
    assert ref.bc_mom(b) == 0
    assert np.array_equal(bits(a), bits(b))


@pytest.mark.parametrize("bc", ["reconnection", "shock"])
def test_wall_particle_boundaries(bc):
    st, ref = setup(bc, nx=20, ny=16, ppc=9, field_amp=0.08, seed=43)
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    a, b = gp.copy(order="F"), gp.copy(order="F")
    O.bc_particle_x_walls(st.par, st.d, a, st.np2)
    assert ref.bc_particle_x_walls(b, st.np2) == 0
    assert np.array_equal(bits(a), bits(b))
    if bc == "shock":
        a, b = gp.copy(order="F"), gp.copy(order="F")
        O.bc_injection(st.par, st.d, a, st.np2, U0)
        assert ref.bc_injection(b, st.np2, U0) == 0
        assert np.array_equal(bits(a), bits(b))
        assert not np.array_equal(bits(a), bits(gp))  # some particles were reflected


@pytest.mark.parametrize("bc", ["reconnection", "shock"])
def test_wall_steps(bc):
    st, ref = setup(bc, nx=32, ny=24, ppc=8, field_amp=0.02, seed=44)
    confine_x(st)  # inside the walls, where the applications keep their particles
    a, b = st.copy(), st.copy()
    S = a.oracle_state()
    iters = []
    for _ in range(8):
        status, it = O.step(a.par, a.d, a.up, a.gp, a.uf, a.cumcnt, a.np2, S)
        assert status == 0
        iters.append(it.copy())
        assert ref.particle_solv(b.gp, b.up, b.uf, b.cumcnt) == 0
        if bc == "shock":
            assert ref.bc_injection(b.gp, b.np2, U0) == 0
        assert ref.field_fdtd_i(b.uf, b.up, b.gp, b.cumcnt) == 0
        if bc == "reconnection":
            assert ref.bc_particle_x_walls(b.gp, b.np2) == 0
        assert ref.bc_particle_y(b.gp, b.np2) == 0
        assert ref.sort_bucket(b.up, b.gp, b.cumcnt, b.np2) == 0
    assert np.array_equal(a.np2, b.np2) and np.array_equal(a.cumcnt, b.cumcnt)
    assert np.array_equal(bits(a.up), bits(b.up))
    assert np.array_equal(bits(a.uf), bits(b.uf))
    df_r, uj_r, _ = ref.get_work()
    assert np.array_equal(bits(S.df), bits(df_r)) and np.array_equal(bits(S.uj), bits(uj_r))
    assert all(i.min() > 0 for i in iters)
