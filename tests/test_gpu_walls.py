"""The reconnection and shock boundary modules on the GPU against the CPU restatement (itself
pinned bit for bit to the translated Fortran in test_reference_pin_walls.py).

Integer and copy work (particle reflections, ghost layers) bit-exact; FP64 arithmetic to a
normwise relative error of 1e-12 per component (TOL), CG iteration counts equal.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import State, confine_x, rel_err
from wumingpic2d_gb300 import api
from wumingpic2d_gb300.sim import Simulation

pytestmark = pytest.mark.gpu
TOL = 1e-12
U0 = -0.1 / np.sqrt(1 - 0.01)
KINDS = ["reconnection", "shock"]


def setup(bc, **kw):
    st = State(**kw)
    st.par = O.make_par(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc, u0=U0)
    api.init_all(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc)
    return st


def mod(bc):
    return {"dfield": getattr(api, f"boundary_{bc}__dfield"), "curre": getattr(api, f"boundary_{bc}__curre"),
        "phi": getattr(api, f"boundary_{bc}__phi"), "mom": getattr(api, f"boundary_{bc}__mom"),
        "particle_x": getattr(api, f"boundary_{bc}__particle_x"), "particle_y": getattr(api, f"boundary_{bc}__particle_y")}


@pytest.mark.parametrize("bc", KINDS)
def test_wall_ghost_routines_bit_exact(gpu, bc):
    st = setup(bc, nx=24, ny=12, ppc=1)
    d, m = st.d, mod(bc)
    rng = np.random.default_rng(8)
    args = (d.nxs, d.nxe, d.nys, d.nye, d.nxgs, d.nxge)
    for nc, fo, fg in ((6, O.bc_dfield, m["dfield"]), (3, O.bc_curre, m["curre"])):
        a = np.asfortranarray(rng.standard_normal((nc, d.nx + 4, d.ny + 4)))
        b = a.copy(order="F")
        fo(st.par, d, a)
        fg(b, *args)
        assert np.array_equal(a, b)
    for l in (1, 2, 3):
        a = np.asfortranarray(rng.standard_normal((d.nx + 2, d.ny + 2)))
        b = a.copy(order="F")
        O.bc_phi(st.par, d, a, l)
        m["phi"](b, d.nxs, d.nxe, d.nys, d.nye, l)
        assert np.array_equal(a, b)
    a = np.asfortranarray(rng.standard_normal((7, d.nx + 2, d.ny + 2, d.nsp)))
    b = a.copy(order="F")
    O.bc_mom(st.par, d, a)
    m["mom"](b)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("bc", KINDS)
def test_wall_particle_boundaries_bit_exact(gpu, bc):
    st = setup(bc, nx=32, ny=16, ppc=8, field_amp=0.06, seed=51)
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    a, b = gp.copy(order="F"), gp.copy(order="F")
    O.bc_particle_x_walls(st.par, st.d, a, st.np2)
    mod(bc)["particle_x"](b, st.np2, st.d.nxs, st.d.nxe)
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    if bc == "shock":
        a, b = gp.copy(order="F"), gp.copy(order="F")
        O.bc_injection(st.par, st.d, a, st.np2, U0)
        api.boundary_shock__injection(b, st.np2, st.d.nxs, st.d.nxe, U0)
        assert np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("bc", KINDS)
def test_wall_field_update(gpu, bc):
    st = setup(bc, nx=40, ny=24, ppc=8, field_amp=0.05, df_amp=1e-3, seed=52)
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    S = st.oracle_state()
    uf_o = st.uf.copy(order="F")
    status, it_o = O.field_fdtd_i(st.par, st.d, uf_o, st.up, gp, st.cumcnt, S)
    assert status == 0
    api.field__set_work(st.df)
    uf_g = st.uf.copy(order="F")
    api.field__fdtd_i(uf_g, st.up, gp, st.cumcnt, st.d.nxs, st.d.nxe)
    assert np.array_equal(api.field__cg_iters(), it_o)
    for k in range(6):
        assert rel_err(uf_g[k], uf_o[k]) <= TOL, k


@pytest.mark.parametrize("bc", KINDS)
def test_wall_resident_steps(gpu, bc):
    """Resident FP64 steps in the application's order against the oracle's steps."""
    st = setup(bc, nx=48, ny=32, ppc=8, field_amp=0.02, seed=53, slack=2.0)
    confine_x(st)  # start where the applications keep their particles (inside the walls)
    ref = st.copy()
    S = ref.oracle_state()
    iters = []
    for _ in range(6):
        status, it = O.step(ref.par, ref.d, ref.up, ref.gp, ref.uf, ref.cumcnt, ref.np2, S)
        assert status == 0
        iters.append(it.copy())
    with Simulation(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc, u0=U0) as sim:
        sim.load(st.up, st.uf, st.np2)
        for _ in range(5):
            sim.step(1)
        sim.step(1)
        it_g = sim.cg_iters()
        up, uf, np2, cc = sim.store()
    assert np.array_equal(it_g, iters[-1])
    assert np.array_equal(np2, ref.np2) and np.array_equal(cc, ref.cumcnt)
    for isp in range(st.d.nsp):
        for j in range(st.d.ny):
            n = np2[j, isp]
            assert np.array_equal(up[5, :n, j, isp].view(np.int64), ref.up[5, :n, j, isp].view(np.int64))
            for k in range(5):  # active slots only (the reference leaves stale data beyond np2)
                assert rel_err(up[k, :n, j, isp], ref.up[k, :n, j, isp]) <= 1e-11, k
    for k in range(6):
        assert rel_err(uf[k], ref.uf[k]) <= 1e-11, k


@pytest.mark.parametrize("bc", KINDS)
def test_wall_mixed_path_tracks_fp64(gpu, bc):
    """The mixed path with walls (reflections in integer cells and FP32 offsets) against the FP64
    path over 10 steps, particles matched by id: positions and momenta within 1e-5, total energy
    within 1e-7."""
    st = setup(bc, nx=64, ny=32, ppc=8, field_amp=0.02, seed=54, slack=2.0)
    confine_x(st)
    out = {}
    for precision in ("fp64", "mixed"):
        with Simulation(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc, u0=U0, precision=precision) as sim:
            sim.load(st.up, st.uf, st.np2)
            sim.step(10)
            up, uf, np2, cc = sim.store()
            out[precision] = (up, uf, np2, sim.energy())
    def by_pid(up, np2):
        cols = [np.concatenate([up[k, :np2[j, s], j, s] for s in range(2) for j in range(st.d.ny)]) for k in range(6)]
        order = np.argsort(cols[5].view(np.int64), kind="stable")
        return [c[order] for c in cols]
    a, b = by_pid(out["fp64"][0], out["fp64"][2]), by_pid(out["mixed"][0], out["mixed"][2])
    assert np.array_equal(a[5].view(np.int64), b[5].view(np.int64))
    errs = [np.max(np.abs(a[k] - b[k])) for k in range(2)] + [rel_err(b[k], a[k]) for k in range(2, 5)]
    de = abs(out["mixed"][3].sum() - out["fp64"][3].sum()) / out["fp64"][3].sum()
    print(f"\n{bc} mixed vs fp64 after 10 steps: x {errs[0]:.1e} y {errs[1]:.1e} u {max(errs[2:]):.1e} energy {de:.1e}")
    assert max(errs) <= 1e-5 and de <= 1e-7
