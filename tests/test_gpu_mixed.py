"""The mixed-precision path (FP32 push and deposit, FP64 fields and CG) against the FP64 oracle.

Stated bounds (normwise relative unless noted), measured with these seeded states:
  * load/store round trip: positions to 1e-7 cells (FP32 in-cell offsets), momenta to 1e-7;
  * one step from a state with fields: positions 2e-6 cells (absolute), momenta 2e-6, J 1e-5,
    E and B 1e-5, same CG iteration counts within one;
  * total energy of a 40-step Weibel run within 1e-6 of the FP64 run; div E - 4 pi rho drifts by
    at most 1e-5 of 4 pi |rho|.
Particles are matched by id, since a particle within an FP32 rounding of a cell edge may land in
the neighbouring cell.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import State, rel_err
from wumingpic2d_gb300.layout import bits_to_pid
from wumingpic2d_gb300.sim import Simulation

pytestmark = pytest.mark.gpu


def _sim(st, precision="mixed"):
    return Simulation(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, precision=precision)


def by_pid(d, up, np2):
    """Per species: (pid-sorted) x, y, ux, uy, uz."""
    out = []
    for isp in range(d.nsp):
        cols = [np.concatenate([up[k, :np2[j, isp], j, isp] for j in range(d.ny)]) for k in range(5)]
        pid = np.concatenate([bits_to_pid(up[5, :np2[j, isp], j, isp]) for j in range(d.ny)])
        order = np.argsort(pid, kind="stable")
        out.append((pid[order], [c[order] for c in cols]))
    return out


def periodic_diff(a, b, n):
    d = a - b
    return d - n * np.round(d / n)


def test_mixed_load_store_roundtrip(gpu):
    st = State(nx=48, ny=32, ppc=8, seed=41)
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        up, uf, np2, cc = sim.store()
    assert np.array_equal(np2, st.np2) and np.array_equal(cc, st.cumcnt)
    for isp in range(2):
        for j in range(st.d.ny):
            n = np2[j, isp]
            assert np.array_equal(bits_to_pid(up[5, :n, j, isp]), bits_to_pid(st.up[5, :n, j, isp]))
            assert np.max(np.abs(up[0:2, :n, j, isp] - st.up[0:2, :n, j, isp]), initial=0) <= 1e-7
            assert np.all(np.floor(up[0, :n, j, isp]) == np.floor(st.up[0, :n, j, isp]))
    assert rel_err(up[2:5], st.up[2:5]) <= 1e-7


def test_mixed_one_step_against_fp64(gpu):
    st = State(nx=64, ny=48, ppc=12, seed=42, field_amp=0.05, df_amp=1e-3)
    ref = st.copy()
    S = ref.oracle_state()
    stt, it_ref = O.step(ref.par, ref.d, ref.up, ref.gp, ref.uf, ref.cumcnt, ref.np2, S)
    assert stt == 0
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        sim.set_work(st.df)
        sim.step(1)
        it = sim.cg_iters()
        up, uf, np2, cc = sim.store()
        df, uj = sim.get_work()
    assert np.all(np.abs(it - it_ref) <= 1)
    a, b = by_pid(st.d, up, np2), by_pid(st.d, ref.up, ref.np2)
    errs = {}
    for isp in range(2):
        assert np.array_equal(a[isp][0], b[isp][0])
        errs[f"x{isp}"] = np.max(np.abs(periodic_diff(a[isp][1][0], b[isp][1][0], st.d.nx)))
        errs[f"y{isp}"] = np.max(np.abs(periodic_diff(a[isp][1][1], b[isp][1][1], st.d.ny)))
        errs[f"u{isp}"] = rel_err(np.stack(a[isp][1][2:5]), np.stack(b[isp][1][2:5]))
    for k in range(3):
        errs[f"J{k}"] = rel_err(uj[k], S.uj[k])
    for k in range(6):
        errs[f"F{k}"] = rel_err(uf[k], ref.uf[k])
    print("mixed vs fp64, one step:", {k: f"{v:.2e}" for k, v in errs.items()})
    for isp in range(2):
        assert errs[f"x{isp}"] <= 2e-6 and errs[f"y{isp}"] <= 2e-6
        assert errs[f"u{isp}"] <= 2e-6
    for k in range(3):
        assert errs[f"J{k}"] <= 1e-5
    for k in range(6):
        assert errs[f"F{k}"] <= 1e-5


def _div_e(d, uf):
    ex = uf[3, 2:d.nx + 3, 2:d.ny + 2]
    ey = uf[4, 2:d.nx + 2, 2:d.ny + 3]
    return (ex[1:, :] - ex[:-1, :]) + (ey[:, 1:] - ey[:, :-1])


def _rho(d, up, np2, q):
    rho = np.zeros((d.nx, d.ny))
    for isp in range(d.nsp):
        for jj in range(d.ny):
            n = np2[jj, isp]
            x, y = up[0, :n, jj, isp], up[1, :n, jj, isp]
            i, j = np.floor(x).astype(int), np.floor(y).astype(int)
            hx, hy = x - 0.5 - i, y - 0.5 - j
            sx = [0.5 * (0.5 - hx) ** 2, 0.75 - hx**2, 0.5 * (0.5 + hx) ** 2]
            sy = [0.5 * (0.5 - hy) ** 2, 0.75 - hy**2, 0.5 * (0.5 + hy) ** 2]
            for a in range(3):
                for b in range(3):
                    np.add.at(rho, ((i + a - 1 - d.nxgs) % d.nx, (j + b - 1 - d.nygs) % d.ny), q[isp] * sx[a] * sy[b])
    return rho


def test_mixed_energy_and_gauss_law_over_a_run(gpu):
    st = State(nx=64, ny=64, ppc=8, seed=43)
    ref = st.copy()
    S = ref.oracle_state()
    q = st.cfg.charge
    e_ref = []
    for _ in range(40):
        assert O.step(ref.par, ref.d, ref.up, ref.gp, ref.uf, ref.cumcnt, ref.np2, S)[0] == 0
    e_ref = O.energy(ref.par, ref.d, ref.up, ref.uf, ref.np2)
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        g0 = _div_e(st.d, st.uf) - 4 * np.pi * _rho(st.d, st.up, st.np2, q)
        sim.step(40)
        e_mix = sim.energy()
        up, uf, np2, _ = sim.store()
    g = _div_e(st.d, uf) - 4 * np.pi * _rho(st.d, up, np2, q)
    scale = np.max(np.abs(4 * np.pi * _rho(st.d, up, np2, np.abs(q))))
    drift = np.max(np.abs(g - g0)) / scale
    de = abs(e_mix.sum() - e_ref.sum()) / e_ref.sum()
    print(f"mixed vs fp64 after 40 steps: total energy rel diff {de:.2e}, gauss drift {drift:.2e}")
    assert de <= 1e-6
    assert drift <= 1e-5


@pytest.mark.parametrize("shape", [(64, 48), (4, 4), (80, 4), (4, 16)])
def test_mixed_rebin_keeps_a_deterministic_cell_sorted_state(gpu, shape):
    """The mixed path's own rebin (direction counts from the push, one move): after steps every
    row is sorted by cell and consistent with cumcnt and np2, every particle is present once, and
    two runs from the same state agree bit for bit.  Small grids exercise the periodic wrap onto
    the same row or cell from both sides."""
    nx, ny = shape
    st = State(nx=nx, ny=ny, ppc=8, seed=47, field_amp=0.02, slack=3.0)
    outs = []
    for _ in range(2):
        with _sim(st) as sim:
            sim.load(st.up, st.uf, st.np2)
            sim.step(12)
            outs.append(sim.store())
    (up, uf, np2, cc), (up2, uf2, np22, cc2) = outs
    # bit patterns: the id component holds int64 bits, some of which read as NaN
    assert np.array_equal(up.view(np.uint64), up2.view(np.uint64)) and np.array_equal(uf, uf2) and np.array_equal(cc, cc2)
    d = st.d
    assert np2.sum() == st.np2.sum()
    for isp in range(d.nsp):
        pids = []
        for j in range(d.ny):
            n = np2[j, isp]
            assert cc[0, j, isp] == 0 and cc[d.nx, j, isp] == n
            x, y = up[0, :n, j, isp], up[1, :n, j, isp]
            cell = np.floor(x).astype(int) - d.nxgs
            assert np.all(np.diff(cell) >= 0) and np.all((cell >= 0) & (cell < d.nx))
            assert np.array_equal(np.searchsorted(cell, np.arange(d.nx + 1)), cc[:, j, isp])
            assert np.all(np.floor(y) == d.nys + j)
            pids.append(bits_to_pid(up[5, :n, j, isp]))
        pids = np.sort(np.concatenate(pids))
        ref = np.sort(np.concatenate([bits_to_pid(st.up[5, :st.np2[j, isp], j, isp]) for j in range(d.ny)]))
        assert np.array_equal(pids, ref)


@pytest.mark.parametrize("bc,shape", [("periodic", (64, 48)), ("periodic", (4, 4)), ("periodic", (80, 4)),
                                      ("reconnection", (64, 32)), ("shock", (64, 32))])
def test_mixed_rebin_permutation_equals_move(gpu, bc, shape):
    """The two rebins of the mixed path -- the permutation that the next push reads through
    (default) and the move into cell order after every step -- give the same state bit for bit:
    particles, their order, ids, fields, cumcnt, energies and CG iterations, including when the
    cell-sorted order is written out in the middle of a run (energy) and the run continues."""
    from tests.helpers import confine_x

    nx, ny = shape
    u0 = -0.1 / np.sqrt(1 - 0.01)
    st = State(nx=nx, ny=ny, ppc=8, seed=48, field_amp=0.02, slack=3.0)
    if bc != "periodic":
        confine_x(st)
    outs = {}
    for mode in ("move", "permute"):
        with Simulation(st.d, st.cfg.delt, st.cfg.charge, st.cfg.mass, bc=bc, u0=u0, precision="mixed") as sim:
            sim.set_rebin(mode)
            sim.load(st.up, st.uf, st.np2)
            sim.step(5)
            e5 = sim.energy()
            it5 = sim.cg_iters()
            sim.step(6)
            outs[mode] = (sim.store(), e5, it5, sim.energy(), sim.cg_iters())
    (a, ea5, ia5, ea, ia), (b, eb5, ib5, eb, ib) = outs["move"], outs["permute"]
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint64) if x.dtype == np.float64 else x, y.view(np.uint64) if y.dtype == np.float64 else y)
    assert np.array_equal(ea5, eb5) and np.array_equal(ea, eb)
    assert np.array_equal(ia5, ib5) and np.array_equal(ia, ib)


def test_mixed_rebin_permutation_equals_move_with_injection(gpu):
    """The same with the shock application's particle injection every step: the new particles take
    fresh slots past the push output and the permutations point at them."""
    from wumingpic2d_gb300.shock import ShockConfig

    cfg = ShockConfig(nx=96, ny=16, n_ppc=8, l_damp_ini=8.0, slack=3.0, seed=23, tracer_window=(30.0, 50.0))
    d = cfg.dims()
    outs = {}
    for mode in ("move", "permute"):
        with Simulation(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0, precision="mixed",
                        capacity=int(4 * cfg.n_ppc * d.nx * d.ny)) as sim:
            sim.set_rebin(mode)
            sim.init_shock(cfg)
            sim.step(4)
            e4 = sim.energy()
            sim.step(5)
            outs[mode] = (sim.store(up=d.alloc_up()), e4, sim.energy(), sim.info()[0])
    (a, ea4, ea, na), (b, eb4, eb, nb) = outs["move"], outs["permute"]
    assert na == nb and na > cfg.n_ppc * (d.nx - 2) * d.ny * 2
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint64) if x.dtype == np.float64 else x, y.view(np.uint64) if y.dtype == np.float64 else y)
    assert np.array_equal(ea4, eb4) and np.array_equal(ea, eb)


def test_mixed_one_step_with_many_cell_changes(gpu):
    """A hot plasma (electrons at 0.5c thermal speed, 96 per cell) in which more than 16 particles
    of a cell change cell in one step.  The push keeps up to 16 such particles per cell in a queue
    that its cell's lanes deposit after the loop; a tile whose queue overflows is recomputed with
    every particle deposited in the loop.  The step must meet the bounds of the one-step test above
    against the FP64 oracle, and two runs of three steps agree bit for bit."""
    st = State(nx=64, ny=32, ppc=96, seed=49, field_amp=0.05, df_amp=1e-3, slack=2.0)
    st.up[2:5, :, :, 1] *= 10.0  # (118 of the 2048 cells see more than 16 electrons leave; the ion tiles none)
    st.gp = st.up.copy(order="F")
    ref = st.copy()
    S = ref.oracle_state()
    assert O.step(ref.par, ref.d, ref.up, ref.gp, ref.uf, ref.cumcnt, ref.np2, S)[0] == 0
    # the electrons of the busiest cell that changed cell in the step: more than the queue holds
    d = st.d
    (pid0, c0), (pid1, c1) = by_pid(d, st.up, st.np2)[1], by_pid(d, ref.up, ref.np2)[1]
    assert np.array_equal(pid0, pid1)
    cell0 = (np.floor(c0[1]) * d.nx + np.floor(c0[0])).astype(int)
    moved = (np.floor(c0[0]) != np.floor(c1[0])) | (np.floor(c0[1]) != np.floor(c1[1]))
    assert np.bincount(cell0[moved]).max() > 16
    with _sim(st) as sim:
        sim.load(st.up, st.uf, st.np2)
        sim.set_work(st.df)
        sim.step(1)
        up, uf, np2, cc = sim.store()
        df, uj = sim.get_work()
    a, b = by_pid(d, up, np2), by_pid(d, ref.up, ref.np2)
    for isp in range(2):
        assert np.array_equal(a[isp][0], b[isp][0])
        assert np.max(np.abs(periodic_diff(a[isp][1][0], b[isp][1][0], d.nx))) <= 2e-6
        assert np.max(np.abs(periodic_diff(a[isp][1][1], b[isp][1][1], d.ny))) <= 2e-6
        assert rel_err(np.stack(a[isp][1][2:5]), np.stack(b[isp][1][2:5])) <= 2e-6
    for k in range(3):
        assert rel_err(uj[k], S.uj[k]) <= 1e-5, k
    for k in range(6):
        assert rel_err(uf[k], ref.uf[k]) <= 1e-5, k
    outs = []
    for _ in range(2):
        with _sim(st) as sim:
            sim.load(st.up, st.uf, st.np2)
            sim.step(3)
            outs.append(sim.store())
    for x, y in zip(*outs):
        assert np.array_equal(x.view(np.uint64) if x.dtype == np.float64 else x, y.view(np.uint64) if y.dtype == np.float64 else y)
