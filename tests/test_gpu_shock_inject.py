"""The shock application's particle injection (proj/shock/app.f90:695-850) in the resident step,
against the oracle: the oracle's shock step (push, injection boundary, field solve, particle_y,
sort) followed by the restated inject on the host arrays, step by step.  Counts per row and cell,
ids and slots exact; positions, momenta and fields to 1e-11 (the new particles' normals differ in
the last bits between libm and CUDA).  The mixed path is checked against the FP64 path."""
import numpy as np
import pytest

from oracle import init as I
from oracle import oracle as O
from tests.helpers import rel_err
from wumingpic2d_gb300.shock import ShockConfig
from wumingpic2d_gb300.sim import Simulation

pytestmark = pytest.mark.gpu
STEPS = 4


def config():
    return ShockConfig(nx=96, ny=16, n_ppc=8, l_damp_ini=8.0, slack=3.0, seed=19, tracer_window=(30.0, 50.0))


def oracle_run(cfg, steps):
    d = cfg.dims()
    q, r = cfg.charge, cfg.mass
    a = cfg.init_args()
    up0, uf, np2 = I.shock(d, *a[:-1], seed=a[-1])
    par = O.make_par(d, cfg.delt, q, r, bc="shock", u0=cfg.u0)
    up, cc = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cc, np2) == 0
    gp = up.copy(order="F")
    S = O.OracleState(d)
    injected = []
    for it in range(steps):
        status, _ = O.step(par, d, up, gp, uf, cc, np2, S)
        assert status == 0
        injected.append(I.inject(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], cfg.delt))
    return up, uf, np2, cc, injected


def test_injection_matches_oracle(gpu):
    cfg = config()
    d = cfg.dims()
    up_o, uf_o, np2_o, cc_o, injected = oracle_run(cfg, STEPS)
    assert sum(int(n.sum()) for n in injected) > 0
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0, capacity=int(4 * cfg.n_ppc * d.nx * d.ny)) as sim:
        sim.init_shock(cfg)
        for _ in range(STEPS):
            sim.step(1)
        assert sim.step_number == STEPS
        up, uf, np2, cc = sim.store(up=d.alloc_up())
    assert np.array_equal(np2, np2_o)
    assert np.array_equal(cc[:d.nx], cc_o[:d.nx])          # cell starts, cumcnt(nxe) advanced as the Fortran does
    assert np.array_equal(cc[d.nx], np2)                   # the row total column follows the rows here
    n = int(np2.max())
    for isp in range(d.nsp):
        for j in range(d.ny):
            m = int(np2[j, isp])
            assert np.array_equal(up[5, :m, j, isp].view(np.int64), up_o[5, :m, j, isp].view(np.int64))
            for k in range(5):
                assert rel_err(up[k, :m, j, isp], up_o[k, :m, j, isp]) <= 1e-11, (isp, j, k)
    for k in range(6):
        assert rel_err(uf[k], uf_o[k]) <= 1e-11, k
    assert n > cfg.n_ppc * (d.nx - 2)  # the rows grew


def test_injection_mixed_tracks_fp64(gpu):
    cfg = config()
    d = cfg.dims()
    out = {}
    for precision in ("fp64", "mixed"):
        with Simulation(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0, precision=precision,
                        capacity=int(4 * cfg.n_ppc * d.nx * d.ny)) as sim:
            sim.init_shock(cfg)
            sim.step(12)
            up, uf, np2, cc = sim.store(up=d.alloc_up())
            out[precision] = (up, np2, sim.energy())

    def by_pid(up, np2):
        cols = [np.concatenate([up[k, :np2[j, s], j, s] for s in range(2) for j in range(d.ny)]) for k in range(6)]
        o = np.argsort(cols[5].view(np.int64), kind="stable")
        return [c[o] for c in cols]

    a, b = by_pid(out["fp64"][0], out["fp64"][1]), by_pid(out["mixed"][0], out["mixed"][1])
    assert np.array_equal(out["fp64"][1].sum(axis=0), out["mixed"][1].sum(axis=0))  # same particles entered
    assert np.array_equal(a[5].view(np.int64), b[5].view(np.int64))
    errs = [np.max(np.abs(a[k] - b[k])) for k in range(2)] + [rel_err(b[k], a[k]) for k in range(2, 5)]
    de = abs(out["mixed"][2].sum() - out["fp64"][2].sum()) / out["fp64"][2].sum()
    print(f"\nshock with injection, mixed vs fp64 after 12 steps: x {errs[0]:.1e} y {errs[1]:.1e} u {max(errs[2:]):.1e} "
          f"energy {de:.1e}")
    assert max(errs) <= 1e-5 and de <= 1e-6


def expand_config():
    return ShockConfig(nx=96, ny=16, n_ppc=8, l_damp_ini=8.0, slack=4.0, seed=29, tracer_window=(30.0, 50.0), n_x_ini=40,
                       intvl_expand=1)


def oracle_expand_run(cfg, steps):
    """The oracle's shock steps over nxs..nxe (nxe = nxgs + n_x_ini, growing), each followed by the
    restated inject and, every intvl_expand steps, relocate (proj/shock/app.f90:110-125)."""
    from dataclasses import replace

    d = replace(cfg.dims(), nxe_act=cfg.dims().nxgs + cfg.n_x_ini)
    a = cfg.init_args()
    up0, uf, np2 = I.shock(d, *a[:-1], seed=a[-1])
    par = O.make_par(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0)
    up, cc = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cc, np2) == 0
    gp = up.copy(order="F")
    S = O.OracleState(d)
    for it in range(steps):
        status, _ = O.step(par, d, up, gp, uf, cc, np2, S)
        assert status == 0
        I.inject(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], cfg.delt)
        if (it + 1) % cfg.intvl_expand == 0:
            d = I.relocate(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7])
    return d, up, uf, np2, cc


def test_expanding_box_matches_oracle(gpu, tmp_path):
    """The expanding box in the resident FP64 step: nxe grows one cell per step from nxgs + 40 with
    n0 new particles per row in the new cell; counts per row, cell starts up to nxe and ids exact,
    positions, momenta and fields to 1e-11; a snapshot keeps nxe."""
    cfg = expand_config()
    d = cfg.dims()
    steps = 6
    d_o, up_o, uf_o, np2_o, cc_o = oracle_expand_run(cfg, steps)
    assert d_o.nxe == d.nxgs + cfg.n_x_ini + steps
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0, capacity=int(4 * cfg.n_ppc * d.nx * d.ny)) as sim:
        sim.init_shock(cfg)
        assert sim.nxe == d.nxgs + cfg.n_x_ini
        for _ in range(steps):
            sim.step(1)
        assert sim.nxe == d_o.nxe
        up, uf, np2, cc = sim.store(up=d.alloc_up())
        sim.write_snapshot(str(tmp_path), "expand", steps)
    nxa = d_o.nxe - d.nxgs + 1
    assert np.array_equal(np2, np2_o)
    assert np.array_equal(cc[:nxa], cc_o[:nxa])  # cell starts nxgs .. nxe
    assert np.array_equal(cc[nxa:], np.broadcast_to(np2, cc[nxa:].shape))  # empty cells past nxe: the row totals
    for isp in range(d.nsp):
        for j in range(d.ny):
            m = int(np2[j, isp])
            assert np.array_equal(up[5, :m, j, isp].view(np.int64), up_o[5, :m, j, isp].view(np.int64))
            for k in range(5):
                assert rel_err(up[k, :m, j, isp], up_o[k, :m, j, isp]) <= 1e-11, (isp, j, k)
    for k in range(6):
        assert rel_err(uf[k], uf_o[k]) <= 1e-11, k
    assert up[0, :int(np2.max())].max() < d_o.nxe  # no particle past the injection boundary
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0, capacity=int(4 * cfg.n_ppc * d.nx * d.ny)) as sim2:
        assert sim2.read_snapshot(str(tmp_path), "expand") == steps
        assert sim2.nxe == d_o.nxe


def test_expanding_box_mixed_tracks_fp64(gpu):
    cfg = expand_config()
    d = cfg.dims()
    out = {}
    for precision in ("fp64", "mixed"):
        with Simulation(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0, precision=precision,
                        capacity=int(4 * cfg.n_ppc * d.nx * d.ny)) as sim:
            sim.init_shock(cfg)
            sim.step(12)
            out[precision] = (sim.store(up=d.alloc_up()), sim.energy(), sim.nxe)
    assert out["fp64"][2] == out["mixed"][2] == d.nxgs + cfg.n_x_ini + 12

    def by_pid(up, np2):
        cols = [np.concatenate([up[k, :np2[j, s], j, s] for s in range(2) for j in range(d.ny)]) for k in range(6)]
        o = np.argsort(cols[5].view(np.int64), kind="stable")
        return [c[o] for c in cols]

    (upf, uff, np2f, ccf), (upm, ufm, np2m, ccm) = out["fp64"][0], out["mixed"][0]
    assert np.array_equal(np2f.sum(axis=0), np2m.sum(axis=0))
    a, b = by_pid(upf, np2f), by_pid(upm, np2m)
    assert np.array_equal(a[5].view(np.int64), b[5].view(np.int64))
    errs = [np.max(np.abs(a[k] - b[k])) for k in range(2)] + [rel_err(b[k], a[k]) for k in range(2, 5)]
    de = abs(out["mixed"][1].sum() - out["fp64"][1].sum()) / out["fp64"][1].sum()
    print(f"\nexpanding shock box, mixed vs fp64 after 12 steps: x {errs[0]:.1e} y {errs[1]:.1e} u {max(errs[2:]):.1e} energy {de:.1e}")
    assert max(errs) <= 1e-5 and de <= 1e-6


def test_expanding_box_dropin_matches_oracle(gpu):
    """The shock application's own loop (proj/shock/app.f90:110-125) through the drop-in module
    procedures with a growing nxe: particle__solv, boundary_shock__injection, field__fdtd_i,
    boundary_shock__particle_y and sort__bucket on the host arrays over nxs..nxe, the
    application's inject and relocate between the steps (its own code, restated in oracle/init.py,
    on the host arrays).  Against the oracle's same loop: row counts, the whole cumcnt (entries past
    nxe + 1 left as they were) and ids exact; positions, momenta and fields to 1e-11."""
    from dataclasses import replace

    from wumingpic2d_gb300 import api

    cfg = expand_config()
    steps = 4
    d_o, up_o, uf_o, np2_o, cc_o = oracle_expand_run(cfg, steps)
    d = replace(cfg.dims(), nxe_act=cfg.dims().nxgs + cfg.n_x_ini)
    a = cfg.init_args()
    up0, uf, np2 = I.shock(d, *a[:-1], seed=a[-1])
    par = O.make_par(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0)
    up, cc = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cc, np2) == 0
    gp = up.copy(order="F")
    api.init_all(d, cfg.delt, cfg.charge, cfg.mass, bc="shock")
    for it in range(steps):
        api.particle__solv(gp, up, uf, cc, d.nxs, d.nxe)
        api.boundary_shock__injection(gp, np2, d.nxs, d.nxe, cfg.u0)
        api.field__fdtd_i(uf, up, gp, cc, d.nxs, d.nxe, api.boundary_shock__dfield, api.boundary_shock__curre,
                          api.boundary_shock__phi)
        api.boundary_shock__particle_y(gp, np2)
        api.sort__bucket(up, gp, cc, np2, d.nxs, d.nxe)
        I.inject(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], cfg.delt)
        if (it + 1) % cfg.intvl_expand == 0:
            d = I.relocate(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7])
    assert d.nxe == d_o.nxe
    assert np.array_equal(np2, np2_o) and np.array_equal(cc, cc_o)
    for isp in range(d.nsp):
        for j in range(d.ny):
            m = int(np2[j, isp])
            assert np.array_equal(up[5, :m, j, isp].view(np.int64), up_o[5, :m, j, isp].view(np.int64))
            for k in range(5):
                assert rel_err(up[k, :m, j, isp], up_o[k, :m, j, isp]) <= 1e-11, (isp, j, k)
    for k in range(6):
        assert rel_err(uf[k], uf_o[k]) <= 1e-11, k
