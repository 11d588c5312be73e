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
