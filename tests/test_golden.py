"""Golden vectors produced by the reference's own code (tests/golden/make_golden.py).

CPU: the hand restatement reproduces every golden array bit for bit (one thread).
GPU: the sm_103a path reproduces the integer and permutation results exactly and the FP64
results to a normwise relative error of 1e-12 per component.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rel_err
from wumingpic2d_gb300.layout import Dims

GOLD = Path(__file__).resolve().parent / "golden" / "golden_weibel_16x12.npz"
TOL = 1e-12


@pytest.fixture(scope="module")
def g():
    z = np.load(GOLD)
    return {k: (np.asfortranarray(z[k]) if z[k].ndim > 1 else z[k]) for k in z.files}


def _setup(g):
    d = Dims(nx=int(g["nx"]), ny=int(g["ny"]), np=int(g["np"]), nsp=int(g["nsp"]))
    par = O.make_par(d, float(g["delt"]), g["q"], g["r"])
    return d, par


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def cp(a):
    return np.array(a, order="F", copy=True)


# ------------------------------------------------------------------------ CPU
def test_oracle_reproduces_reference_routines(g):
    O.set_threads(1)
    d, par = _setup(g)
    gp = cp(g["in_gp"])
    O.particle_solv(par, d, gp, g["in_up"], g["in_uf"], g["in_cumcnt"])
    assert np.array_equal(bits(gp), bits(g["push_gp"]))
    acc = cp(g["in_gp"])
    O.mom_accl(par, d, acc, g["in_up"], g["in_uf"], g["in_cumcnt"])
    assert np.array_equal(bits(acc), bits(g["accl_gp"]))
    S = O.OracleState(d)
    S.df[:] = g["in_df"]
    uf = cp(g["in_uf"])
    assert O.field_fdtd_i(par, d, uf, g["in_up"], gp, g["in_cumcnt"], S)[0] == 0
    for a, k in ((uf, "fdtd_uf"), (S.df, "fdtd_df"), (S.uj, "fdtd_uj"), (S.gkl, "fdtd_gkl")):
        assert np.array_equal(bits(a), bits(g[k])), k
    np2 = cp(g["in_np2"])
    O.bc_particle_x(par, d, gp, np2)
    assert np.array_equal(bits(gp), bits(g["px_gp"]))
    assert O.bc_particle_y(par, d, gp, np2) == 0
    assert np.array_equal(np2, g["py_np2"]) and np.array_equal(bits(gp), bits(g["py_gp"]))
    out, cum = cp(g["in_up"]), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, out, gp, cum, np2) == 0
    assert np.array_equal(cum, g["sort_cumcnt"]) and np.array_equal(bits(out), bits(g["sort_up"]))
    mom = d.alloc_mom()
    O.mom_nvt(par, d, mom, g["in_up"], g["in_np2"])
    assert np.array_equal(bits(mom), bits(g["nvt_mom"]))
    O.bc_mom(par, d, mom)
    assert np.array_equal(bits(mom), bits(g["bcmom_mom"]))


def test_oracle_reproduces_reference_run(g):
    O.set_threads(1)
    d, par = _setup(g)
    up, uf, cum, np2 = cp(g["run_in_up"]), cp(g["run_in_uf"]), cp(g["run_in_cumcnt"]), cp(g["run_in_np2"])
    gp = cp(up)
    S = O.OracleState(d)
    for _ in range(5):
        assert O.step(par, d, up, gp, uf, cum, np2, S)[0] == 0
    assert np.array_equal(np2, g["run_np2"]) and np.array_equal(cum, g["run_cumcnt"])
    assert np.array_equal(bits(up), bits(g["run_up"]))
    assert np.array_equal(bits(uf), bits(g["run_uf"]))
    assert np.array_equal(bits(S.df), bits(g["run_df"]))


# ------------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_gpu_reproduces_reference_routines(gpu, g):
    from wumingpic2d_gb300 import api

    d, par = _setup(g)
    api.init_all(d, float(g["delt"]), g["q"], g["r"])
    gp = cp(g["in_gp"])
    api.particle__solv(gp, g["in_up"], g["in_uf"], g["in_cumcnt"], d.nxs, d.nxe)
    for k in range(5):
        assert rel_err(gp[k], g["push_gp"][k]) <= TOL
    assert np.array_equal(bits(gp[5]), bits(g["push_gp"][5]))
    gp = cp(g["push_gp"])
    api.field__set_work(cp(g["in_df"]))
    uf = cp(g["in_uf"])
    api.field__fdtd_i(uf, g["in_up"], gp, g["in_cumcnt"], d.nxs, d.nxe)
    for k in range(6):
        assert rel_err(uf[k], g["fdtd_uf"][k]) <= TOL
    np2 = cp(g["in_np2"])
    api.boundary_periodic__particle_x(gp, np2)
    assert np.array_equal(bits(gp), bits(g["px_gp"]))
    api.boundary_periodic__particle_y(gp, np2)
    assert np.array_equal(np2, g["py_np2"]) and np.array_equal(bits(gp), bits(g["py_gp"]))
    out, cum = cp(g["in_up"]), d.alloc_cumcnt()
    api.sort__bucket(out, gp, cum, np2, d.nxs, d.nxe)
    assert np.array_equal(cum, g["sort_cumcnt"]) and np.array_equal(bits(out), bits(g["sort_up"]))
    mom = d.alloc_mom()
    api.mom_calc__nvt(mom, g["in_up"], g["in_np2"])
    api.boundary_periodic__mom(mom)
    for k in range(7):
        assert rel_err(mom[k], g["bcmom_mom"][k]) <= TOL


@pytest.mark.gpu
def test_gpu_reproduces_reference_run(gpu, g):
    from wumingpic2d_gb300.sim import Simulation

    d, _ = _setup(g)
    with Simulation(d, float(g["delt"]), g["q"], g["r"]) as sim:
        sim.load(cp(g["run_in_up"]), cp(g["run_in_uf"]), cp(g["run_in_np2"]))
        sim.step(5)
        up, uf, np2, cum = sim.store()
    assert np.array_equal(np2, g["run_np2"]) and np.array_equal(cum, g["run_cumcnt"])
    for isp in range(d.nsp):
        for j in range(d.ny):
            n = np2[j, isp]
            assert np.array_equal(bits(up[5, :n, j, isp]), bits(g["run_up"][5, :n, j, isp]))
    for k in range(5):
        a = np.concatenate([up[k, :np2[j, s], j, s] for s in range(d.nsp) for j in range(d.ny)])
        b = np.concatenate([g["run_up"][k, :np2[j, s], j, s] for s in range(d.nsp) for j in range(d.ny)])
        assert rel_err(a, b) <= 1e-11
    for k in range(6):
        assert rel_err(uf[k], g["run_uf"][k]) <= 1e-11
