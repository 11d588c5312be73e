"""2000-step Weibel runs (256 x 256 cells, 16 particles per cell per species, cfl 0.5,
omega_pe dt 0.05) on the FP64 path and the mixed path from the same seeded state.

Stated bounds:
  * total energy: the FP64 run conserves it to 1e-3 relative over the 2000 steps (the implicit
    scheme with gfac = 0.501 is slightly dissipative and the plasma heats numerically); the mixed
    run's total energy stays within 1e-4 of the FP64 run's at every sample;
  * div E - 4 pi rho (quadratic-shape charge density) drifts from its initial value by at most
    1e-10 (FP64) and 1e-5 (mixed) of the electron charge density 4 pi |q_e| n0;
  * growth rate of the magnetic energy over the linear phase: mixed within 5 % of FP64, and both
    positive.
"""
import math

import numpy as np
import pytest

from wumingpic2d_gb300.diagnostics import energy_history, gauss_residual, growth_rate
from wumingpic2d_gb300.sim import Simulation
from wumingpic2d_gb300.weibel import WeibelConfig, weibel_particles

pytestmark = pytest.mark.gpu

NSTEPS, EVERY = 2000, 20


def _run(precision):
    cfg = WeibelConfig(nx=256, ny=256, ppc=16, seed=2024, slack=2.5)  # rows bunch up in the filaments
    d = cfg.dims()
    up, np2 = weibel_particles(cfg)
    uf = d.alloc_uf()
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision=precision) as sim:
        sim.load(up, uf, np2)
        up0, uf0, n0, _ = sim.store()
        g0 = gauss_residual(d, up0, uf0, n0, cfg.charge)
        steps, e = energy_history(sim, NSTEPS, EVERY)
        up1, uf1, n1, _ = sim.store()
        g1 = gauss_residual(d, up1, uf1, n1, cfg.charge)
        iters = sim.cg_iters()
    scale = 4 * math.pi * abs(cfg.charge[1]) * cfg.ppc
    t = steps * cfg.delt * cfg.omega_pe
    return dict(t=t, e=e, gauss=float(np.max(np.abs(g1 - g0)) / scale), iters=iters,
                np=int(n1.sum()), np0=int(n0.sum()))


@pytest.fixture(scope="module")
def runs():
    return {p: _run(p) for p in ("fp64", "mixed")}


def test_particle_count_is_conserved(gpu, runs):
    for r in runs.values():
        assert r["np"] == r["np0"]


def test_energy_history(gpu, runs):
    f, m = runs["fp64"], runs["mixed"]
    tot_f, tot_m = f["e"].sum(axis=1), m["e"].sum(axis=1)
    drift_f = np.max(np.abs(tot_f - tot_f[0])) / tot_f[0]
    drift_m = np.max(np.abs(tot_m - tot_m[0])) / tot_m[0]
    diff = np.max(np.abs(tot_m - tot_f)) / tot_f[0]
    print(f"\nenergy over {NSTEPS} steps: fp64 drift {drift_f:.2e}, mixed drift {drift_m:.2e}, "
          f"mixed - fp64 {diff:.2e}; final E_B/E_tot fp64 {f['e'][-1, -1] / tot_f[-1]:.3e} "
          f"mixed {m['e'][-1, -1] / tot_m[-1]:.3e}; cg iters last step {f['iters']} {m['iters']}")
    assert drift_f <= 1e-3
    assert diff <= 1e-4


def test_gauss_law(gpu, runs):
    print(f"\ngauss drift over {NSTEPS} steps: fp64 {runs['fp64']['gauss']:.2e} mixed {runs['mixed']['gauss']:.2e}")
    assert runs["fp64"]["gauss"] <= 1e-10
    assert runs["mixed"]["gauss"] <= 1e-5


def test_magnetic_growth_rate(gpu, runs):
    gf = growth_rate(runs["fp64"]["t"], runs["fp64"]["e"][:, -1])
    gm = growth_rate(runs["mixed"]["t"], runs["mixed"]["e"][:, -1])
    print(f"\nmagnetic growth rate (omega_pe): fp64 {gf[0]:.4f} over t = {gf[1]:.1f}..{gf[2]:.1f}, "
          f"mixed {gm[0]:.4f} over t = {gm[1]:.1f}..{gm[2]:.1f}")
    assert gf[0] > 0 and gm[0] > 0
    assert abs(gm[0] - gf[0]) <= 0.05 * gf[0]
