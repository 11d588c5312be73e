"""The learned CG initial guess trained on the reconnection application's Harris-sheet pairs
(wumingpic2d_gb300/guess_harris.npz): on a held-out seed with walls in x it never costs CG
iterations, saves some at the 1e-10 tolerance of the reconnection workload, and leaves the answer
unchanged beyond the solver tolerance."""
from pathlib import Path

import numpy as np
import pytest

import wumingpic2d_gb300
from wumingpic2d_gb300.harris import HarrisConfig
from wumingpic2d_gb300.sim import Simulation

pytestmark = pytest.mark.gpu


def test_harris_guess_saves_cg_iterations(gpu):
    params = np.load(Path(wumingpic2d_gb300.__file__).with_name("guess_harris.npz"))["params"]
    cfg = HarrisConfig(nx=256, ny=128, seed=404, slack=2.0)
    d = cfg.dims()
    runs = {}
    for mode in ("prev", "net"):
        with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="mixed", cg_err=1e-10, bc="reconnection") as sim:
            sim.init_harris(cfg)
            sim.step(20)
            if mode == "net":
                sim.set_guess(params)
            its = []
            for _ in range(30):
                sim.step(1)
                its.append(int(sim.cg_iters().sum()))
            runs[mode] = (np.array(its), sim.energy())
    print(f"\nHarris sheet, CG to 1e-10: iterations per step (3 components): previous-step guess "
          f"{runs['prev'][0].mean():.2f}, learned guess {runs['net'][0].mean():.2f}")
    assert runs["net"][0].mean() < runs["prev"][0].mean()
    assert abs(runs["net"][1].sum() - runs["prev"][1].sum()) <= 1e-8 * runs["prev"][1].sum()
