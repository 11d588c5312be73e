"""A long run of the shock workload, timed in windows as the downstream pileup forms.

    python -m wumingpic2d_gb300.shock_run [--steps 5000] [--every 500] [--window 20] [--out run.json]

The shock application (proj/shock/app.f90:110-166): 16384 x 1024 cells, 32 ppc per species upstream,
u0 = -0.1c, mi/me = 100, sigma_e = 0.01, a reflecting wall at x = 0 and particles injected every
step at x = nxe, on the mixed path (the box at full size from the start).  Every `every` steps the
run times `window` steps with CUDA events and reads the cell counts (cumcnt) and row counts (np2):

  density profile   particles per cell averaged over the rows, in 32-cell bins from the wall, and
                    the largest bin against the upstream mean (the pileup);
  tile imbalance    particles in the most loaded 32-cell tile of a row (one push CTA) against the
                    mean tile, and the trip count of the push's busiest warp (4 lanes per cell,
                    8 cells per warp: max over its cells of ceil(n / 4)) against the mean cell's;
  row skew          the largest np2 against the mean (the rebin's rows);
  ms per step, particle count, CG iterations.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from ._native import check, lib
from .shock import ShockConfig
from .sim import Simulation

TILE = 32


def counts(sim):
    """Per-cell counts [nsp][ny][nx] and np2 [nsp][ny] from the resident state (no particle copy)."""
    d = sim.dims
    np2 = d.alloc_np2()
    cc = d.alloc_cumcnt()
    check(lib().wm_sim_store(sim._h, None, None, np2.ctypes.data, cc.ctypes.data), "wm_sim_store")
    cum = np.asarray(cc).reshape((d.nx + 1, d.ny, d.nsp), order="F")
    cells = np.diff(cum, axis=0)  # (nx, ny, nsp)
    return np.transpose(cells, (2, 1, 0)), np.asarray(np2).reshape((d.ny, d.nsp), order="F").T


def stats(cells, np2, n0):
    nsp, ny, nx = cells.shape
    prof = cells.sum(axis=0).mean(axis=0)  # particles per cell (both species), mean over rows
    nb = nx // TILE
    bins = prof[:nb * TILE].reshape(nb, TILE).mean(axis=1)
    upstream = float(np.median(bins[nb // 2:]))
    tiles = cells[..., :nb * TILE].reshape(nsp, ny, nb, TILE).sum(axis=3)
    warps = np.ceil(cells[..., :nb * TILE].reshape(nsp, ny, nb * 4, 8) / 4.0).max(axis=3)
    mean_cell_trip = float(np.mean(np.ceil(cells / 4.0)))
    return {"upstream_ppc_both_species": round(upstream, 2),
            "pileup": round(float(bins.max()) / upstream, 3),
            "pileup_bin": int(np.argmax(bins)),
            "cells_above_2x_upstream": int(np.sum(prof > 2 * upstream)),
            "bins_near_wall": [round(float(b) / upstream, 3) for b in bins[:16]],
            "tile_max_over_mean": round(float(tiles.max()) / float(tiles.mean()), 3),
            "warp_trip_max_over_mean_cell": round(float(warps.max()) / mean_cell_trip, 3),
            "warp_trip_mean_over_mean_cell": round(float(warps.mean()) / mean_cell_trip, 3),
            "row_skew": round(float(np2.max()) / float(np2.mean()), 4)}


def run(steps=5000, every=500, window=20, nx=16384, ny=1024, ppc=32, seed=13):
    cfg = ShockConfig(nx=nx, ny=ny, n_ppc=ppc, l_damp_ini=64.0, slack=1.1, seed=seed)
    d = cfg.dims()
    n0 = 2 * cfg.n_ppc * (d.nx - 2) * d.ny
    out = {"workload": f"shock {cfg.nx}x{cfg.ny}, {cfg.n_ppc} ppc/species upstream, u0 {cfg.u0:g}c, mi/me {cfg.mass_ratio:g}, "
                       f"sigma_e {cfg.sigma_e:g}, omega_pe {cfg.omega_pe:g}, wall + injection, mixed path", "checkpoints": []}
    t_start = time.perf_counter()
    ends = sorted(set([window] + list(range(every, steps + 1, every)) + [steps]))  # each checkpoint times the window ending there
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="mixed", bc="shock", u0=cfg.u0,
                    capacity=int(n0 * 1.3)) as sim:
        sim.init_shock(cfg)
        it = 0
        for end in ends:
            if end - window > it:
                sim.step(end - window - it)
                it = end - window
            sim.set_timing(True)
            ms = sim.step_timed(end - it)
            kt = sim.kernel_times()
            sim.set_timing(False)
            nt, it = end - it, end
            cells, np2 = counts(sim)
            rec = {"step": it, "ms_per_step": round(ms / nt, 3), "particles": int(sim.info()[0]),
                   "push_ms_per_step": round(kt.get("push_deposit", 0.0) / nt, 3),
                   "cg_iters": sim.cg_iters().tolist(), **stats(cells, np2, cfg.n_ppc)}
            out["checkpoints"].append(rec)
            print(json.dumps(rec), flush=True)
    out["seconds"] = round(time.perf_counter() - t_start, 1)
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--steps", type=int, default=5000)
    p.add_argument("--every", type=int, default=500)
    p.add_argument("--window", type=int, default=20)
    p.add_argument("--nx", type=int, default=16384)
    p.add_argument("--ny", type=int, default=1024)
    p.add_argument("--out", default=None)
    a = p.parse_args(argv)
    r = run(a.steps, a.every, a.window, a.nx, a.ny)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(r, f, indent=1)


if __name__ == "__main__":
    main()
