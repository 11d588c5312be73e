"""Long-run physics check of the Weibel workload on both arithmetic paths.

    python -m wumingpic2d_gb300.validate [--nx 2048 --ny 2048 --ppc 64 --steps 2000 --every 20]

The same seeded state (generated on the GPU) runs on the FP64 path and on the mixed path; for
each, the energies of proj/weibel/app.f90:507-541 every `every` steps, the growth rate of the
magnetic energy over the linear phase, and the drift of div E - 4 pi rho (second-order shape,
which the Esirkepov deposit conserves exactly) between the first and the last step on a strip of
rows.  Prints one JSON object (and writes it to --out): per path the total-energy drift and the
history, and the mixed path against the FP64 one (largest relative difference of the total energy
at the samples, ratio of the growth rates).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from .diagnostics import div_e, growth_rate
from .sim import Simulation
from .weibel import WeibelConfig


def strip_gauss(d, up, uf, np2, q, j0: int, k: int) -> np.ndarray:
    """div E - 4 pi rho on interior rows j0 .. j0+k-1 (0-based), (nx, k): rho with the deposit's
    quadratic shape from the particle rows j0-1 .. j0+k (a particle of row r reaches r-1 .. r+1)."""
    rho = np.zeros((d.nx, k))
    for isp in range(d.nsp):
        for jr in range(j0 - 1, j0 + k + 1):
            jj = jr % d.ny
            n = int(np2[jj, isp])
            x, y = up[0, :n, jj, isp], up[1, :n, jj, isp]
            i, j = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64)
            hx, hy = x - 0.5 - i, y - 0.5 - j
            sx = (0.5 * (0.5 - hx) ** 2, 0.75 - hx ** 2, 0.5 * (0.5 + hx) ** 2)
            sy = (0.5 * (0.5 - hy) ** 2, 0.75 - hy ** 2, 0.5 * (0.5 + hy) ** 2)
            for b in range(3):
                rows = (j + b - 1 - d.nygs) % d.ny - j0
                rows = np.where(rows < 0, rows + d.ny, rows)
                keep = rows < k
                for a in range(3):
                    cols = (i + a - 1 - d.nxgs) % d.nx
                    w = (q[isp] * sx[a] * sy[b])[keep]
                    rho += np.bincount(cols[keep] * k + rows[keep], weights=w, minlength=d.nx * k).reshape(d.nx, k)
    return div_e(d, uf)[:, j0:j0 + k] - 4.0 * np.pi * rho


def run(cfg: WeibelConfig, precision: str, steps: int, every: int, strip=(0, 16)):
    d = cfg.dims()
    out = {"precision": precision}
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision=precision) as sim:
        t0 = time.perf_counter()
        sim.init_weibel(cfg.ppc, cfg.v_drift, cfg.vth_e, cfg.vth_i, cfg.seed)
        up, uf, np2, _ = sim.store(up=d.alloc_up())
        g0 = strip_gauss(d, up, uf, np2, cfg.charge, *strip)
        del up
        hist, t = [sim.energy()], [0]
        done = 0
        while done < steps:
            n = min(every, steps - done)
            sim.step(n)
            done += n
            hist.append(sim.energy())
            t.append(done)
        up, uf, np2, _ = sim.store(up=d.alloc_up())
        g1 = strip_gauss(d, up, uf, np2, cfg.charge, *strip)
        del up
        out["seconds"] = round(time.perf_counter() - t0, 1)
        out["cg_iters_last_step"] = sim.cg_iters().tolist()
    hist = np.asarray(hist)
    tot = hist.sum(axis=1)
    scale = 4 * math.pi * abs(cfg.charge[1]) * cfg.ppc  # electron charge density 4 pi |q_e| n0
    gamma, t_lo, t_hi = growth_rate(np.asarray(t) * cfg.delt, hist[:, -1])
    out.update({
        "steps": steps, "every": every,
        "total_energy_first": float(tot[0]), "total_energy_last": float(tot[-1]),
        "total_energy_max_rel_change": float(np.max(np.abs(tot - tot[0])) / tot[0]),
        "magnetic_energy_last": float(hist[-1, -1]),
        "growth_rate": gamma, "growth_window": [t_lo, t_hi],
        "gauss_drift_rel": float(np.max(np.abs(g1 - g0)) / scale),
        "gauss_strip_rows": list(strip),
        "energy_history": {"step": [int(v) for v in t], "columns": "kinetic per species, electric, magnetic",
                           "values": hist.tolist()},
    })
    return out, t, hist


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--nx", type=int, default=2048)
    p.add_argument("--ny", type=int, default=2048)
    p.add_argument("--ppc", type=int, default=64)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--every", type=int, default=20)
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--paths", default="fp64,mixed")
    p.add_argument("--out", default=None, help="also write the result object to this JSON file")
    args = p.parse_args(argv)
    cfg = WeibelConfig(nx=args.nx, ny=args.ny, ppc=args.ppc, seed=args.seed, slack=3.0)  # rows bunch up in the filaments
    res, hists = {"workload": f"Weibel {args.nx}x{args.ny}, {args.ppc} ppc/species, {args.steps} steps"}, {}
    for path in args.paths.split(","):
        r, t, h = run(cfg, path, args.steps, args.every)
        res[path] = r
        hists[path] = h
        print(json.dumps({path: r}), flush=True)
    if "fp64" in hists and "mixed" in hists:
        a, b = hists["fp64"].sum(axis=1), hists["mixed"].sum(axis=1)
        res["mixed_vs_fp64"] = {
            "total_energy_max_rel_diff": float(np.max(np.abs(b - a)) / a[0]),
            "magnetic_energy_last_ratio": float(hists["mixed"][-1, -1] / hists["fp64"][-1, -1]),
            "growth_rate_ratio": float(res["mixed"]["growth_rate"] / res["fp64"]["growth_rate"]),
        }
    print(json.dumps(res), flush=True)
    if args.out:
        res["command"] = "python -m wumingpic2d_gb300.validate " + " ".join(argv if argv is not None else __import__("sys").argv[1:])
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
