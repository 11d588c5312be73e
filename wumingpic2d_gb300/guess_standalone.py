"""The learned CG guess on its own workload.

    python -m wumingpic2d_gb300.guess_standalone [--pairs 20000] [--out result.json]

System: the implicit field update of common/field.f90:319-461 on a 4096 x 4096 periodic grid,
the fields and currents of a seeded Weibel plasma (16 particles per cell per species, the
benchmark's plasma parameters), solved every step to a relative residual of 1e-10, once from the
previous step's dB (field.f90:355) and once from the network's guess (the better of the two per
component), from the same seeded state.  Reported: CG iterations per step (3 components) both ways,
time per step both ways, the network's inference time at 4096^2.

Training pairs: (E, B at step n; J at n+1/2) -> the converged dB, cut as crops of size x size cells
(random positions, periodic in y and, for the Weibel box, in x) from seeded runs of the 2048^2
Weibel workload (64 ppc per species) and of the 4096 x 2048 Harris-sheet workload (walls in x),
both on the mixed path with the CG at 1e-10.  Each crop is normalised per input group by the root
mean square over its whole grid, as the inference inside the step does; the loss covers the crop
interior only (a border of 8 cells, deeper than the network's 6-cell reach, is left out), so no
prediction that trains the network sees the crop's periodic padding.  Training runs the library's
BF16 tensor-core kernels (forward, input gradient and weight gradient on tcgen05) with Adam.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import cnn
from .harris import HarrisConfig
from .sim import Simulation
from .weibel import WeibelConfig

BORDER = 8


def collect(pairs: int, size: int, steps: int, every: int, seed: int, weibel=(2048, 64), harris=(4096, 2048)):
    """Crops from the Weibel run (weibel = (n, ppc): the 2048^2 x 64 ppc workload) and the Harris
    run (harris = (nx, ny): the 4096 x 2048 workload), half each."""
    rng = np.random.default_rng(seed)
    nsamp = len(range(0, steps, every))
    per = max(1, (pairs // 2 + nsamp - 1) // nsamp)  # crops per sampled step
    xs, ys, info = [], [], {}
    cfg = WeibelConfig(nx=weibel[0], ny=weibel[0], ppc=weibel[1], seed=seed + 1, slack=2.0)
    d = cfg.dims()
    t0 = time.perf_counter()
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="mixed", cg_err=1e-10) as sim:
        sim.init_weibel(cfg.ppc, cfg.v_drift, cfg.vth_e, cfg.vth_i, cfg.seed)
        x, y = cnn.capture_crops(sim, steps, every, per, size, rng, wrap_x=True)
    xs.append(x[:pairs // 2])
    ys.append(y[:pairs // 2])
    info["weibel"] = {"grid": [weibel[0], weibel[0]], "ppc": weibel[1], "steps": steps, "every": every, "crops": int(xs[-1].shape[0]),
                      "seconds": round(time.perf_counter() - t0, 1)}
    hc = HarrisConfig(nx=harris[0], ny=harris[1], seed=seed + 2, slack=2.0)
    hd = hc.dims()
    t0 = time.perf_counter()
    with Simulation(hd, hc.delt, hc.charge, hc.mass, precision="mixed", cg_err=1e-10, bc="reconnection") as sim:
        sim.init_harris(hc)
        x, y = cnn.capture_crops(sim, steps, every, per, size, rng, wrap_x=False)
    xs.append(x[:pairs - pairs // 2])
    ys.append(y[:pairs - pairs // 2])
    info["harris"] = {"grid": list(harris), "steps": steps, "every": every, "crops": int(xs[-1].shape[0]),
                      "seconds": round(time.perf_counter() - t0, 1)}
    return torch.cat(xs), torch.cat(ys), info


def measure(params, n: int, ppc: int, warm: int, steps: int, seed: int):
    """CG iterations and ms per step on the n x n periodic Weibel system, both guesses, from the
    same seeded state after `warm` steps."""
    cfg = WeibelConfig(nx=n, ny=n, ppc=ppc, seed=seed, slack=1.1)
    d = cfg.dims()
    out = {}
    for mode in ("previous_step", "learned"):
        with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="mixed", cg_err=1e-10) as sim:
            sim.init_weibel(cfg.ppc, cfg.v_drift, cfg.vth_e, cfg.vth_i, cfg.seed)
            out["particles"] = int(sim.info()[0])
            sim.step(warm)
            if mode == "learned":
                sim.set_guess(params)
                sim.step(1)
            sim.set_timing(True)
            its, ms, kt = [], 0.0, {}
            for _ in range(steps):
                ms += sim.step_timed(1)
                its.append(int(sim.cg_iters().sum()))
                for name, v in sim.kernel_times().items():  # the last step's kernels
                    kt[name] = kt.get(name, 0.0) + v
            sim.set_timing(False)
            r = {"cg_iters_per_step": round(float(np.mean(its)), 2), "ms_per_step": round(ms / steps, 3),
                 "cg_iterate_ms_per_step": round(kt.get("cg_iterate", 0.0) / steps, 3)}
            if mode == "learned":
                st = sim.guess_stats()
                r["guess_net_ms_per_step"] = round(kt.get("guess_net", 0.0) / steps, 3)
                r["initial_relative_residual"] = {
                    "network": np.sqrt(st[0:3] / np.maximum(st[9:12], 1e-300)).round(4).tolist(),
                    "previous_step": np.sqrt(st[3:6] / np.maximum(st[9:12], 1e-300)).round(4).tolist()}
            out[mode] = r
    return out


def run(pairs: int = 20000, size: int = 144, steps: int = 1000, every: int = 20, train_steps: int = 6000, batch: int = 16,
        lr: float = 3e-3, n: int = 4096, ppc: int = 16, warm: int = 100, measure_steps: int = 20, seed: int = 2024,
        weibel=(2048, 64), harris=(4096, 2048)) -> dict:
    t0 = time.perf_counter()
    x, y, info = collect(pairs, size, steps, every, seed, weibel, harris)
    t_data = time.perf_counter() - t0
    net = cnn.GuessNet(seed=seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = cnn.train(net, x, y, steps=train_steps, batch=batch, lr=lr, seed=seed + 3, log_every=max(1, train_steps // 6), border=BORDER)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    npairs = int(x.shape[0])
    del x, y
    torch.cuda.empty_cache()
    params = net.host_params()
    res = measure(params, n, ppc, warm, measure_steps, seed + 5)
    cg_ms_it = res["previous_step"]["cg_iterate_ms_per_step"] / max(res["previous_step"]["cg_iters_per_step"], 1e-9)
    saved = res["previous_step"]["cg_iters_per_step"] - res["learned"]["cg_iters_per_step"]
    return {
        "workload": f"implicit field system of a {n}x{n} periodic Weibel plasma ({ppc} ppc/species), CG to 1e-10, mixed path",
        "pairs": {"count": npairs, "crop": [size, size], "loss_border": BORDER, "sources": info, "seconds": round(t_data, 1)},
        "training": {"steps": train_steps, "batch": batch, "seconds": round(t_train, 1),
                     "pixels_per_s": train_steps * batch * size * size / t_train, "loss_history": hist,
                     "kernels": "forward, input gradient and weight gradient on tcgen05, Adam"},
        "cg": res,
        "break_even": {"cg_ms_per_iteration": round(cg_ms_it, 4), "iterations_saved_per_step": round(saved, 2),
                       "ms_saved_by_iterations": round(saved * cg_ms_it, 3),
                       "network_ms": res["learned"].get("guess_net_ms_per_step"),
                       "iterations_to_pay_for_the_network": round(res["learned"].get("guess_net_ms_per_step", 0.0) / max(cg_ms_it, 1e-9), 1)},
        "params": params,
    }


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--pairs", type=int, default=20000)
    p.add_argument("--size", type=int, default=144)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--every", type=int, default=20)
    p.add_argument("--train-steps", type=int, default=6000)
    p.add_argument("--n", type=int, default=4096)
    p.add_argument("--ppc", type=int, default=16)
    p.add_argument("--out", default=None)
    a = p.parse_args(argv)
    r = run(pairs=a.pairs, size=a.size, steps=a.steps, every=a.every, train_steps=a.train_steps, n=a.n, ppc=a.ppc)
    params = r.pop("params")
    print(json.dumps(r))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(r, f, indent=1)
        np.savez(a.out.rsplit(".", 1)[0] + "_params.npz", params=params)


if __name__ == "__main__":
    main()
