"""Train the learned CG initial guess on the GPU and save its parameters.

    python -m wumingpic2d_gb300.train_guess [--app weibel|harris] [--out ...npz]

Pairs (E, B at time n; J at n+1/2) -> converged dB come from seeded FP64 runs on the resident
simulation.  weibel: a 128 x 128 box with the benchmark's plasma parameters (whose length scales
-- the skin depth in cells, c dt/dx -- do not depend on the box size), one run sampled every step
over its first steps and one sampled every 10 steps over a long run that reaches the nonlinear
phase.  harris: the reconnection application's Harris sheet (walls in x) on a 256 x 128 box,
generated on the GPU (wm_sim_init_harris), sampled the same way.  Training runs the library's
BF16 tensor-core kernels (cnn.Trainer).  A held-out seed then measures CG iterations per step
from the previous step's dB and from the network's guess.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import cnn
from .sim import Simulation
from .weibel import WeibelConfig, weibel_particles

DEFAULT_OUT = {"weibel": Path(__file__).resolve().parent / "guess_weibel.npz",
               "harris": Path(__file__).resolve().parent / "guess_harris.npz"}
APP = {"name": "weibel"}


def _sim(seed, nx, ny, ppc, cg_err=1e-6):
    if APP["name"] == "harris":
        from .harris import HarrisConfig
        cfg = HarrisConfig(nx=nx, ny=ny, seed=seed, slack=2.0)
        d = cfg.dims()
        sim = Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="fp64", cg_err=cg_err, bc="reconnection")
        sim.init_harris(cfg)
        return sim
    cfg = WeibelConfig(nx=nx, ny=ny, ppc=ppc, seed=seed, slack=2.5)
    d = cfg.dims()
    up, np2 = weibel_particles(cfg)
    sim = Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="fp64", cg_err=cg_err)
    sim.load(up, d.alloc_uf(), np2)
    return sim


def collect(nx, ny, ppc, seeds_early, seeds_long, early_steps, long_steps, long_every):
    xs, ys = [], []
    for s in seeds_early:
        with _sim(s, nx, ny, ppc) as sim:
            a, b = cnn.capture_pairs(sim, early_steps, every=1)
        xs.append(a)
        ys.append(b)
    for s in seeds_long:
        with _sim(s, nx, ny, ppc) as sim:
            a, b = cnn.capture_pairs(sim, long_steps, every=long_every)
        xs.append(a)
        ys.append(b)
    return np.concatenate(xs), np.concatenate(ys)


def cg_iterations(params, seed, nx, ny, ppc, cg_err, warm, steps):
    """Mean CG iterations per step (3 components) without and with the guess."""
    out = {}
    for mode in ("previous_step", "learned"):
        with _sim(seed, nx, ny, ppc, cg_err) as sim:
            sim.step(warm)
            if mode == "learned":
                sim.set_guess(params)
            its = []
            for _ in range(steps):
                sim.step(1)
                its.append(int(sim.cg_iters().sum()))
        out[mode] = float(np.mean(its))
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--app", choices=["weibel", "harris"], default="weibel")
    p.add_argument("--out", type=Path, default=None)
    p.add_argument("--nx", type=int, default=None)
    p.add_argument("--ny", type=int, default=128)
    p.add_argument("--ppc", type=int, default=16)
    p.add_argument("--early-steps", type=int, default=200)
    p.add_argument("--long-steps", type=int, default=2000)
    p.add_argument("--long-every", type=int, default=10)
    p.add_argument("--train-steps", type=int, default=8000)
    p.add_argument("--batch", type=int, default=16)
    p.add_argument("--lr", type=float, default=3e-3)
    p.add_argument("--seed", type=int, default=7)
    args = p.parse_args(argv)
    APP["name"] = args.app
    args.out = args.out or DEFAULT_OUT[args.app]
    args.nx = args.nx or (256 if args.app == "harris" else 128)

    t0 = time.perf_counter()
    xs, ys = collect(args.nx, args.ny, args.ppc, [101], [102], args.early_steps, args.long_steps, args.long_every)
    t_data = time.perf_counter() - t0
    xn, yn = cnn.normalise(xs, ys)
    x, y = cnn.to_device(xn, yn)
    net = cnn.GuessNet(seed=args.seed)
    t0 = time.perf_counter()
    hist = cnn.train(net, x, y, steps=args.train_steps, batch=args.batch, lr=args.lr, seed=args.seed + 1, log_every=1000)
    t_train = time.perf_counter() - t0
    params = net.host_params()
    evals = {str(e): cg_iterations(params, 103, args.nx, args.ny, args.ppc, e, 20, 40) for e in (1e-6, 1e-10)}
    meta = {"app": args.app, "samples": int(xs.shape[0]), "grid": [args.nx, args.ny], "ppc": args.ppc, "train_steps": args.train_steps,
            "batch": args.batch, "lr": args.lr, "loss_history": hist, "seconds_data": round(t_data, 1),
            "seconds_train": round(t_train, 1), "cg_iterations_held_out": evals}
    args.out.parent.mkdir(parents=True, exist_ok=True)
    np.savez(args.out, params=params, meta=json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
