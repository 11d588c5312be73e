#!/usr/bin/env python
"""Particle-updates per second of the WumingPIC2D time step on one GB300.

Workload (default): the 2048 x 2048 periodic Weibel plasma, 64 particles per cell per
species (5.37e8 particles), c dt/dx = 0.5, omega_pe dt = 0.05, mi/me = 25, electron beams
at +/-0.3c with vth_e = 0.05c, vth_i = 0.01c, fields start at zero; seeded synthetic state.
One step = push + Esirkepov deposit + implicit field solve (CG) + periodic particle
boundaries + per-cell counting sort (proj/weibel/app.f90:102-107).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value    particle-updates/s of the mixed-precision path (FP32 particles, FP64 fields and CG) with
         the state resident in HBM, K steps timed with CUDA events; the FP64 path is timed the same
         way and reported under "fp64_path".
e2e      the same metric through the host-buffer entry point (wm_sim_step_host): every step
         copies the reference-layout state in from pinned host memory and back out.
roofline the dominant particle kernel's algorithmic bytes per launch / its event time.
cpu_baseline  the CPU restatement of the reference step (oracle/, OpenMP on every host core)
         on a bounded sample of the same workload.
learned_guess, reconnection_cg, shock, cnn
         the Weibel loop with the learned CG guess; the reconnection workload (Harris sheet
         4096 x 2048, CG to 1e-10) with and without its learned guess; the shock workload
         (16384 x 1024, 32 ppc, injection every step), all on the mixed path; the guess's network
         alone (inference on a 4096^2 image, training steps on 8 x 512^2).
--impl reference times that CPU restatement alone (the reference is Fortran + MPI and no
Fortran compiler exists on this machine).
Under torchrun (N > 1) each rank runs an independent replica on its own GPU (the path does
not shard: replicas only); rank 0 prints the line, value = total over ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particle-updates/s, full PIC step (Weibel 2048^2, 64 ppc/species)"
UNIT = "particle-updates/s"
L2_BYTES = 129e6


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="both", choices=["both", "fp64", "mixed"],
                   help="both: the mixed path is the headline value, the FP64 path is timed beside it")
    p.add_argument("--nx", type=int, default=2048)
    p.add_argument("--ny", type=int, default=2048)
    p.add_argument("--ppc", type=int, default=64)
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--cpu-rows", type=int, default=64, help="rows of the CPU sample strip")
    p.add_argument("--guess", default=os.path.join(ROOT, "wumingpic2d_gb300", "guess_weibel.npz"),
                   help="trained CG-guess network (wumingpic2d_gb300.train_guess); 'none' skips the learned-guess leg")
    p.add_argument("--cpu-steps", type=int, default=2)
    p.add_argument("--reconnection-guess", default=os.path.join(ROOT, "wumingpic2d_gb300", "guess_harris.npz"),
                   help="network trained on Harris-sheet pairs for the reconnection CG leg; 'none' skips the leg")
    p.add_argument("--reconnection-steps", type=int, default=10)
    p.add_argument("--shock-steps", type=int, default=5, help="steps of the shock leg (0 skips it)")
    p.add_argument("--rebin", default="permute", choices=["permute", "move"],
                   help="mixed path: the next push reads through the new order (permute) or the particles are moved every step")
    p.add_argument("--cnn-steps", type=int, default=5, help="repetitions of the network-alone leg (0 skips it)")
    p.add_argument("--standalone-pairs", type=int, default=20000,
                   help="training crops of the learned guess's standalone 4096^2 workload (0 skips the leg)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


# ------------------------------------------------------------------ distributed
class Dist:
    def __init__(self, n):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    """nvidia-smi samples every 50 ms, started before the warm-up (its start-up takes longer than a
    short timed region); only the samples taken between mark_start() and mark_stop() count."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []  # (host time, line)
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_stop(self):
        self.t1 = time.perf_counter()

    def stop(self):
        if self.t1 is None:
            self.mark_stop()
        time.sleep(0.06)  # the sample that covers the end of the region
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0 = self.t0 if self.t0 is not None else -1.0
        for tl, ln in self.lines:
            if not (t0 <= tl <= self.t1 + 0.06):
                continue
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic():
    """DRAM bytes per particle of the particle kernels from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ CPU baseline
def cpu_cores():
    """Host cores this process may run on (its affinity mask, which the container sets) and the
    cores the host has online."""
    try:
        allowed = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        allowed = os.cpu_count() or 1
    online = None
    try:
        with open("/sys/devices/system/cpu/online") as f:
            online = sum(int(b) - int(a) + 1 for a, _, b in (r.partition("-") if "-" in r else (r, "-", r)
                                                             for r in f.read().strip().split(",")))
    except (OSError, ValueError):
        pass
    return {"allowed": allowed, "host_online": online}


def cpu_sample(args, steps: int):
    """The CPU restatement (OpenMP, every host core) on a strip of the workload."""
    from oracle import init as I
    from oracle import oracle as O
    from wumingpic2d_gb300.weibel import WeibelConfig

    cfg = WeibelConfig(nx=args.nx, ny=args.cpu_rows, ppc=args.ppc, seed=args.seed + 7, slack=1.2)
    d = cfg.dims()
    threads = cpu_cores()["allowed"]
    O.set_threads(threads)
    par = O.make_par(d, cfg.delt, cfg.charge, cfg.mass)
    up0, _, np2 = I.weibel(d, cfg.ppc, cfg.v_drift, cfg.vth_e, cfg.vth_i, cfg.seed)  # the GPU generator's state
    up, cum = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cum, np2) == 0
    del up0
    gp, uf, st = up.copy(order="F"), d.alloc_uf(), O.OracleState(d)
    npart = int(np2.sum())
    O.step(par, d, up, gp, uf, cum, np2, st)  # warm caches and thread pool
    t0 = time.perf_counter()
    for _ in range(steps):
        s, _ = O.step(par, d, up, gp, uf, cum, np2, st)
        assert s == 0
    dt = time.perf_counter() - t0
    sample = (f"{args.nx}x{args.cpu_rows}-cell periodic strip of the workload, {args.ppc} ppc/species "
              f"({npart} particles), {steps} steps, OMP_NUM_THREADS={threads}")
    return npart * steps / dt, threads, sample


# ---------------------------------------------------------------------- GB300 arm
def make_state(args, dist: Dist):
    """The workload's parameters; the particles are generated on the GPU (wm_sim_init_weibel)."""
    from wumingpic2d_gb300.weibel import WeibelConfig

    return WeibelConfig(nx=args.nx, ny=args.ny, ppc=args.ppc, seed=args.seed + dist.rank, slack=1.1)


def reconnection_cg(args):
    """The reconnection workload (Harris sheet, walls in x, 4096 x 2048 cells, 64 ppc in the sheet
    centre, mixed path) with the CG tolerance at 1e-10: CG iterations per step (3 components) and
    time per step from the previous step's dB and from the network trained on Harris pairs."""
    from wumingpic2d_gb300.harris import HarrisConfig
    from wumingpic2d_gb300.sim import Simulation

    if args.reconnection_guess == "none" or not os.path.exists(args.reconnection_guess):
        return None
    params = np.load(args.reconnection_guess)["params"]
    cfg = HarrisConfig(nx=4096, ny=2048, seed=args.seed + 11, slack=1.3)
    d = cfg.dims()
    out = {"workload": f"Harris sheet {cfg.nx}x{cfg.ny} (walls in x, periodic y), nbg {cfg.nbg} + ncs {cfg.ncs} ppc/species, "
                       f"mi/me {cfg.mass_ratio:g}, Te/Ti {cfg.rtemp:g}, cg_tol 1e-10, mixed path",
           "steps": args.reconnection_steps, "weights": os.path.relpath(args.reconnection_guess, ROOT)}
    for mode in ("previous_step", "learned"):
        with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="mixed", cg_err=1e-10, bc="reconnection") as sim:
            sim.init_harris(cfg)
            out["particles"] = sim.info()[0]
            sim.step(3)
            if mode == "learned":
                sim.set_guess(params)
                sim.step(1)
            its, ms = [], 0.0
            for _ in range(args.reconnection_steps):
                ms += sim.step_timed(1)
                its.append(int(sim.cg_iters().sum()))
            out[mode] = {"cg_iters_per_step": round(float(np.mean(its)), 2), "ms_per_step": round(ms / args.reconnection_steps, 3)}
    return out


def shock_leg(args):
    """The shock workload (16384 x 1024 cells, 32 ppc per species upstream, u0 = -0.1c, mi/me 100,
    sigma_e 0.01, reflecting wall and injection boundary, particles injected every step; the box
    at full size), mixed path: particle-updates/s over the first steps of the run, and the
    particles injected meanwhile."""
    from wumingpic2d_gb300.shock import ShockConfig
    from wumingpic2d_gb300.sim import Simulation

    if args.shock_steps <= 0:
        return None
    cfg = ShockConfig(nx=16384, ny=1024, n_ppc=32, l_damp_ini=64.0, slack=1.0, seed=args.seed + 13)
    d = cfg.dims()
    n0 = 2 * cfg.n_ppc * (d.nx - 2) * d.ny
    with Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision="mixed", bc="shock", u0=cfg.u0,
                    capacity=int(n0 * 1.02)) as sim:
        t0 = time.perf_counter()
        sim.init_shock(cfg)
        t_init = time.perf_counter() - t0
        sim.step(2)
        n_start = sim.info()[0]
        ms = sim.step_timed(args.shock_steps)
        n_end = sim.info()[0]
        iters = sim.cg_iters().tolist()
    return {"workload": f"shock {cfg.nx}x{cfg.ny}, {cfg.n_ppc} ppc/species upstream, u0 {cfg.u0:g}c, mi/me {cfg.mass_ratio:g}, "
                        f"sigma_e {cfg.sigma_e:g}, wall + injection boundary, injection every step, mixed path",
            "value": (n_start + n_end) / 2 * args.shock_steps / (ms / 1e3), "unit": UNIT,
            "ms_per_step": round(ms / args.shock_steps, 3), "steps": args.shock_steps, "particles": n_end,
            "injected_per_step": round((n_end - n_start) / args.shock_steps, 1), "setup_s": round(t_init, 2),
            "cg_iters_last_step": iters}


def guess_standalone_leg(args):
    """The learned guess on its own workload (wumingpic2d_gb300.guess_standalone): the implicit field
    system of a 4096 x 4096 periodic Weibel plasma solved to 1e-10 from the previous step's dB and
    from the network's guess, the network trained here on 20k solver-generated crops from runs of
    the 2048^2 Weibel and 4096 x 2048 Harris workloads; iterations and time both ways, training and
    inference throughput, and the break-even of the guess."""
    if args.standalone_pairs <= 0:
        return None
    from wumingpic2d_gb300 import guess_standalone

    r = guess_standalone.run(pairs=args.standalone_pairs, seed=args.seed)
    r.pop("params")
    return r


def cnn_leg(args):
    """The learned guess's network alone: inference on one 4096 x 4096 image (its forward layers
    on the tcgen05 tensor cores) and training steps (forward, MSE, input and weight gradients, Adam)
    on batches of 8 images of 512 x 512, random inputs, the shipped weights."""
    if args.cnn_steps <= 0 or args.guess == "none" or not os.path.exists(args.guess):
        return None
    import torch

    from wumingpic2d_gb300 import cnn

    net = cnn.GuessNet(np.load(args.guess)["params"])
    g = torch.Generator(device="cuda").manual_seed(args.seed)

    def image(n, h, w):
        x = torch.zeros((n, h, w, cnn.LAYERS[0][0]), device="cuda")
        x[..., :11] = torch.randn((n, h, w, 11), device="cuda", generator=g)
        return x.to(torch.bfloat16)

    def timed(fn, reps):
        for _ in range(2):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # dense multiply-adds per pixel of the convolutions as computed (the last layer's 8 outputs padded to 16)
    flop_px = 2 * 9 * (16 * 48 + 4 * 48 * 48 + 48 * 16)
    x = image(1, 4096, 4096)
    ms_inf = timed(lambda: net.forward(x, train=False), args.cnn_steps)
    del x
    peaks, src = measured_peaks()
    npx = 4096 * 4096
    tflops = flop_px * npx / (ms_inf / 1e3) / 1e12
    xb, yb = image(8, 512, 512), torch.randn((8, 512, 512, 3), device="cuda", generator=g)
    tr = cnn.Trainer(net)
    ms_tr = timed(lambda: tr.step(xb, yb), args.cnn_steps)
    return {"workload": "learned-guess network alone (6 x conv3x3, 48 channels, BF16, FP32 accumulation), random inputs",
            "inference": {"image": "1 x 4096 x 4096", "ms": round(ms_inf, 3), "pixels_per_s": npx / (ms_inf / 1e3),
                          "tflops_dense": round(tflops, 1), "frac_of_bf16_peak": round(tflops / peaks["bf16_tflops"], 4),
                          "peak_source": f"{src} (MEASURED_PEAKS.json bf16_tflops)", "kernels": "tcgen05 (forward layers)"},
            "training": {"batch": "8 x 512 x 512", "ms_per_step": round(ms_tr, 3), "pixels_per_s": 8 * 512 * 512 / (ms_tr / 1e3),
                         "kernels": "forward, input gradient and weight gradient on tcgen05"},
            "steps": args.cnn_steps}


def run_gpu(args, dist: Dist, precision: str, state, do_e2e: bool):
    from wumingpic2d_gb300.sim import Simulation, pinned_zeros, set_device

    set_device(dist.local)
    cfg = state
    d = cfg.dims()
    t0 = time.perf_counter()
    sim = Simulation(d, cfg.delt, cfg.charge, cfg.mass, precision=precision)
    if precision == "mixed":
        sim.set_rebin(args.rebin)
    sim.init_weibel(cfg.ppc, cfg.v_drift, cfg.vth_e, cfg.vth_i, cfg.seed)
    t_init = time.perf_counter() - t0
    ntot, dev_bytes = sim.info()
    clocks = ClockSampler(dist.local)
    clocks.start()
    sim.step(args.warmup)
    sim.set_timing(True)

    dist.barrier()
    clocks.mark_start()
    ms = sim.step_timed(args.steps)
    clocks.mark_stop()
    clk = clocks.stop()
    dist.barrier()
    launches = sim.launches()
    ktimes = sim.kernel_times()
    iters = sim.cg_iters().tolist()
    sim.set_timing(False)
    ms_max = dist.max(ms)
    total = dist.sum(float(ntot)) * args.steps
    value = total / (ms_max / 1e3)

    # e2e through the host-buffer entry point; the host state lives in page-locked memory from
    # wm_host_alloc (registering an existing array instead copies several times slower on Grace)
    e2e = None
    if do_e2e:
        up_h = pinned_zeros((d.ndim, d.np, d.ny, d.nsp))
        uf_h = pinned_zeros((6, d.nx + 4, d.ny + 4))
        np2_h, cc_h = d.alloc_np2(), d.alloc_cumcnt()
        sim.store(up_h, uf_h, np2_h, cc_h)
        maxc = int(np2_h.max())
        h2d = 48 * maxc * d.nsp * d.ny + uf_h.nbytes + np2_h.nbytes + cc_h.nbytes
        d2h = h2d
        sim.step_host(up_h, uf_h, np2_h, cc_h, 1)  # warm-up of the copy path
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            sim.step_host(up_h, uf_h, np2_h, cc_h, 1)
        dt = dist.max(time.perf_counter() - t0)
        sim.set_timing(True)  # one more call, untimed, for the phase breakdown
        sim.step_host(up_h, uf_h, np2_h, cc_h, 1)
        phases = {k: round(v, 2) for k, v in sim.kernel_times().items() if k.startswith(("host_", "copy_"))}
        sim.set_timing(False)
        e2e = {"value": dist.sum(float(ntot)) * args.e2e_steps / dt, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "path": "wm_sim_step_host: reference-layout host arrays (page-locked, wm_host_alloc) in and out every step",
               "phase_ms": phases}
        del up_h, uf_h

    # the same loop with the learned CG initial guess (each component starts from the better of the
    # network's dB and the previous step's; same tolerance)
    guess = None
    if precision == "mixed" and args.guess != "none" and os.path.exists(args.guess):
        sim.set_guess(np.load(args.guess)["params"])
        sim.step(2)
        sim.set_timing(True)
        dist.barrier()
        ms_g = dist.max(sim.step_timed(args.steps))
        kt_g = sim.kernel_times()
        st = sim.guess_stats()
        sim.set_timing(False)
        guess = {"value": dist.sum(float(ntot)) * args.steps / (ms_g / 1e3), "unit": UNIT, "ms_per_step": ms_g / args.steps,
                 "cg_iters_last_step": sim.cg_iters().tolist(), "cg_iters_previous_step_guess": iters,
                 "initial_relative_residual": {"network": np.sqrt(st[0:3] / st[9:12]).round(4).tolist(),
                                               "previous_step": np.sqrt(st[3:6] / st[9:12]).round(4).tolist()},
                 "guess_net_ms_per_step": round(kt_g.get("guess_net", 0.0) / args.steps, 3),
                 "cg_iterate_ms_per_step": round(kt_g.get("cg_iterate", 0.0) / args.steps, 3),
                 "weights": os.path.relpath(args.guess, ROOT)}
    sim.close()
    return dict(ntot=ntot, ms=ms_max, value=value, launches=launches, ktimes=ktimes, iters=iters, clocks=clk, e2e=e2e,
                dev_bytes=dev_bytes, t_init=t_init, d=d, cfg=cfg, precision=precision, guess=guess)


# Algorithmic bytes per particle of the particle kernels.  FP64: 8 B per component (push reads and
# writes x, y, u; the deposit reads old x, y and new x, y, u; the sort moves 6 components).  Mixed,
# with the rebin as a permutation (the default): the fused push+deposit reads its particle's slot
# in the permutation (4 B), reads and writes 5 FP32 components (20 + 20 B) and writes the 4-byte
# move code; the permutation kernel reads the code and the id permutation and writes both
# permutations (4 x 4 B; the ids themselves stay put).  With the move rebin the push reads and
# writes the 5 components and the code (44 B) and the move reads the code and moves 5 FP32
# components and the i64 id (60 B).
# FP64 operations per particle of the FP64 path's compute-bound kernels, counted from the
# reference's code (particle.f90:96-161: ~215 plus 2 square roots and 3 divisions; field.f90:224-298:
# ~570 plus a square root and a division).  The denominator is GB300's FP64 rate as measured by
# wm_fp64_fma_rate (independent FP64 FMA chains on whole waves of the SMs, CUDA events); the
# nominal 1.25 TFLOP/s only where that measurement is unavailable.
FP64_FLOP = {"push": 215, "deposit": 570}
FP64_NOMINAL_TFLOPS = 1.25


def fp64_peak():
    import ctypes

    from wumingpic2d_gb300._native import check, lib

    tf, ms = ctypes.c_double(), ctypes.c_double()
    try:
        check(lib().wm_fp64_fma_rate(ctypes.byref(tf), ctypes.byref(ms)), "wm_fp64_fma_rate")
    except Exception as exc:  # noqa: BLE001 -- reported, the nominal rate is used instead
        return FP64_NOMINAL_TFLOPS, f"nominal (measurement failed: {exc})"
    return tf.value, f"measured: k_fp64_fma (independent FP64 FMA chains, whole SM waves), {ms.value:.1f} ms, CUDA events"


def fp64_rooflines(res, args, peak):
    tflops, src = peak
    out = {}
    for name, f in FP64_FLOP.items():
        t = res["ktimes"].get(name)
        if t:
            tf = f * res["ntot"] / (t / args.steps / 1e3) / 1e12
            out[name] = {"flop_per_particle": f, "achieved_tflops": round(tf, 3), "frac": round(tf / tflops, 3)}
    out["peak"] = {"tflops": round(tflops, 4), "source": src, "nominal_tflops": FP64_NOMINAL_TFLOPS}
    return out


ALGO_BYTES = {"fp64": {"push": 80, "deposit": 56, "sort_move": 96},
              "mixed": {"push_deposit": 48, "sort_perm": 16},
              "mixed_move": {"push_deposit": 44, "sort_move": 60}}
# The path's own algorithmic bytes per particle, independent of this design: the push reads and
# writes x, y, u (FP64 80 B; mixed: two FP32 offsets and three FP32 momenta, 40 B), the deposit
# reads old x, y and new x, y, u (56 B; mixed 28 B, which the fused kernel takes from registers).
# ALGO_BYTES above adds what this design moves on top (the permutation entry, the move code).
PATH_BYTES = {"fp64": {"push": 80, "deposit": 56, "sort_move": 96},
              "mixed": {"push_deposit": 40}, "mixed_move": {"push_deposit": 40}}


def prec_key(res, args):
    return "mixed_move" if res["precision"] == "mixed" and args.rebin == "move" else res["precision"]


def all_rooflines(res, args):
    """achieved GB/s and fraction of the measured HBM peak for every particle kernel"""
    peaks, _ = measured_peaks()
    out = {}
    for name, b in ALGO_BYTES[prec_key(res, args)].items():
        t = res["ktimes"].get(name)
        if t:
            gbs = b * res["ntot"] / (t / args.steps / 1e3) / 1e9
            out[name] = {"achieved": round(gbs, 1), "frac": round(gbs / peaks["hbm_gbs"], 4), "bytes_per_particle": b,
                         "ms_per_launch": round(t / args.steps, 3)}
            if name == "sort_perm":  # on a low-priority stream beside the field solve: its event time includes the time it yields
                out[name]["beside_field_solve"] = True
    return out


def roofline(res, args, name=None):
    peaks, src = measured_peaks()
    kt = res["ktimes"]
    steps = args.steps
    ntot = res["ntot"]
    algo = ALGO_BYTES[prec_key(res, args)]
    cand = {k: v for k, v in kt.items() if k in algo}
    if not cand:
        return None
    name = name or max(cand, key=cand.get)
    t = cand[name] / steps / 1e3
    path_b = PATH_BYTES[prec_key(res, args)].get(name, algo[name])
    achieved = path_b * ntot / t / 1e9
    design = algo[name] * ntot / t / 1e9
    tr = ncu_traffic().get(f"{prec_key(res, args)}:{name}")
    return {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4), "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": (tr * ntot if tr else None), "bytes_per_particle_algorithmic": path_b,
            "bytes_per_particle_design": algo[name], "achieved_at_design_bytes": round(design, 1),
            "frac_at_design_bytes": round(design / peaks["hbm_gbs"], 4),
            "ms_per_launch": round(t * 1e3, 3)}


def main():
    args = parse()
    dist = Dist(args.gpus)
    workload = (f"Weibel {args.nx}x{args.ny} periodic, {args.ppc} ppc/species, 2 species, cfl 0.5, "
                f"omega_pe dt 0.05, mi/me 25, beams +/-0.3c")
    if args.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        v, cores, sample = cpu_sample(args, max(1, args.steps))
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox)",
                "config": {"workload": workload, "nx": args.nx, "ny": args.ny, "ppc": args.ppc},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                 "host_online": cpu_cores()["host_online"],
                                 "note": "C restatement of the reference step (no Fortran compiler on this machine)"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        dist.close()
        return

    state = make_state(args, dist)
    head = "mixed" if args.precision in ("both", "mixed") else "fp64"
    res = run_gpu(args, dist, head, state, do_e2e=not args.no_e2e)
    other = None
    if args.precision == "both":
        other = run_gpu(args, dist, "fp64", state, do_e2e=False)
    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        v, cores, sample = cpu_sample(args, args.cpu_steps)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "core_note": "cores = OpenMP threads = the cores in this process's affinity mask (host_online: all the host has)",
               "host_online": cpu_cores()["host_online"]}
    if dist.rank == 0:
        d = res["d"]
        kt = res["ktimes"]
        line = {
            "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if head == "fp64" else "f32 particles + f64 fields",
            "data": "synthetic (seeded Philox4x32-10 Weibel beams generated on the GPU)",
            "config": {"workload": workload, "nx": d.nx, "ny": d.ny, "ppc": args.ppc, "particles": res["ntot"],
                       "precision": head, "rebin": args.rebin if head == "mixed" else None,
                       "parallelism": f"replicas x{dist.world}",
                       "l2": f"inputs larger than L2 ({res['ntot'] * 48 / 1e9:.1f} GB of particles vs 129 MB)",
                       "cg_iters_last_step": res["iters"], "cg_tol": 1e-6},
            "roofline": roofline(res, args),
            "cpu_baseline": cpu,
            "e2e": res["e2e"],
            "gpu_launches": res["launches"],
            "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in kt.items()},
            "clocks": res["clocks"],
            "device_bytes": res["dev_bytes"],
            "setup_s": round(res["t_init"], 1),
            "rooflines": all_rooflines(res, args),
        }
        if res.get("guess") is not None:
            line["learned_guess"] = res["guess"]
        rc = reconnection_cg(args) if head == "mixed" else None
        if rc is not None:
            line["reconnection_cg"] = rc
        sh = shock_leg(args) if head == "mixed" else None
        if sh is not None:
            line["shock"] = sh
        sa = guess_standalone_leg(args) if head == "mixed" else None
        if sa:
            line["guess_standalone"] = sa
        cl = cnn_leg(args) if head == "mixed" else None
        if cl is not None:
            line["cnn"] = cl
        if other is not None:
            line["fp64_path"] = {"value": other["value"], "unit": UNIT, "ms_per_step": other["ms"] / args.steps,
                                 "speedup_of_mixed": res["value"] / other["value"],
                                 "cg_iters_last_step": other["iters"],
                                 "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in other["ktimes"].items()},
                                 "roofline": roofline(other, args), "roofline_fp64": fp64_rooflines(other, args, fp64_peak()),
                                 "gpu_launches": other["launches"],
                                 "clocks": other["clocks"]}
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
