"""Run diagnostics of a Weibel run: energy history, growth rate of the magnetic energy, and the
Gauss-law residual div E - 4 pi rho.

The energies are the ones proj/weibel/app.f90:507-541 writes (kinetic energy per species, then
the electric and magnetic field energies).  The charge density uses the same second-order
shape as the Esirkepov deposit (field.f90:224-236), for which the scheme conserves charge
exactly: div E - 4 pi rho then stays at its initial value up to round-off, so its drift over a
run measures the error of the current deposit.
"""
from __future__ import annotations

import numpy as np

from .layout import Dims


def div_e(d: Dims, uf: np.ndarray) -> np.ndarray:
    """Cell-centred divergence of E on the interior, (nx, ny); uf in the reference layout."""
    ex = uf[3, 2:d.nx + 3, 2:d.ny + 2]
    ey = uf[4, 2:d.nx + 2, 2:d.ny + 3]
    return (ex[1:, :] - ex[:-1, :]) + (ey[:, 1:] - ey[:, :-1])


def charge_density(d: Dims, up: np.ndarray, np2: np.ndarray, q) -> np.ndarray:
    """Charge density with the deposit's quadratic shape on the periodic interior, (nx, ny)."""
    rho = np.zeros((d.nx, d.ny))
    for isp in range(d.nsp):
        for jj in range(d.ny):
            n = int(np2[jj, isp])
            if n == 0:
                continue
            x, y = up[0, :n, jj, isp], up[1, :n, jj, isp]
            i, j = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64)
            hx, hy = x - 0.5 - i, y - 0.5 - j
            sx = (0.5 * (0.5 - hx) ** 2, 0.75 - hx**2, 0.5 * (0.5 + hx) ** 2)
            sy = (0.5 * (0.5 - hy) ** 2, 0.75 - hy**2, 0.5 * (0.5 + hy) ** 2)
            for a in range(3):
                ia = (i + a - 1 - d.nxgs) % d.nx
                for b in range(3):
                    np.add.at(rho, (ia, (j + b - 1 - d.nygs) % d.ny), q[isp] * sx[a] * sy[b])
    return rho


def gauss_residual(d: Dims, up: np.ndarray, uf: np.ndarray, np2: np.ndarray, q) -> np.ndarray:
    return div_e(d, uf) - 4.0 * np.pi * charge_density(d, up, np2, q)


def growth_rate(t: np.ndarray, e_b: np.ndarray, lo: float = 10**-4.5, hi: float = 10**-1.5):
    """Growth rate of the field amplitude, gamma = 0.5 d ln(E_B)/dt, fitted over the linear phase.

    The linear phase is taken as the samples before E_B first reaches hi * max(E_B) and at or
    above lo * max(E_B).  Returns (gamma, t_start, t_end), or (nan, nan, nan) without a phase.
    """
    t = np.asarray(t, dtype=np.float64)
    e_b = np.asarray(e_b, dtype=np.float64)
    top = e_b.max()
    if not np.isfinite(top) or top <= 0:
        return float("nan"), float("nan"), float("nan")
    above = np.nonzero(e_b >= hi * top)[0]
    end = above[0] if above.size else len(e_b)
    sel = np.nonzero(e_b[:end] >= lo * top)[0]
    if sel.size < 3:
        return float("nan"), float("nan"), float("nan")
    sel = np.arange(sel[0], end)
    slope = np.polyfit(t[sel], np.log(e_b[sel]), 1)[0]
    return 0.5 * slope, float(t[sel[0]]), float(t[sel[-1]])


def energy_history(sim, nsteps: int, every: int):
    """Step a resident Simulation nsteps times; energies every `every` steps (and at step 0).

    Returns (steps, energies) with energies of shape (samples, nsp + 2).
    """
    steps, rows = [0], [sim.energy()]
    done = 0
    while done < nsteps:
        k = min(every, nsteps - done)
        sim.step(k)
        done += k
        steps.append(done)
        rows.append(sim.energy())
    return np.asarray(steps), np.asarray(rows)
