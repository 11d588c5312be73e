"""Seeded Harris current-sheet initial condition of the reconnection application.

Follows proj/reconnection/app.f90 (load_config :245-255, init :290-310, set_initial_condition
:353-470): walls in x and periodic in y, as the reference is; the sheet is the plane x = x0, so
By(x) = b0 tanh((x - x0)/lcs) reverses across it, plus the reference's localized perturbation
(e1 = 0.12 of b0, Gaussian of width 2 lcs around the X point).  Densities: nbg background
particles per cell and ncs at the sheet centre; the sheet is drawn from the logistic
distribution of :429-433 and the background uniformly in [nxgs+1, nxge-1) (:423-424).  Ions and
electrons start at the same positions; drifts from jz/density as at :440-446 (f1, f2 split the
current in the temperature ratio).  Random numbers come from numpy's counter-based Philox
generator instead of the reference's random_number, so a seed gives the same state everywhere.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .layout import Dims, pid_to_bits


@dataclass
class HarrisConfig:
    nx: int = 256
    ny: int = 128
    mass_ratio: float = 25.0
    alpha: float = 2.0      # omega_pe / omega_ce
    rtemp: float = 0.2      # Te / Ti
    lcs: float = 0.5        # half-thickness in ion inertial lengths c/omega_pi
    nbg: int = 6            # background particles per cell per species
    ncs: int = 58           # sheet-centre particles per cell per species
    e1: float = 0.12        # perturbation B1/B0 (app.f90:375)
    cfl: float = 0.5
    c: float = 1.0
    delx: float = 1.0
    gfac: float = 0.501
    slack: float = 1.5      # slots per row = slack * particles per row
    seed: int = 7

    @property
    def n0(self):
        return self.nbg + self.ncs

    @property
    def delt(self):
        return self.cfl * self.delx / self.c

    @property
    def mass(self):
        return np.array([self.mass_ratio, 1.0])

    def plasma(self):
        """(vte, vti, wpe, wpi, q, b0, lcs in cells) as app.f90:290-305."""
        c, delx = self.c, self.delx
        r = self.mass
        ldb = delx
        vte = math.sqrt(self.rtemp) * c / (math.sqrt(1 + self.rtemp) * self.alpha)
        vti = vte * math.sqrt(r[1] / r[0]) / math.sqrt(self.rtemp)
        wpe = vte / ldb / math.sqrt(2.0)
        wpi = wpe * math.sqrt(r[1] / r[0])
        wge = wpe / self.alpha
        wgi = wge / self.mass_ratio
        q = np.array([+math.sqrt(r[0] / (4 * math.pi * self.n0 / delx**2)) * wpi,
                      -math.sqrt(r[1] / (4 * math.pi * self.n0 / delx**2)) * wpe])
        b0 = r[0] * c / q[0] * wgi
        return vte, vti, wpe, wpi, q, b0, self.lcs * c / wpi

    @property
    def charge(self):
        return self.plasma()[4]

    def per_row(self):
        lcs = self.plasma()[6]
        return int(self.nbg * (self.nx - 1) + self.ncs * 2 * lcs)  # np2 of app.f90:309 (nxge-nxgs = nx-1)

    def dims(self) -> Dims:
        return Dims(nx=self.nx, ny=self.ny, np=int(math.ceil(self.slack * self.per_row())))


def harris_state(cfg: HarrisConfig):
    """(up, uf, np2) in the reference layout; rows filled, not yet cell-sorted."""
    d = cfg.dims()
    vte, vti, wpe, wpi, q, b0, lcs = cfg.plasma()
    delx = cfg.delx
    nxgs, nxge, nygs, nyge = d.nxgs, d.nxge, d.nygs, d.nyge
    x0 = 0.5 * (nxge + nxgs) * delx
    y0 = 0.5 * (nyge - nygs) * delx
    e1 = cfg.e1

    def bx_pert(x, y):
        return +e1 * b0 * ((y - y0) / lcs) * np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2)

    def by_pert(x, y):
        return -e1 * b0 * ((x - x0) / lcs) * np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2)

    def density(x):
        return cfg.ncs * np.cosh((x - x0) / lcs) ** (-2) + cfg.nbg

    def jz(x, y):
        g = np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2)
        return (b0 / (4 * math.pi * lcs) * np.cosh((x - x0) / lcs) ** (-2)
                - 2 * e1 * b0 / (4 * math.pi * lcs) * (1.0 - ((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2) * g)

    # fields on nxs-2..nxe+2, nys-2..nye+2 (app.f90:397-410), evaluated at the integer index * delx
    uf = d.alloc_uf()
    ii = (np.arange(d.nx + 4) + nxgs - 2)[:, None] * delx
    jj = (np.arange(d.ny + 4) + nygs - 2)[None, :] * delx
    uf[0] = bx_pert(ii, jj)
    uf[1] = b0 * np.tanh((ii - x0) / lcs) + by_pert(ii, jj)

    rng = np.random.Generator(np.random.Philox(cfg.seed))
    n_row = cfg.per_row()
    ibg = cfg.nbg * (nxge - nxgs - 2)
    up = d.alloc_up()
    np2 = d.alloc_np2()
    np2[:, :] = n_row
    rows = np.arange(d.nys, d.nye + 1, dtype=np.float64)
    x = np.empty((n_row, d.ny))
    x[:ibg] = (nxgs + 1) * delx + rng.random((ibg, d.ny)) * delx * (nxge - nxgs - 2)
    r1 = (2.0 * rng.random((n_row - ibg, d.ny)) - 1.0) * math.tanh(0.5 * (nxge - nxgs - 2) * delx / lcs)
    x[ibg:] = lcs * 0.5 * (np.log1p(r1) - np.log1p(-r1)) + x0
    y = rows[None, :] * delx + rng.random((n_row, d.ny)) * delx
    np.minimum(y, np.nextafter(rows[None, :] + 1.0, 0.0), out=y)
    f1 = 1.0 / ((1.0 + cfg.rtemp) * q[0])
    f2 = cfg.rtemp / ((1.0 + cfg.rtemp) * q[1])
    drift = jz(x, y) / density(x)
    for isp, (sd, f) in enumerate(((vti / math.sqrt(2.0), f1), (vte / math.sqrt(2.0), f2))):
        up[0, :n_row, :, isp] = x
        up[1, :n_row, :, isp] = y
        up[2, :n_row, :, isp] = sd * rng.standard_normal((n_row, d.ny))
        up[3, :n_row, :, isp] = sd * rng.standard_normal((n_row, d.ny))
        up[4, :n_row, :, isp] = sd * rng.standard_normal((n_row, d.ny)) + f * drift
        pid = 1 + np.arange(n_row * d.ny, dtype=np.int64).reshape(d.ny, n_row).T
        up[5, :n_row, :, isp] = pid_to_bits(-pid)  # negative ids, app.f90:489-491
    return up, uf, np2
