"""Seeded Weibel-instability initial condition (two counter-streaming electron beams).

Physical constants and charge/mass conventions follow proj/weibel/app.f90:
c = 1, delx = 1, gfac = 0.501 (:64-67), delt = cfl*delx/c (:292),
r(1) = mass_ratio (ions), r(2) = 1 (electrons) (:299-300),
q(s) = +/-sqrt(r(s)/(4*pi*n0/delx**2))*omega_p,s (:301-302), n0 = particles per
cell per species.  Particles are placed row by row, n0*nx per row as the
reference does (:306), ions and electrons at the same positions so that the
initial charge density is zero.

The beam set-up replaces the reference's anisotropic Maxwellian (:419-432):
positions are uniform random over each row, electrons drift along z with
four-velocity +/- v/sqrt(1-v^2) (even/odd particle index) plus an isotropic
Gaussian spread vth_e in each momentum component, ions carry vth_i.  Fields
start at zero.  Random numbers come from numpy's counter-based Philox
generator, so a seed gives the same state on every machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .layout import Dims, pid_to_bits


@dataclass
class WeibelConfig:
    nx: int = 256
    ny: int = 256
    ppc: int = 16  # particles per cell per species
    cfl: float = 0.5
    omega_pe: float = 0.1
    mass_ratio: float = 25.0
    v_drift: float = 0.3  # beam speed in units of c
    vth_e: float = 0.05
    vth_i: float = 0.01
    gfac: float = 0.501
    c: float = 1.0
    delx: float = 1.0
    slack: float = 1.25  # slots per row = ceil(slack * ppc * nx)
    seed: int = 12345
    extra: dict = field(default_factory=dict)

    @property
    def delt(self) -> float:
        return self.cfl * self.delx / self.c

    @property
    def mass(self) -> np.ndarray:
        return np.array([self.mass_ratio, 1.0])

    @property
    def charge(self) -> np.ndarray:
        n0 = self.ppc
        wpe = self.omega_pe
        wpi = wpe / math.sqrt(self.mass_ratio)
        r = self.mass
        q1 = +math.sqrt(r[0] / (4 * math.pi * n0 / self.delx**2)) * wpi
        q2 = -math.sqrt(r[1] / (4 * math.pi * n0 / self.delx**2)) * wpe
        return np.array([q1, q2])

    def dims(self) -> Dims:
        npr = int(math.ceil(self.slack * self.ppc * self.nx))
        return Dims(nx=self.nx, ny=self.ny, np=npr)


def weibel_particles(cfg: WeibelConfig):
    """Return (up, np2) in the reference layout, rows filled but not yet cell-sorted."""
    d = cfg.dims()
    n_row = cfg.ppc * cfg.nx
    rng = np.random.Generator(np.random.Philox(cfg.seed))
    up = d.alloc_up()
    np2 = d.alloc_np2()
    np2[:, :] = n_row
    rows = np.arange(d.nys, d.nye + 1, dtype=np.float64)
    x = d.nxgs + cfg.nx * rng.random((n_row, d.ny))
    y = rows[None, :] + rng.random((n_row, d.ny))
    # guard the open upper edge: x < nxge+1, y < j+1 after rounding
    np.minimum(x, np.nextafter(d.nxge + 1.0, 0.0), out=x)
    np.minimum(y, np.nextafter(rows[None, :] + 1.0, 0.0), out=y)
    ud = cfg.v_drift / math.sqrt(1.0 - cfg.v_drift**2)
    sign = np.where(np.arange(n_row) % 2 == 0, 1.0, -1.0)[:, None]
    for isp, vth in ((0, cfg.vth_i), (1, cfg.vth_e)):
        up[0, :n_row, :, isp] = x
        up[1, :n_row, :, isp] = y
        up[2, :n_row, :, isp] = vth * rng.standard_normal((n_row, d.ny))
        up[3, :n_row, :, isp] = vth * rng.standard_normal((n_row, d.ny))
        uz = vth * rng.standard_normal((n_row, d.ny))
        if isp == 1:
            uz += sign * ud
        up[4, :n_row, :, isp] = uz
        pid = 1 + np.arange(n_row * d.ny, dtype=np.int64).reshape(d.ny, n_row).T
        up[5, :n_row, :, isp] = pid_to_bits(pid)
    return up, np2
