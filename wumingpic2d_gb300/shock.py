"""Parameters of the collisionless-shock application, proj/shock/app.f90.

load_config (:230-287) and init (:292-336): u0 = -|u_inject| is the upstream four-velocity,
gam0 = sqrt(1 + u0^2/c^2), v0 = u0/gam0; wpe = omega_pe, wge = omega_pe sqrt(sigma_e),
wpi = wpe/sqrt(mass_ratio), wgi = wge/mass_ratio; r = (mass_ratio, 1);
q(1) = +sqrt(gam0 r1 / (4 pi n0/delx^2)) wpi, q(2) = -sqrt(gam0 r2 / (4 pi n0/delx^2)) wpe;
b0 = r1 c / q1 * wgi * gam0; angles given in degrees.  The box starts at nxe = nxgs + n_x_ini
(n_x_ini = 0 here: the full box, nxe = nxge), np2 = n0 (nxe - nxs - 1) per row, and grows by one
cell every intvl_expand steps (0: never) until nxe = nxge.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .layout import Dims


@dataclass
class ShockConfig:
    nx: int = 512
    ny: int = 64
    n_ppc: int = 32
    u_inject: float = 0.1
    mass_ratio: float = 100.0
    sigma_e: float = 0.01
    omega_pe: float = 0.05
    v_the: float = 0.05
    v_thi: float = 0.005      # beta_i = beta_e at Ti = Te: v_the / sqrt(mass_ratio)
    theta_bn: float = 90.0    # degrees
    phi_bn: float = 90.0
    l_damp_ini: float = 16.0  # in cells
    tracer_window: tuple = (0.0, 0.0)  # [xrs, xre]: ids made positive there
    cfl: float = 0.5
    c: float = 1.0
    delx: float = 1.0
    gfac: float = 0.501
    slack: float = 2.0        # slots per row = slack * n_ppc * nx (the reference allots 5x)
    seed: int = 11
    n_x_ini: int = 0          # initial box nxe = nxgs + n_x_ini (app.f90:277); 0: the full box, nx - 1
    intvl_expand: int = 0     # nxe grows by one cell every intvl_expand steps (app.f90:123-125); 0: never

    @property
    def delt(self):
        return self.cfl * self.delx / self.c

    @property
    def u0(self):
        return -abs(self.u_inject)

    def plasma(self):
        """(gam0, v0, wpe, wpi, wge, wgi, q, b0) as app.f90:316-332."""
        c, delx, n0 = self.c, self.delx, self.n_ppc
        u0 = self.u0
        gam0 = math.sqrt(1 + (u0 * u0) / (c * c))
        v0 = u0 / gam0
        wpe = self.omega_pe
        wge = self.omega_pe * math.sqrt(self.sigma_e)
        wpi = wpe / math.sqrt(self.mass_ratio)
        wgi = wge / self.mass_ratio
        r = self.mass
        q = np.array([+math.sqrt(gam0 * r[0] / (4 * math.pi * n0 / delx ** 2)) * wpi,
                      -math.sqrt(gam0 * r[1] / (4 * math.pi * n0 / delx ** 2)) * wpe])
        b0 = r[0] * c / q[0] * wgi * gam0
        return gam0, v0, wpe, wpi, wge, wgi, q, b0

    @property
    def mass(self):
        return np.array([self.mass_ratio, 1.0])

    @property
    def charge(self):
        return self.plasma()[6]

    def dims(self) -> Dims:
        return Dims(nx=self.nx, ny=self.ny, np=int(math.ceil(self.slack * self.n_ppc * self.nx)))

    def init_args(self):
        """Arguments of wm_sim_init_shock after the simulation handle."""
        b0 = self.plasma()[7]
        xrs, xre = self.tracer_window
        return (self.n_ppc, self.u0, self.v_the, self.v_thi, b0, self.theta_bn * math.pi / 180, self.phi_bn * math.pi / 180,
                self.l_damp_ini * self.delx, xrs, xre, self.seed)
