"""Shared test inputs: seeded reference-layout states and comparison helpers."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from wumingpic2d_gb300.layout import bits_to_pid
from wumingpic2d_gb300.weibel import WeibelConfig, weibel_particles


def periodic_ghosts(f: np.ndarray, nx: int, ny: int) -> None:
    """Fill the two ghost layers of a (nc, nx+4, ny+4) array with periodic copies."""
    f[:, :, 0] = f[:, :, ny]
    f[:, :, 1] = f[:, :, ny + 1]
    f[:, :, ny + 2] = f[:, :, 2]
    f[:, :, ny + 3] = f[:, :, 3]
    f[:, 0, :] = f[:, nx, :]
    f[:, 1, :] = f[:, nx + 1, :]
    f[:, nx + 2, :] = f[:, 2, :]
    f[:, nx + 3, :] = f[:, 3, :]


class State:
    """A sorted Weibel state with optional random fields, in the reference layout."""

    def __init__(self, nx=32, ny=24, ppc=8, seed=7, field_amp=0.0, df_amp=0.0, slack=1.5, cfl=0.5):
        self.cfg = WeibelConfig(nx=nx, ny=ny, ppc=ppc, seed=seed, slack=slack, cfl=cfl)
        self.d = self.cfg.dims()
        self.par = O.make_par(self.d, self.cfg.delt, self.cfg.charge, self.cfg.mass)
        up0, self.np2 = weibel_particles(self.cfg)
        self.up = self.d.alloc_up()
        self.cumcnt = self.d.alloc_cumcnt()
        assert O.sort_bucket(self.par, self.d, self.up, up0, self.cumcnt, self.np2) == 0
        self.gp = self.up.copy(order="F")
        rng = np.random.default_rng(seed + 1000)
        self.uf = self.d.alloc_uf()
        if field_amp:
            self.uf[:] = field_amp * rng.standard_normal(self.uf.shape)
            periodic_ghosts(self.uf, nx, ny)
        self.df = self.d.alloc_uf()
        if df_amp:
            self.df[:] = df_amp * rng.standard_normal(self.df.shape)
            periodic_ghosts(self.df, nx, ny)

    def copy(self):
        c = object.__new__(State)
        c.__dict__.update(self.__dict__)
        for k in ("up", "gp", "uf", "cumcnt", "np2", "df"):
            setattr(c, k, getattr(self, k).copy(order="F"))
        return c

    def oracle_state(self):
        s = O.OracleState(self.d)
        s.df[:] = self.df
        return s


def confine_x(st: "State", margin_lo: int = 1, margin_hi: int = 2) -> None:
    """Squeeze the particles of st into [nxgs + margin_lo, nxge + 1 - margin_hi) (where the wall
    applications keep them) and cell-sort them again; up, gp and cumcnt are replaced."""
    d = st.d
    lo, hi = d.nxgs + margin_lo, d.nxge + 1 - margin_hi
    up = st.up.copy(order="F")
    for isp in range(d.nsp):
        for j in range(d.ny):
            n = int(st.np2[j, isp])
            x = up[0, :n, j, isp]
            up[0, :n, j, isp] = lo + (x - d.nxgs) * (hi - lo) / (d.nxge + 1 - d.nxgs)
    st.up = d.alloc_up()
    st.cumcnt = d.alloc_cumcnt()
    assert O.sort_bucket(st.par, d, st.up, up, st.cumcnt, st.np2) == 0
    st.gp = st.up.copy(order="F")


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| (normwise relative error, 0 when both are zero)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if a.size else 0.0
    if den == 0.0:
        return float(num)
    return float(num / den)


def active_particles(d, up, np2):
    """Concatenate the active slots of every row: returns (x, y, ux, uy, uz, pid, row)."""
    cols = [[] for _ in range(7)]
    for isp in range(d.nsp):
        for j in range(d.ny):
            n = int(np2[j, isp])
            for k in range(5):
                cols[k].append(up[k, :n, j, isp])
            cols[5].append(bits_to_pid(up[5, :n, j, isp]))
            cols[6].append(np.full(n, isp * d.ny + j))
    return [np.concatenate(c) for c in cols]
