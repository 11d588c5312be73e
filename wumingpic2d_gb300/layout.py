"""Host-side arrays in the reference's Fortran layout.

The reference keeps its state in column-major arrays with custom lower bounds
(proj/weibel/app.f90:73-81, :278-283).  On the host this package holds them as
numpy arrays in Fortran order whose shapes are the Fortran extents; the lower
bounds are implicit and fixed by ``Dims``:

    up, gp  (ndim, np, nys:nye, nsp)               -> shape (ndim, np, ny, nsp)
    uf      (6, nxgs-2:nxge+2, nys-2:nye+2)        -> shape (6, nx+4, ny+4)
    cumcnt  (nxgs:nxge+1, nys:nye, nsp)  int32     -> shape (nx+1, ny, nsp)
    np2     (nys:nye, nsp)               int32     -> shape (ny, nsp)
    mom     (7, nxgs-1:nxge+1, nys-1:nye+1, nsp)   -> shape (7, nx+2, ny+2, nsp)

One process owns the whole domain, so nys = nygs and nye = nyge (the
reference's single-rank decomposition, common/mpi_set.f90:37-41).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Dims:
    nx: int
    ny: int
    np: int  # particle slots per row and species (the reference's ``np``)
    nsp: int = 2
    ndim: int = 6
    nxgs: int = 2
    nygs: int = 2
    nxe_act: int = 0  # the active right end nxe when the shock's box expands (0: nxge)

    @property
    def nxge(self) -> int:
        return self.nxgs + self.nx - 1

    @property
    def nyge(self) -> int:
        return self.nygs + self.ny - 1

    @property
    def nys(self) -> int:
        return self.nygs

    @property
    def nye(self) -> int:
        return self.nyge

    @property
    def nxs(self) -> int:
        return self.nxgs

    @property
    def nxe(self) -> int:
        return self.nxe_act if self.nxe_act else self.nxge

    # ---- allocation in the reference layout
    def alloc_up(self) -> np.ndarray:
        return np.zeros((self.ndim, self.np, self.ny, self.nsp), dtype=np.float64, order="F")

    def alloc_uf(self) -> np.ndarray:
        return np.zeros((6, self.nx + 4, self.ny + 4), dtype=np.float64, order="F")

    def alloc_uj(self) -> np.ndarray:
        return np.zeros((3, self.nx + 4, self.ny + 4), dtype=np.float64, order="F")

    def alloc_gkl(self) -> np.ndarray:
        return np.zeros((3, self.nx, self.ny), dtype=np.float64, order="F")

    def alloc_cumcnt(self) -> np.ndarray:
        return np.zeros((self.nx + 1, self.ny, self.nsp), dtype=np.int32, order="F")

    def alloc_np2(self) -> np.ndarray:
        return np.zeros((self.ny, self.nsp), dtype=np.int32, order="F")

    def alloc_mom(self) -> np.ndarray:
        return np.zeros((7, self.nx + 2, self.ny + 2, self.nsp), dtype=np.float64, order="F")

    # ---- index helpers (Fortran index -> 0-based numpy index)
    def fi(self, i: int) -> int:
        """Field x index i (nxgs-2..nxge+2) -> numpy axis-1 index."""
        return i - (self.nxgs - 2)

    def fj(self, j: int) -> int:
        """Field y index j (nys-2..nye+2) -> numpy axis-2 index."""
        return j - (self.nys - 2)


def check_fortran(a: np.ndarray, dtype, shape, name: str) -> None:
    if a.dtype != np.dtype(dtype):
        raise TypeError(f"{name}: dtype {a.dtype}, expected {np.dtype(dtype)}")
    if tuple(a.shape) != tuple(shape):
        raise ValueError(f"{name}: shape {a.shape}, expected {tuple(shape)}")
    if not a.flags.f_contiguous:
        raise ValueError(f"{name}: must be Fortran-contiguous (column-major)")


def pid_to_bits(pid: np.ndarray) -> np.ndarray:
    """Particle ids as the reference stores them: transfer(-pid, 1.0_8) (app.f90:468)."""
    return (-np.asarray(pid, dtype=np.int64)).view(np.float64)


def bits_to_pid(col: np.ndarray) -> np.ndarray:
    return -np.ascontiguousarray(col).view(np.int64)
