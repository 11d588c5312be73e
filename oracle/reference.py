"""The reference's own hot-path code, translated to C by oracle/f90c.py and compiled here.

TEST INFRASTRUCTURE ONLY.  generate() translates the reference's common/*.f90 (only where the
reference source tree exists) into oracle/_ref/wuming_ref.c; build() compiles it with the
single-rank glue (oracle/ref_glue.c) into oracle/_ref/libref.so.  Both outputs are git-ignored.
The functions below take the same reference-layout numpy arrays as oracle.py and run the
translated Fortran procedures, so tests can compare the hand restatement with the reference
itself, bit for bit.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
GEN_C = REF_DIR / "wuming_ref.c"
LIB = REF_DIR / "libref.so"
# The reference checkout's common/ directory: $WM_REFERENCE_COMMON, else a checkout named
# "reference" beside this repository.
DEFAULT_SOURCE = Path(os.environ.get("WM_REFERENCE_COMMON", str(HERE.parent.parent / "reference" / "common")))


def generate(source: Path = DEFAULT_SOURCE) -> bool:
    """Translate the reference modules; False when the reference source tree is absent."""
    if not (source / "particle.f90").exists():
        return GEN_C.exists()
    sys.path.insert(0, str(HERE))
    import f90c  # noqa: E402

    REF_DIR.mkdir(exist_ok=True)
    proj = source.parent / "proj"
    extra = [proj / "reconnection" / "boundary_reconnection.f90", proj / "shock" / "boundary_shock.f90"]
    text = f90c.translate(source, [e for e in extra if e.exists()])
    if not GEN_C.exists() or GEN_C.read_text() != text:
        GEN_C.write_text(text)
    return True


def build() -> Path | None:
    if not generate():
        return None
    deps = [GEN_C, HERE / "ref_glue.c", HERE / "ref_runtime.h"]
    if not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-frounding-math", "-fPIC", "-shared", "-I", str(HERE), "-o", str(tmp),
               str(HERE / "ref_glue.c"), str(GEN_C), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def available() -> bool:
    try:
        return build() is not None
    except (OSError, subprocess.CalledProcessError):
        return False


def lib():
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            raise RuntimeError("the reference source tree is not available to translate")
        L = ctypes.CDLL(str(path))
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        sig = {
            "wmr_init": [I, I, I, I, I, I, I, D, D, D, P, P, D],
            "wmr_particle_solv": [P, P, P, P, I, I],
            "wmr_mom_accl": [P, P, P, P, I, I],
            "wmr_mom_nvt": [P, P, P],
            "wmr_field_fdtd_i": [P, P, P, P, I, I],
            "wmr_field_work": [P, P, P, I],
            "wmr_bc_particle_x": [P, P],
            "wmr_bc_particle_y": [P, P],
            "wmr_sort_bucket": [P, P, P, P, I, I],
            "wmr_bc_dfield": [P, I, I, I, I, I, I],
            "wmr_bc_curre": [P, I, I, I, I, I, I],
            "wmr_bc_phi": [P, I, I, I, I, I],
            "wmr_bc_mom": [P],
            "wmr_set_bc": [I],
            "wmr_bc_particle_x_walls": [P, P, I, I],
            "wmr_bc_injection": [P, P, I, I, D],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


class Reference:
    """One configuration of the translated reference modules (their module state is global)."""

    BC = {"periodic": 0, "reconnection": 1, "shock": 2}

    def __init__(self, dims, delt, q, r, c=1.0, delx=1.0, gfac=0.501, bc="periodic"):
        self.d = dims
        q = np.ascontiguousarray(q, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        d = dims
        assert lib().wmr_init(d.ndim, d.np, d.nsp, d.nxgs, d.nxge, d.nygs, d.nyge, delx, delt, c, _p(q), _p(r), gfac) == 0
        assert lib().wmr_set_bc(self.BC[bc]) == 0
        self._fdtd_ready = False

    def particle_solv(self, gp, up, uf, cumcnt):
        return lib().wmr_particle_solv(_p(gp), _p(up), _p(uf), _p(cumcnt), self.d.nxs, self.d.nxe)

    def mom_accl(self, gp, up, uf, cumcnt):
        return lib().wmr_mom_accl(_p(gp), _p(up), _p(uf), _p(cumcnt), self.d.nxs, self.d.nxe)

    def mom_nvt(self, mom, up, np2):
        return lib().wmr_mom_nvt(_p(mom), _p(up), _p(np2))

    def _prime_field(self):
        """Let field__fdtd_i allocate its SAVE'd arrays (first call) on an empty state."""
        if self._fdtd_ready:
            return
        d = self.d
        z_up, z_uf, z_cc = d.alloc_up(), d.alloc_uf(), d.alloc_cumcnt()
        assert lib().wmr_field_fdtd_i(_p(z_uf), _p(z_up), _p(z_up), _p(z_cc), d.nxs, d.nxe) == 0
        self._fdtd_ready = True

    def set_df(self, df):
        self._prime_field()
        assert lib().wmr_field_work(_p(df), None, None, 0) == 0

    def get_work(self):
        d = self.d
        df, uj, gkl = d.alloc_uf(), d.alloc_uj(), d.alloc_gkl()
        assert lib().wmr_field_work(_p(df), _p(uj), _p(gkl), 1) == 0
        return df, uj, gkl

    def field_fdtd_i(self, uf, up, gp, cumcnt):
        self._fdtd_ready = True
        return lib().wmr_field_fdtd_i(_p(uf), _p(up), _p(gp), _p(cumcnt), self.d.nxs, self.d.nxe)

    def bc_particle_x_walls(self, up, np2):
        return lib().wmr_bc_particle_x_walls(_p(up), _p(np2), self.d.nxs, self.d.nxe)

    def bc_injection(self, up, np2, u0):
        return lib().wmr_bc_injection(_p(up), _p(np2), self.d.nxs, self.d.nxe, u0)

    def bc_particle_x(self, up, np2):
        return lib().wmr_bc_particle_x(_p(up), _p(np2))

    def bc_particle_y(self, up, np2):
        return lib().wmr_bc_particle_y(_p(up), _p(np2))

    def sort_bucket(self, gp, up, cumcnt, np2):
        return lib().wmr_sort_bucket(_p(gp), _p(up), _p(cumcnt), _p(np2), self.d.nxs, self.d.nxe)

    def bc_dfield(self, df):
        d = self.d
        return lib().wmr_bc_dfield(_p(df), d.nxs, d.nxe, d.nys, d.nye, d.nxgs, d.nxge)

    def bc_curre(self, uj):
        d = self.d
        return lib().wmr_bc_curre(_p(uj), d.nxs, d.nxe, d.nys, d.nye, d.nxgs, d.nxge)

    def bc_phi(self, phi, l=1):
        d = self.d
        return lib().wmr_bc_phi(_p(phi), d.nxs, d.nxe, d.nys, d.nye, l)

    def bc_mom(self, mom):
        return lib().wmr_bc_mom(_p(mom))

    def step(self, up, gp, uf, cumcnt, np2):
        """The main-loop body of proj/weibel/app.f90:102-107."""
        calls = (lambda: self.particle_solv(gp, up, uf, cumcnt), lambda: self.field_fdtd_i(uf, up, gp, cumcnt),
                 lambda: self.bc_particle_x(gp, np2), lambda: self.bc_particle_y(gp, np2),
                 lambda: self.sort_bucket(up, gp, cumcnt, np2))
        for call in calls:
            st = call()
            if st:
                return st
        return 0
