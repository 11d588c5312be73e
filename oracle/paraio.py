"""Oracle (test infrastructure only): a CPU restatement of the reference's snapshot and output
files, common/paraio.f90 for one MPI rank, with the two I/O layers it calls:

* utils/iocore/jsonio.f90 -- one JSON object per attribute / dataset with the keys datatype,
  offset, size, ndim, shape, description (+ data for attributes), put_metadata_ik :128-170,
  put_scalar_* / put_array_* :173-346;
* utils/iocore/mpiio.f90 -- the raw file: every write lands at the running displacement `disp`
  and advances it by its byte size (write_atomic_array_type :272-291, write_collective_type
  :440-468, write_collective_*_64bit :553-594); endian flag 1 on little-endian hosts (:102-109);
* json-fortran 8.2.1 (vendored in utils/json, built with -DINT64 -DREAL64, utils/json/Makefile):
  the printer's layout (two-space indent, one array element per line) and its real format
  '(ss,E27.17E4)' (json_parameters.F90:76) compacted by compact_real_string
  (json_string_utilities.F90:266-334).

The JSON printer is pinned to utils/iocore/jsonio_expected.json (tests/test_paraio_oracle.py);
the raw layout follows the Fortran column-major order of each array.  Only tests/ import this.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

ENDIAN_FLAG = 1  # mpiio.f90:102-109 on a little-endian host
MOK = 8          # MPI_OFFSET_KIND, the value of dummy_attribute (paraio.f90:19)


# ------------------------------------------------------------------------------ JSON printer
def fortran_real(v: float) -> str:
    """json-fortran's text for a real(8): '(ss,E27.17E4)' then compact_real_string."""
    v = float(v)
    neg = math.copysign(1.0, v) < 0
    a = abs(v)
    if a == 0.0:
        digits, exp = "0" * 17, 0
    else:
        s = "%.16e" % a            # d.dddddddddddddddde+XX, correctly rounded to 17 digits
        mant, e = s.split("e")
        digits, exp = mant.replace(".", ""), int(e) + 1   # 0.d1...d17 x 10^exp
    sig = digits.rstrip("0") or "0"   # keep one digit after the decimal point
    return ("-" if neg else "") + "0." + sig + "E" + ("-" if exp < 0 else "+") + str(abs(exp))


def _scalar(v) -> str:
    if isinstance(v, str):
        return json.dumps(v, ensure_ascii=False)
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return fortran_real(v)


def dumps(obj: dict) -> str:
    """Print a tree of dicts / lists / scalars the way json%print lays it out."""
    out = []

    def emit(v, ind, prefix):
        pad = "  " * ind
        if isinstance(v, dict):
            out.append(pad + prefix + "{")
            items = list(v.items())
            for n, (k, x) in enumerate(items):
                emit(x, ind + 1, json.dumps(k) + ": ")
                if n < len(items) - 1:
                    out[-1] += ","
            out.append(pad + "}")
        elif isinstance(v, (list, tuple)):
            out.append(pad + prefix + "[")
            for n, x in enumerate(v):
                emit(x, ind + 1, "")
                if n < len(v) - 1:
                    out[-1] += ","
            out.append(pad + "]")
        else:
            out.append(pad + prefix + _scalar(v))

    emit(obj, 0, "")
    return "\n".join(out) + "\n"


# ---------------------------------------------------------------------------- file assembly
_DT = {"i4": np.int32, "i8": np.int64, "f4": np.float32, "f8": np.float64}


class Writer:
    """One JSON document and its raw file, built in the order the Fortran writes them."""

    def __init__(self, rawfile: str):
        self.root = {"meta": {"endian": ENDIAN_FLAG, "rawfile": rawfile}}
        self.raw = bytearray()

    def _entry(self, group, name, dt, shape, desc):
        size = int(np.prod(shape)) * np.dtype(_DT[dt]).itemsize
        e = {"datatype": dt, "offset": len(self.raw), "size": size, "ndim": len(shape),
             "shape": [int(s) for s in shape], "description": desc}
        self.root.setdefault(group, {})[name] = e
        return e

    def attribute(self, name, value, dt, desc=""):
        """jsonio_put_attribute + mpiio_write_atomic: scalar or 1-D array."""
        arr = np.atleast_1d(np.asarray(value, dtype=_DT[dt]))
        e = self._entry("attribute", name, dt, arr.shape, desc)
        e["data"] = arr[0].item() if np.ndim(value) == 0 else [x.item() for x in arr]
        self.raw += arr.tobytes()

    def dataset(self, name, array, dt, shape, desc):
        """jsonio_put_metadata + mpiio_write_collective: the array in Fortran order."""
        self._entry("dataset", name, dt, shape, desc)
        self.raw += np.asarray(array, dtype=_DT[dt]).reshape(-1, order="F").tobytes()

    def files(self):
        return dumps(self.root), bytes(self.raw)


class Params:
    """The module variables that paraio__init keeps (paraio.f90:37-72), one rank."""

    def __init__(self, ndim, np_, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c, q, r):
        self.ndim, self.np, self.nsp = ndim, np_, nsp
        self.nxgs, self.nxge, self.nygs, self.nyge, self.nys, self.nye = nxgs, nxge, nygs, nyge, nys, nye
        self.nproc, self.nrank = 1, 0
        self.delx, self.delt, self.c = float(delx), float(delt), float(c)
        self.q = np.asarray(q, dtype=np.float64)[:nsp].copy()
        self.r = np.asarray(r, dtype=np.float64)[:nsp].copy()


def _head(w: Writer, P: Params, it: int, extra=()):
    w.attribute("dummy_attribute", MOK, "i8")
    w.attribute("it", it, "i4")
    for name, v in extra:
        w.attribute(name, v, "i4")
    # put_metadata, paraio.f90:947-1002
    for name in ("ndim", "np", "nxgs", "nxge", "nygs", "nyge", "nsp", "nproc"):
        w.attribute(name, getattr(P, name), "i4")
    w.attribute("delx", P.delx, "f8")
    w.attribute("delt", P.delt, "f8")
    w.attribute("c", P.c, "f8")
    w.attribute("r", P.r, "f8")
    w.attribute("q", P.q, "f8")


def output(P: Params, up, uf, np2, nxs, nxe, it, filename):
    """paraio__output (paraio.f90:93-222): the restart snapshot.  Returns (json text, raw bytes)."""
    w = Writer(filename + ".raw")
    _head(w, P, it, (("nxs", nxs), ("nxe", nxe)))
    w.root["dataset"] = {}
    nyl = P.nye - P.nys + 1
    w.dataset("up", up, "f8", (P.ndim, P.np, nyl, P.nsp, P.nproc), "particles")
    w.dataset("np2", np2, "i4", (nyl, P.nsp, P.nproc), "number of active particles")
    w.dataset("uf", uf, "f8", (6, uf.shape[1], uf.shape[2], P.nproc), "electromagnetic fields including ghost cells")
    return w.files()


def read(json_text: str, raw: bytes) -> dict:
    """Every attribute and dataset of a file pair as numpy arrays (Fortran order, as json2hdf5 and
    paraio__input read them)."""
    obj = json.loads(json_text)
    out = {}
    for group in ("attribute", "dataset"):
        for name, e in obj.get(group, {}).items():
            n = int(np.prod(e["shape"]))
            a = np.frombuffer(raw, dtype=_DT[e["datatype"]], count=n, offset=e["offset"])
            out[name] = a.reshape(e["shape"], order="F").copy()
    return out


def input(P: Params, json_text: str, raw: bytes):
    """paraio__input (paraio.f90:227-417): (up, uf, np2, nxs, nxe, it); raises where the Fortran
    stops on a parameter mismatch."""
    d = read(json_text, raw)
    for name in ("nxgs", "nxge", "nygs", "nyge", "np", "nsp", "nproc"):
        if int(d[name][0]) != getattr(P, name):
            raise ValueError("invalid input parameters")
    nyl = P.nye - P.nys + 1
    if d["up"].shape != (P.ndim, P.np, nyl, P.nsp, P.nproc) or d["np2"].shape != (nyl, P.nsp, P.nproc):
        raise ValueError("fatal error in reading particle data")
    nxw, nyw = P.nxge - P.nxgs + 5, P.nye - P.nys + 5
    if d["uf"].shape != (6, nxw, nyw, P.nproc):
        raise ValueError("fatal error in reading particle data")
    up = np.asfortranarray(d["up"][..., 0])
    np2 = np.asfortranarray(d["np2"][..., 0])
    uf = np.asfortranarray(d["uf"][..., 0])
    return up, uf, np2, int(d["nxs"][0]), int(d["nxe"][0]), int(d["it"][0])


def param(P: Params, n0, wpe, wpi, wge, wgi, vti, vte, filename):
    """paraio__param (paraio.f90:422-550)."""
    w = Writer(filename + ".raw")
    vai = P.c * wgi / wpi
    vae = P.c * wge / wpe
    w.attribute("dummy_attribute", MOK, "i8")
    w.attribute("nx", P.nxge - P.nxgs + 1, "i4")
    w.attribute("ny", P.nyge - P.nygs + 1, "i4")
    w.attribute("np", P.np, "i4")
    for name, v in (("delx", P.delx), ("delt", P.delt), ("c", P.c)):
        w.attribute(name, v, "f8")
    w.attribute("r", P.r, "f8")
    w.attribute("q", P.q, "f8")
    for name, v in (("wpe", wpe), ("wge", wge), ("wpi", wpi), ("wgi", wgi), ("vti", vti), ("vte", vte),
                    ("vai", vai), ("vae", vae)):
        w.attribute(name, v, "f8")
    w.attribute("n0", n0, "i4")
    return w.files()


def cell_fields(P: Params, uf):
    """The cell-centred fields of paraio.f90:661-671 (tmp(6, nxgs:nxge, nys:nye)), kept as written:
    the Bz average takes uf(3,i+1,j) twice and not uf(3,i,j+1)."""
    ox, oy = P.nxgs - 2, P.nys - 2
    i = np.arange(P.nxgs, P.nxge + 1) - ox
    j = np.arange(P.nys, P.nye + 1) - oy
    I, J = np.meshgrid(i, j, indexing="ij")
    t = np.empty((6, len(i), len(j)))
    t[0] = (uf[0, I, J] + uf[0, I, J + 1]) / 2
    t[1] = (uf[1, I, J] + uf[1, I + 1, J]) / 2
    t[2] = (uf[2, I, J] + uf[2, I + 1, J] + uf[2, I + 1, J] + uf[2, I + 1, J + 1]) / 4
    t[3] = (uf[3, I, J] + uf[3, I + 1, J]) / 2
    t[4] = (uf[4, I, J] + uf[4, I, J + 1]) / 2
    t[5] = uf[5, I, J]
    return t


def mom(P: Params, mom, uf, it):
    """paraio__mom (paraio.f90:555-713).  mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp) is divided in place
    by the density as the Fortran does (intent(inout), ghost cells included)."""
    w = Writer("%07d_mom.raw" % it)
    _head(w, P, it)
    w.root["dataset"] = {}
    nxg, nyg = P.nxge - P.nxgs + 1, P.nyge - P.nygs + 1
    inner = (slice(1, 1 + nxg), slice(1, 1 + P.nye - P.nys + 1))
    w.dataset("den", mom[0][inner[0], inner[1], :], "f8", (nxg, nyg, P.nsp), "density")
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in (1, 2, 3):
            mom[k] = mom[k] / mom[0]
        w.dataset("vel", mom[1:4, inner[0], inner[1], :], "f8", (3, nxg, nyg, P.nsp), "velocity")
        for k in (4, 5, 6):
            mom[k] = mom[k] / mom[0]
    w.dataset("temp", mom[4:7, inner[0], inner[1], :], "f8", (3, nxg, nyg, P.nsp), "temperature")
    w.dataset("uf", cell_fields(P, uf), "f8", (6, nxg, nyg), "electromagnetic field")
    return w.files()


def particles(P: Params, up, uf, np2, it, mode):
    """write_particle (paraio.f90:743-849) with get_particle_count (:854-942): mode 0 = every
    active particle (paraio__ptcl, suffix _ptcl), 1 = tracers with a positive id (paraio__orb, _orb)."""
    suffix = "_ptcl" if mode == 0 else "_orb"
    w = Writer("%07d%s.raw" % (it, suffix))
    _head(w, P, it)
    w.root["dataset"] = {}
    nxg, nyg = P.nxge - P.nxgs + 1, P.nyge - P.nygs + 1
    ox, oy = P.nxgs - 2, P.nys - 2
    w.dataset("uf", uf[:, P.nxgs - ox:P.nxge + 1 - ox, P.nys - oy:P.nye + 1 - oy], "f8", (6, nxg, nyg),
              "electromagnetic field")
    for isp in range(P.nsp):
        cols = []
        for j in range(P.nye - P.nys + 1):
            blk = up[:, :np2[j, isp], j, isp]
            if mode == 1:
                blk = blk[:, blk[P.ndim - 1].view(np.int64) > 0]
            cols.append(blk)
        packed = np.concatenate(cols, axis=1) if cols else np.zeros((P.ndim, 0))
        w.dataset("up%02d" % (isp + 1), packed, "f8", (P.ndim, packed.shape[1]), "particle species #%02d" % (isp + 1))
    return w.files()


def save(dirname: str, filename: str, files) -> None:
    js, raw = files
    with open(os.path.join(dirname, filename + ".json"), "w") as f:
        f.write(js)
    with open(os.path.join(dirname, filename + ".raw"), "wb") as f:
        f.write(raw)
