"""The snapshot/output restatement (oracle/paraio.py) on the CPU: its JSON printer against the
reference's own known answer (utils/iocore/jsonio_expected.json, written by
utils/iocore/jsonio_test.f90:117-250 and compared as text by utils/iocore/unittest.py), and the
raw layout and round trips of the paraio files."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

from oracle import paraio as PIO

# the reference checkout: $WM_REFERENCE_ROOT, else a checkout named "reference" beside this repository
EXPECTED = Path(os.environ.get("WM_REFERENCE_ROOT", str(Path(__file__).resolve().parents[2] / "reference"))) / "utils/iocore/jsonio_expected.json"


def test_fortran_real_format():
    assert PIO.fortran_real(1.0) == "0.1E+1"
    assert PIO.fortran_real(100.0) == "0.1E+3"
    assert PIO.fortran_real(-1.0) == "-0.1E+1"
    assert PIO.fortran_real(0.0) == "0.0E+0"
    assert PIO.fortran_real(0.5) == "0.5E+0"
    assert PIO.fortran_real(1e-3) == "0.1E-2"
    assert PIO.fortran_real(0.1) == "0.10000000000000001E+0"
    assert PIO.fortran_real(1.0 / 3.0) == "0.33333333333333331E+0"
    for v in (1.0 / 3.0, 0.1, 2.0 ** 70, -7.25e-300, 6.02214076e23):
        assert float(PIO.fortran_real(v)) == v


@pytest.mark.skipif(not EXPECTED.exists(), reason="reference known-answer file unavailable")
def test_json_printer_matches_reference_known_answer():
    """jsonio_test.f90 write_json, restated call by call through the oracle's printer."""
    nx, ny, ns = 16, 32, 2
    root = {"meta": {"endian": 1, "rawfile": "test.raw", "info": "some information", "large_int": 2 ** 32}}
    att, off = {}, 0

    def put(group, name, dt, size, shape, desc, data=None):
        nonlocal off
        e = {"datatype": dt, "offset": off, "size": size, "ndim": len(shape), "shape": list(shape), "description": desc}
        if data is not None:
            e["data"] = data
        group[name] = e
        off += size

    put(att, "nx", "i4", 4, (1,), "# grid in x", nx)
    put(att, "ny", "i4", 4, (1,), "# grid in y", ny)
    put(att, "ns", "i4", 4, (1,), "# species", ns)
    put(att, "mass", "f8", 16, (2,), "mass", [1.0, 100.0])
    put(att, "charge", "f8", 16, (2,), "charge", [-1.0, 1.0])
    root["attribute"] = att
    ds = {}
    put(ds, "emf", "f8", 6 * ny * nx * 8, (6, ny, nx), "electromagnetic fields")
    put(ds, "mom", "f8", 10 * ny * nx * 8, (10, ny, nx), "moments")
    root["dataset"] = ds
    expected = EXPECTED.read_text()
    assert PIO.dumps(root).rstrip("\n") == expected.rstrip("\n")


def small_params(nsp=2):
    return PIO.Params(6, 12, nsp, 2, 9, 2, 7, 2, 7, 1.0, 0.5, 1.0, [-1.0, 1.0], [1.0, 25.0])


def test_snapshot_layout_and_round_trip():
    P = small_params()
    rng = np.random.default_rng(3)
    ny, nx = P.nye - P.nys + 1, P.nxge - P.nxgs + 1
    up = np.asfortranarray(rng.standard_normal((6, P.np, ny, P.nsp)))
    uf = np.asfortranarray(rng.standard_normal((6, nx + 4, ny + 4)))
    np2 = np.asfortranarray(rng.integers(0, P.np + 1, (ny, P.nsp)).astype(np.int32))
    js, raw = PIO.output(P, up, uf, np2, 2, 9, 1234, "snap")
    obj = json.loads(js)
    # attributes at the running displacement: dummy (i8) then it, nxs, nxe and the common block
    att = obj["attribute"]
    assert [att[k]["offset"] for k in ("dummy_attribute", "it", "nxs", "nxe", "ndim")] == [0, 8, 12, 16, 20]
    assert att["delx"]["offset"] == 52 and att["r"]["offset"] == 76 and att["q"]["offset"] == 76 + 8 * P.nsp
    assert obj["meta"] == {"endian": 1, "rawfile": "snap.raw"}
    ds = obj["dataset"]
    assert ds["up"]["offset"] == 76 + 16 * P.nsp and ds["up"]["shape"] == [6, P.np, ny, P.nsp, 1]
    assert ds["np2"]["offset"] == ds["up"]["offset"] + up.nbytes
    assert ds["uf"]["offset"] == ds["np2"]["offset"] + np2.nbytes and len(raw) == ds["uf"]["offset"] + uf.nbytes
    up2, uf2, np22, nxs, nxe, it = PIO.input(P, js, raw)
    assert np.array_equal(up2, up) and np.array_equal(uf2, uf) and np.array_equal(np22, np2)
    assert (nxs, nxe, it) == (2, 9, 1234)
    with pytest.raises(ValueError):
        PIO.input(PIO.Params(6, 13, 2, 2, 9, 2, 7, 2, 7, 1.0, 0.5, 1.0, [-1, 1], [1, 25]), js, raw)


def test_moment_file_divides_in_place_and_keeps_the_bz_average():
    P = small_params()
    rng = np.random.default_rng(4)
    ny, nx = P.nye - P.nys + 1, P.nxge - P.nxgs + 1
    mom = np.asfortranarray(rng.uniform(0.5, 2.0, (7, nx + 2, ny + 2, P.nsp)))
    mom0 = mom.copy()
    uf = np.asfortranarray(rng.standard_normal((6, nx + 4, ny + 4)))
    js, raw = PIO.mom(P, mom, uf, 7)
    d = PIO.read(js, raw)
    assert json.loads(js)["meta"]["rawfile"] == "0000007_mom.raw"
    assert np.array_equal(d["den"], mom0[0, 1:-1, 1:-1])
    assert np.array_equal(mom[1:7], mom0[1:7] / mom0[0])  # the caller's array, ghosts included
    assert np.array_equal(d["vel"], (mom0[1:4] / mom0[0])[:, 1:-1, 1:-1])
    i, j = 3, 4  # interior cell (nxgs + i, nys + j)
    bz = (uf[2, i + 2, j + 2] + uf[2, i + 3, j + 2] + uf[2, i + 3, j + 2] + uf[2, i + 3, j + 3]) / 4
    assert d["uf"][2, i, j] == bz


def test_particle_and_tracer_files():
    P = small_params()
    rng = np.random.default_rng(5)
    ny, nx = P.nye - P.nys + 1, P.nxge - P.nxgs + 1
    up = np.asfortranarray(rng.standard_normal((6, P.np, ny, P.nsp)))
    pid = rng.integers(-50, 50, (P.np, ny, P.nsp)).astype(np.int64)
    up[5] = pid.view(np.float64)
    np2 = np.asfortranarray(rng.integers(0, P.np + 1, (ny, P.nsp)).astype(np.int32))
    uf = np.asfortranarray(rng.standard_normal((6, nx + 4, ny + 4)))
    for mode, suffix in ((0, "_ptcl"), (1, "_orb")):
        js, raw = PIO.particles(P, up, uf, np2, 42, mode)
        assert json.loads(js)["meta"]["rawfile"] == "0000042%s.raw" % suffix
        d = PIO.read(js, raw)
        assert np.array_equal(d["uf"], uf[:, 2:-2, 2:-2])
        for isp in range(P.nsp):
            want = [up[:, s, j, isp] for j in range(ny) for s in range(np2[j, isp])
                    if mode == 0 or pid[s, j, isp] > 0]
            got = d["up%02d" % (isp + 1)]
            assert got.shape == (6, len(want))
            if want:  # ids are integer bit patterns in the doubles: compare bits
                assert np.array_equal(got.view(np.uint64), np.stack(want, axis=1).view(np.uint64))


def test_param_file():
    P = small_params()
    js, raw = PIO.param(P, 64, 1.0, 0.2, -0.1, 0.004, 0.01, 0.05, "param")
    d = PIO.read(js, raw)
    assert d["n0"][0] == 64 and d["nx"][0] == 8 and d["ny"][0] == 6
    assert d["vai"][0] == 1.0 * 0.004 / 0.2 and d["vae"][0] == 1.0 * -0.1 / 1.0
    assert "dataset" not in json.loads(js)
