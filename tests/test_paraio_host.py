"""The drop-in paraio procedures of the library (wm_paraio_*, host file I/O, no GPU) against the
oracle's restatement of common/paraio.f90: identical JSON text and raw bytes for the snapshot,
parameter, moment, particle and tracer files; paraio__input reads back what was written and
rejects a mismatched module."""
import json

import numpy as np
import pytest

from oracle import paraio as PIO
from wumingpic2d_gb300 import api
from wumingpic2d_gb300._native import WmError

NDIM, NP, NSP = 6, 16, 2
NXGS, NXGE, NYGS, NYGE = 2, 13, 2, 9
Q, R = [-1.0, 1.0], [1.0, 25.0]
DELX, DELT, C = 1.0, 0.5, 1.0


def params():
    return PIO.Params(NDIM, NP, NSP, NXGS, NXGE, NYGS, NYGE, NYGS, NYGE, DELX, DELT, C, Q, R)


@pytest.fixture
def module(tmp_path):
    api.paraio__init(NDIM, NP, NSP, NXGS, NXGE, NYGS, NYGE, NYGS, NYGE, 1, 0, DELX, DELT, C, Q, R, str(tmp_path) + "/")
    yield tmp_path
    api.paraio__finalize()


def state(seed):
    rng = np.random.default_rng(seed)
    nx, ny = NXGE - NXGS + 1, NYGE - NYGS + 1
    up = np.asfortranarray(rng.standard_normal((NDIM, NP, ny, NSP)))
    pid = rng.integers(-1000, 1000, (NP, ny, NSP)).astype(np.int64)
    up[5] = pid.view(np.float64)
    uf = np.asfortranarray(rng.standard_normal((6, nx + 4, ny + 4)))
    np2 = np.asfortranarray(rng.integers(0, NP + 1, (ny, NSP)).astype(np.int32))
    return up, uf, np2


def files(tmp, name):
    return (tmp / (name + ".json")).read_text(), (tmp / (name + ".raw")).read_bytes()


def test_snapshot_bytes_and_input(module):
    up, uf, np2 = state(1)
    api.paraio__output(up, uf, np2, NXGS, NXGE, 77, "snap")
    js, raw = files(module, "snap")
    js_o, raw_o = PIO.output(params(), up, uf, np2, NXGS, NXGE, 77, "snap")
    assert js == js_o and raw == raw_o
    up2, uf2, np22 = np.zeros_like(up, order="F"), np.zeros_like(uf, order="F"), np.zeros_like(np2, order="F")
    assert api.paraio__input(up2, uf2, np22, "snap") == (NXGS, NXGE, 77)
    assert np.array_equal(up2.view(np.uint64), up.view(np.uint64))
    assert np.array_equal(uf2, uf) and np.array_equal(np22, np2)


def test_input_rejects_other_parameters(module):
    up, uf, np2 = state(2)
    api.paraio__output(up, uf, np2, NXGS, NXGE, 1, "snap")
    api.paraio__init(NDIM, NP + 1, NSP, NXGS, NXGE, NYGS, NYGE, NYGS, NYGE, 1, 0, DELX, DELT, C, Q, R, str(module) + "/")
    with pytest.raises(WmError):
        api.paraio__input(np.zeros((NDIM, NP + 1, NYGE - NYGS + 1, NSP), order="F"), uf.copy(order="F"),
                          np2.copy(order="F"), "snap")
    with pytest.raises(WmError):
        api.paraio__input(up.copy(order="F"), uf.copy(order="F"), np2.copy(order="F"), "missing")


def test_param_file(module):
    api.paraio__param(64, 1.0, 0.2, -0.1, 0.004, 0.01, 0.05, "param")
    assert files(module, "param") == PIO.param(params(), 64, 1.0, 0.2, -0.1, 0.004, 0.01, 0.05, "param")


def test_moment_file_and_in_place_division(module):
    rng = np.random.default_rng(3)
    nx, ny = NXGE - NXGS + 1, NYGE - NYGS + 1
    mom = np.asfortranarray(rng.uniform(0.0, 2.0, (7, nx + 2, ny + 2, NSP)))
    mom[0, 0, :, :] = 0.0  # ghost densities of zero: the Fortran divides there too (inf / nan)
    _, uf, _ = state(3)
    mom_o = mom.copy(order="F")
    api.paraio__mom(mom, uf, 123)
    js_o, raw_o = PIO.mom(params(), mom_o, uf, 123)
    assert files(module, "0000123_mom") == (js_o, raw_o)
    assert np.array_equal(mom.view(np.uint64), mom_o.view(np.uint64))


@pytest.mark.parametrize("mode", [0, 1])
def test_particle_and_tracer_files(module, mode):
    up, uf, np2 = state(4 + mode)
    (api.paraio__ptcl if mode == 0 else api.paraio__orb)(up, uf, np2, 9)
    name = "0000009" + ("_ptcl" if mode == 0 else "_orb")
    js, raw = files(module, name)
    assert (js, raw) == PIO.particles(params(), up, uf, np2, 9, mode)
    counts = [json.loads(js)["dataset"]["up%02d" % (s + 1)]["shape"][1] for s in range(NSP)]
    if mode == 1:
        assert 0 < sum(counts) < int(np2.sum())


def test_uninitialised_module_reports():
    api.paraio__finalize()
    up, uf, np2 = state(6)
    with pytest.raises(WmError):
        api.paraio__output(up, uf, np2, NXGS, NXGE, 0, "x")
