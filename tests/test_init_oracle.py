"""The initial-condition restatement (oracle/init.py) on the CPU: Philox4x32-10 against the
published known-answer vectors of Salmon et al. (Random123 kat_vectors), the uniform and normal
transforms, and the generated states' layout and distributions."""
import math

import numpy as np
import pytest

from oracle import init as I
from wumingpic2d_gb300.harris import HarrisConfig
from wumingpic2d_gb300.layout import Dims
from wumingpic2d_gb300.shock import ShockConfig


@pytest.mark.parametrize("ctr,key,want", [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0), (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
])
def test_philox_known_answers(ctr, key, want):
    got = I.philox4x32_10(*ctr, *key)
    assert tuple(int(x) for x in got) == want


def test_uniform_and_normal_transforms():
    idx = np.arange(200000)
    u1, u2 = I.uniform2(99, idx, 0, 1)
    assert u1.min() >= 0.0 and u1.max() < 1.0 and u2.min() >= 0.0 and u2.max() < 1.0
    assert abs(u1.mean() - 0.5) < 0.005 and abs(u2.var() - 1 / 12) < 0.002
    assert np.array_equal(u1, I.uniform2(99, idx, 0, 1)[0])          # a pure function of the counter
    assert not np.array_equal(u1, I.uniform2(100, idx, 0, 1)[0])      # and of the key
    n1, n2 = I.normal2(99, idx, 1, 1)
    for n in (n1, n2):
        assert abs(n.mean()) < 0.01 and abs(n.var() - 1.0) < 0.01
    assert abs(np.corrcoef(n1, n2)[0, 1]) < 0.01


def test_weibel_state():
    d = Dims(nx=32, ny=16, np=8 * 32 * 2)
    up, uf, np2 = I.weibel(d, 8, 0.3, 0.05, 0.01, seed=5)
    n = 8 * 32
    assert (np2 == n).all() and not uf.any()
    x, y = up[0, :n, :, 0], up[1, :n, :, 0]
    assert x.min() >= d.nxgs and x.max() < d.nxge + 1
    rows = np.arange(d.nys, d.nye + 1)[None, :]
    assert ((y >= rows) & (y < rows + 1)).all()
    assert np.array_equal(up[0, :n, :, 0], up[0, :n, :, 1])           # ions and electrons co-located
    ud = 0.3 / math.sqrt(1 - 0.09)
    uz = up[4, :n, :, 1]
    assert abs(uz[0::2].mean() - ud) < 0.01 and abs(uz[1::2].mean() + ud) < 0.01
    assert abs(up[2, :n, :, 0].std() - 0.01) < 0.001
    pid = up[5, :n, :, 0].view(np.int64)
    assert np.array_equal(np.sort(pid.ravel()), np.arange(1, n * d.ny + 1))


def test_harris_state():
    cfg = HarrisConfig(nx=64, ny=16, seed=3)
    d = cfg.dims()
    vte, vti, wpe, wpi, q, b0, lcs = cfg.plasma()
    up, uf, np2 = I.harris(d, cfg.nbg, cfg.ncs, lcs, b0, cfg.e1, vte, vti, cfg.rtemp, q, seed=3)
    n = int(np2[0, 0])
    assert n == I.harris_rows(d.nx, cfg.nbg, cfg.ncs, lcs)
    x = up[0, :n]
    assert x.min() >= d.nxgs + 1 and x.max() < d.nxge
    x0 = 0.5 * (d.nxge + d.nxgs)
    sheet = x[cfg.nbg * (d.nxge - d.nxgs - 2):]
    assert abs(np.median(sheet) - x0) < 0.5 and np.percentile(np.abs(sheet - x0), 50) < 2 * lcs
    assert (up[5, :n].view(np.int64) < 0).all()
    xe = d.nxgs - 2 + (d.nx + 4 - 3)  # x index of the column uf[:, -3]
    assert np.sign(uf[1, 2, 10]) != np.sign(uf[1, -3, 10])
    y0, yj = 0.5 * (d.nyge - d.nygs), d.nygs - 2 + 10
    gg = math.exp(-((xe - x0) ** 2 + (yj - y0) ** 2) / (2 * lcs) ** 2)
    assert abs(uf[1, -3, 10] - (b0 * math.tanh((xe - x0) / lcs) - cfg.e1 * b0 * (xe - x0) / lcs * gg)) < 1e-12 * b0


def test_shock_state():
    cfg = ShockConfig(nx=64, ny=8, n_ppc=4, tracer_window=(20.0, 30.0))
    d = cfg.dims()
    gam0, v0, *_ , q, b0 = cfg.plasma()
    args = cfg.init_args()
    up, uf, np2 = I.shock(d, *args[:-1], seed=args[-1])
    n = int(np2[0, 0])
    assert n == cfg.n_ppc * (d.nxge - d.nxgs - 1)
    x = up[0, :n, 0, 0]
    assert np.all(np.diff(x) > 0) and x[0] >= d.nxgs + 1 and x[-1] < d.nxge
    counts = np.bincount(x.astype(int) - d.nxgs, minlength=d.nx)
    assert counts[0] == 0 and (counts[1:d.nx - 1] == cfg.n_ppc).all() and counts[d.nx - 1] == 0
    pid = up[5, :n, 0, 0].view(np.int64)
    inside = (x >= 20.0) & (x <= 30.0)
    assert (pid[inside] > 0).all() and (pid[~inside] < 0).all()
    # far upstream the plasma drifts at v0 along x (vprofile -> v0)
    far = up[0, :n, :, 1] > d.nxgs + 3 * cfg.l_damp_ini
    ux = up[2, :n, :, 1][far]
    assert abs(ux.mean() - gam0 * v0) < 0.01
    bz = b0 * math.sin(math.pi / 2) * math.sin(math.pi / 2)
    assert np.all(uf[2] == bz)
    assert abs(uf[4, -3, 4] - v0 * bz) < 1e-12 * abs(v0 * bz) and abs(uf[4, 0, 4]) < 1e-3 * abs(v0 * bz)  # motional Ey
