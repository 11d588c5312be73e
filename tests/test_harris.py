"""The seeded Harris-sheet initial condition (proj/reconnection/app.f90:265-470)."""
import math

import numpy as np

from wumingpic2d_gb300.harris import HarrisConfig, harris_state
from wumingpic2d_gb300.layout import bits_to_pid


def test_harris_state_layout_and_physics():
    cfg = HarrisConfig(nx=96, ny=32, nbg=2, ncs=10, seed=3)
    d = cfg.dims()
    up, uf, np2 = harris_state(cfg)
    n = cfg.per_row()
    assert np.all(np2 == n) and n <= d.np
    vte, vti, wpe, wpi, q, b0, lcs = cfg.plasma()
    assert q[0] > 0 > q[1] and b0 > 0
    # the reference's sample parameters: omega_pe/omega_ce = alpha, lcs in c/omega_pi
    assert abs(wpe / (abs(q[1]) * b0 / cfg.c) - cfg.alpha) < 1e-12
    assert abs(lcs - cfg.lcs * cfg.c / wpi) < 1e-12
    x = up[0, :n]
    assert np.all(x >= d.nxgs + 1) and np.all(x < d.nxge)  # inside the walls
    assert np.array_equal(up[0:2, :n, :, 0], up[0:2, :n, :, 1])  # ions and electrons co-located
    y = up[1, :n, :, 0]
    assert np.all(np.floor(y) == d.nys + np.arange(d.ny)[None, :])
    # By reverses across the sheet; the perturbation is odd about the X point
    x0 = 0.5 * (d.nxge + d.nxgs)
    ix = np.arange(d.nx + 4) + d.nxgs - 2
    by = uf[1, :, d.ny // 2 + 2]
    assert np.all(np.sign(by[ix < x0 - 3 * lcs]) < 0) and np.all(np.sign(by[ix > x0 + 3 * lcs]) > 0)
    # electron drift carries the sheet current against the ions' (f1, f2 of app.f90:414-415)
    centre = np.abs(up[0, :n, :, 1] - x0) < 0.5 * lcs
    assert up[4, :n, :, 0][centre].mean() > 0 > up[4, :n, :, 1][centre].mean()
    pid = bits_to_pid(up[5, :n, :, 0])
    assert pid.max() == -1 and np.unique(pid).size == pid.size


def test_harris_config_3_sizes():
    cfg = HarrisConfig(nx=4096, ny=2048)
    # 64 particles per cell per species at the sheet centre, background 6 (0.094 of the peak)
    assert cfg.n0 == 64
    total = 2 * cfg.per_row() * cfg.ny
    assert 1.0e8 < total < 1.3e8
    assert math.isclose(cfg.plasma()[6], 0.5 * cfg.c / cfg.plasma()[3])
