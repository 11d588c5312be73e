"""Initial conditions generated on the GPU (wm_sim_init_*) against the oracle's restatement
(oracle/init.py) cell-sorted by the oracle's sort: identical row and cell counts, ids and slot
order; positions bit-exact where they need no transcendental function (FP64 path), momenta to
1e-13 (log, sin/cos, tanh, exp on the two sides)."""
import math

import numpy as np
import pytest

from oracle import init as I
from oracle import oracle as O
from wumingpic2d_gb300.harris import HarrisConfig
from wumingpic2d_gb300.layout import Dims
from wumingpic2d_gb300.shock import ShockConfig
from wumingpic2d_gb300.sim import Simulation

pytestmark = pytest.mark.gpu


def sorted_oracle(d, q, r, state):
    up0, uf, np2 = state
    par = O.make_par(d, 0.5, q, r)
    up, cc = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cc, np2) == 0
    return up, uf, np2, cc


def compare(d, sim, want, pos_exact, precision):
    up_w, uf_w, np2_w, cc_w = want
    up, uf, np2, cc = sim.store(up=d.alloc_up())
    assert np.array_equal(np2, np2_w) and np.array_equal(cc, cc_w)
    n = int(np2.max())
    if precision == "mixed":  # the mixed path keeps its own order inside a cell: match by id
        for isp in range(d.nsp):
            for a in (up, up_w):
                for j in range(d.ny):
                    o = np.argsort(a[5, :n, j, isp].view(np.int64), kind="stable")
                    a[:, :n, j, isp] = a[:, o, j, isp]
    assert np.array_equal(up[5, :n].view(np.int64), up_w[5, :n].view(np.int64))  # ids in the same slots
    if precision == "fp64":
        pos_tol, mom_tol = (0.0 if pos_exact else 1e-12), 1e-13
    else:  # FP32 offsets and momenta
        pos_tol, mom_tol = 1e-6, 1e-6
    for k in range(2):
        assert np.max(np.abs(up[k, :n] - up_w[k, :n])) <= pos_tol * max(d.nx, d.ny), k
    for k in range(2, 5):
        scale = max(np.max(np.abs(up_w[k, :n])), 1e-300)
        assert np.max(np.abs(up[k, :n] - up_w[k, :n])) <= mom_tol * scale, k
    assert np.allclose(uf, uf_w, rtol=1e-13, atol=1e-13 * max(np.max(np.abs(uf_w)), 1e-300))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_weibel_on_device(gpu, precision):
    d = Dims(nx=64, ny=32, np=8 * 64 * 2)
    q, r = np.array([0.02, -0.1]), np.array([25.0, 1.0])
    want = sorted_oracle(d, q, r, I.weibel(d, 8, 0.3, 0.05, 0.01, seed=2024))
    with Simulation(d, 0.5, q, r, precision=precision) as sim:
        sim.init_weibel(8, 0.3, 0.05, 0.01, 2024)
        compare(d, sim, want, True, precision)
        sim.step(2)  # the generated state steps like a loaded one


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_harris_on_device(gpu, precision):
    cfg = HarrisConfig(nx=96, ny=32, seed=77)
    d = cfg.dims()
    vte, vti, wpe, wpi, q, b0, lcs = cfg.plasma()
    want = sorted_oracle(d, q, cfg.mass, I.harris(d, cfg.nbg, cfg.ncs, lcs, b0, cfg.e1, vte, vti, cfg.rtemp, q, seed=77))
    with Simulation(d, cfg.delt, q, cfg.mass, bc="reconnection", precision=precision) as sim:
        sim.init_harris(cfg)
        compare(d, sim, want, False, precision)
        sim.step(2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_shock_on_device(gpu, precision):
    cfg = ShockConfig(nx=128, ny=16, n_ppc=8, tracer_window=(40.0, 60.0), l_damp_ini=8.0)
    d = cfg.dims()
    q = cfg.charge
    args = cfg.init_args()
    want = sorted_oracle(d, q, cfg.mass, I.shock(d, *args[:-1], seed=args[-1]))
    # room for the particles the application injects every step
    with Simulation(d, cfg.delt, q, cfg.mass, bc="shock", u0=cfg.u0, precision=precision,
                    capacity=2 * cfg.n_ppc * d.nx * d.ny) as sim:
        sim.init_shock(cfg)
        compare(d, sim, want, False, precision)
        sim.step(2)


def test_weibel_statistics_at_scale(gpu):
    """512^2 x 16 ppc (8.4M particles per species): the beams and temperatures of the set-up."""
    d = Dims(nx=512, ny=512, np=16 * 512)
    q, r = np.array([0.02, -0.1]), np.array([25.0, 1.0])
    with Simulation(d, 0.5, q, r) as sim:
        sim.init_weibel(16, 0.3, 0.05, 0.01, 7)
        up, uf, np2, cc = sim.store(up=d.alloc_up())
    n = 16 * 512
    assert (np2 == n).all() and not uf.any()
    ud = 0.3 / math.sqrt(1 - 0.09)
    uz = up[4, :n, :, 1].ravel()
    hi, lo = uz[uz > 0], uz[uz < 0]
    assert abs(hi.size - lo.size) < 0.001 * uz.size
    assert abs(hi.mean() - ud) < 1e-3 and abs(lo.mean() + ud) < 1e-3
    assert abs(up[2, :n, :, 1].std() - 0.05) < 1e-3 and abs(up[3, :n, :, 0].std() - 0.01) < 1e-4
    counts = cc[1:, :, 0] - cc[:-1, :, 0]
    assert abs(counts.mean() - 16) < 1e-9 and counts.std() < 6  # Poisson-like cell occupancy
