"""Host-side run diagnostics: growth-rate fit and the Gauss-law residual."""
import numpy as np

from wumingpic2d_gb300.diagnostics import charge_density, div_e, growth_rate
from wumingpic2d_gb300.weibel import WeibelConfig, weibel_particles


def test_growth_rate_recovers_an_exponential_phase():
    t = np.linspace(0, 100, 501)
    gamma = 0.23
    # noise floor, exponential growth, then saturation
    e_b = np.minimum(1e-12 + 1e-14 * np.exp(2 * gamma * t), 1e-3)
    g, t0, t1 = growth_rate(t, e_b)
    assert abs(g - gamma) <= 1e-3 * gamma
    assert 0 < t0 < t1 < 100


def test_growth_rate_without_growth_is_nan():
    g, _, _ = growth_rate(np.arange(10.0), np.zeros(10))
    assert np.isnan(g)


def test_charge_density_sums_to_total_charge():
    cfg = WeibelConfig(nx=16, ny=12, ppc=4, seed=3)
    d = cfg.dims()
    up, np2 = weibel_particles(cfg)
    q = np.array([1.0, 0.0])
    rho = charge_density(d, up, np2, q)
    assert abs(rho.sum() - np2[:, 0].sum()) <= 1e-9 * np2[:, 0].sum()
    # ions and electrons co-located with opposite unit charges: no net charge anywhere
    assert np.max(np.abs(charge_density(d, up, np2, np.array([1.0, -1.0])))) <= 1e-12


def test_div_e_of_a_uniform_field_is_zero():
    cfg = WeibelConfig(nx=8, ny=6, ppc=1)
    d = cfg.dims()
    uf = d.alloc_uf()
    uf[3] = 0.7
    uf[4] = -0.2
    assert np.max(np.abs(div_e(d, uf))) == 0.0


def test_strip_gauss_residual_matches_the_full_grid():
    """The row-strip Gauss residual of the long-run check equals the full-grid one on its rows."""
    from oracle import oracle as O
    from wumingpic2d_gb300.diagnostics import gauss_residual
    from wumingpic2d_gb300.validate import strip_gauss
    from wumingpic2d_gb300.weibel import WeibelConfig, weibel_particles

    cfg = WeibelConfig(nx=16, ny=12, ppc=4, seed=3, slack=2)
    d = cfg.dims()
    up0, np2 = weibel_particles(cfg)
    par = O.make_par(d, cfg.delt, cfg.charge, cfg.mass)
    up, cc = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cc, np2) == 0
    uf = d.alloc_uf()
    uf[:] = np.random.default_rng(1).standard_normal(uf.shape)
    full = gauss_residual(d, up, uf, np2, cfg.charge)
    for j0, k in ((0, 4), (5, 3), (9, 3)):
        assert np.allclose(strip_gauss(d, up, uf, np2, cfg.charge, j0, k), full[:, j0:j0 + k], rtol=0, atol=1e-12)
