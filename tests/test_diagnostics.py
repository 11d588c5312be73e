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
