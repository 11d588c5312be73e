"""The CPU restatement against known answers and conservation laws (no GPU).

The reference ships no test vectors for its hot path, so these pin the oracle:
analytic Boris results, Esirkepov charge conservation (div E - 4 pi rho is
invariant), the CG residual bound, the stable counting sort against numpy, the
closed-form particle_y permutation used by the GPU against the oracle's
sequential loop, and the periodic ghost patterns against numpy.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import State, periodic_ghosts, rel_err
from wumingpic2d_gb300.layout import Dims


def _single_particle_state(nx=8, ny=8, u=(0.1, 0.2, -0.05), x=(5.3, 4.7), np_=4):
    d = Dims(nx=nx, ny=ny, np=np_)
    up = d.alloc_up()
    np2 = d.alloc_np2()
    j = int(x[1])
    up[0, 0, j - d.nys, 0] = x[0]
    up[1, 0, j - d.nys, 0] = x[1]
    up[2:5, 0, j - d.nys, 0] = u
    np2[j - d.nys, 0] = 1
    cum = d.alloc_cumcnt()
    gp = d.alloc_up()
    return d, up, gp, np2, cum


def _sorted(d, par, up, np2):
    out = d.alloc_up()
    cum = d.alloc_cumcnt()
    assert O.sort_bucket(par, d, out, up, cum, np2) == 0
    return out, cum


def test_boris_pure_B_conserves_momentum_magnitude():
    d = Dims(nx=16, ny=16, np=64)
    st = State(nx=16, ny=16, ppc=4)
    par = st.par
    uf = d.alloc_uf()
    rng = np.random.default_rng(0)
    uf[0:3] = 0.3 * rng.standard_normal(uf[0:3].shape)
    periodic_ghosts(uf, 16, 16)
    gp = st.gp.copy(order="F")
    O.particle_solv(par, st.d, gp, st.up, uf, st.cumcnt)
    for isp in range(2):
        for j in range(16):
            n = st.np2[j, isp]
            u0 = np.linalg.norm(st.up[2:5, :n, j, isp], axis=0)
            u1 = np.linalg.norm(gp[2:5, :n, j, isp], axis=0)
            assert np.max(np.abs(u1 - u0) / u0) < 1e-13


def test_uniform_E_kick_is_analytic():
    d, up, gp, np2, _ = _single_particle_state()
    q, r, dt = np.array([0.3, -0.3]), np.array([4.0, 1.0]), 0.5
    par = O.make_par(d, dt, q, r)
    up, cum = _sorted(d, par, up, np2)
    uf = d.alloc_uf()
    E = np.array([0.01, -0.02, 0.005])
    uf[3:6] = E[:, None, None]
    O.particle_solv(par, d, gp, up, uf, cum)
    j = int(up[1, 0, :, 0].max()) - d.nys
    expect = up[2:5, 0, j, 0] + q[0] / r[0] * dt * E
    assert np.allclose(gp[2:5, 0, j, 0], expect, rtol=0, atol=1e-15)


def test_gyration_angle_is_boris_rotation():
    d, up, gp, np2, _ = _single_particle_state(u=(0.2, 0.0, 0.0))
    q, r, dt, B = np.array([0.5, -0.5]), np.array([2.0, 1.0]), 0.5, 0.4
    par = O.make_par(d, dt, q, r)
    up, cum = _sorted(d, par, up, np2)
    uf = d.alloc_uf()
    uf[2] = B
    O.particle_solv(par, d, gp, up, uf, cum)
    j = int(up[1, 0, :, 0].max()) - d.nys
    u0 = up[2:4, 0, j, 0]
    u1 = gp[2:4, 0, j, 0]
    gam = math.sqrt(1 + u0 @ u0)
    t = q[0] / r[0] * 0.5 * dt * B / gam
    expected = -2 * math.atan(t)  # positive charge rotates clockwise about +z
    got = math.atan2(u0[0] * u1[1] - u0[1] * u1[0], u0 @ u1)
    assert abs(got - expected) < 1e-14


def _rho_tsc(d, up, np2, q):
    rho = np.zeros((d.nx, d.ny))
    for isp in range(d.nsp):
        for jj in range(d.ny):
            n = np2[jj, isp]
            x, y = up[0, :n, jj, isp], up[1, :n, jj, isp]
            i, j = x.astype(int), y.astype(int)
            hx, hy = x - 0.5 - i, y - 0.5 - j
            sx = [0.5 * (0.5 - hx) ** 2, 0.75 - hx**2, 0.5 * (0.5 + hx) ** 2]
            sy = [0.5 * (0.5 - hy) ** 2, 0.75 - hy**2, 0.5 * (0.5 + hy) ** 2]
            for a in range(3):
                for b in range(3):
                    np.add.at(rho, ((i + a - 1 - d.nxgs) % d.nx, (j + b - 1 - d.nygs) % d.ny), q[isp] * sx[a] * sy[b])
    return rho


def _div_e(d, uf):
    ex = uf[3, 2:d.nx + 3, 2:d.ny + 2]
    ey = uf[4, 2:d.nx + 2, 2:d.ny + 3]
    return (ex[1:, :] - ex[:-1, :]) + (ey[:, 1:] - ey[:, :-1])


def test_esirkepov_keeps_gauss_law_invariant():
    st = State(nx=24, ny=20, ppc=6, seed=3, field_amp=0.0)
    O.set_threads(1)
    S = st.oracle_state()
    q = st.cfg.charge
    g0 = _div_e(st.d, st.uf) - 4 * np.pi * _rho_tsc(st.d, st.up, st.np2, q)
    scale = np.max(np.abs(4 * np.pi * _rho_tsc(st.d, st.up, st.np2, np.abs(q))))
    for _ in range(6):
        stt, _ = O.step(st.par, st.d, st.up, st.gp, st.uf, st.cumcnt, st.np2, S)
        assert stt == 0
        g = _div_e(st.d, st.uf) - 4 * np.pi * _rho_tsc(st.d, st.up, st.np2, q)
        assert np.max(np.abs(g - g0)) < 1e-13 * scale


def _apply_A(phi, f4):
    return f4 * phi - (np.roll(phi, 1, 0) + np.roll(phi, -1, 0) + np.roll(phi, 1, 1) + np.roll(phi, -1, 1))


def test_cg_meets_its_residual_tolerance():
    st = State(nx=32, ny=24, ppc=6, field_amp=0.05, df_amp=1e-3)
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    S = st.oracle_state()
    stt, iters = O.field_fdtd_i(st.par, st.d, st.uf.copy(order="F"), st.up, gp, st.cumcnt, S)
    assert stt == 0 and np.all(iters > 0)
    c, dt, dx, g = st.par.c, st.par.delt, st.par.delx, st.par.gfac
    f5 = (dx / (c * dt * g)) ** 2
    f4 = 4.0 + f5
    for l in range(3):
        b = f5 * S.gkl[l]
        x = S.df[l, 2:-2, 2:-2]
        res = np.linalg.norm(b - _apply_A(x, f4)) / np.linalg.norm(b)
        assert res < 1e-6


def test_cg_iteration_limit_is_reported():
    st = State(nx=16, ny=16, ppc=4, field_amp=0.05)
    st.par.cg_itemax = 1
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    stt, _ = O.field_fdtd_i(st.par, st.d, st.uf.copy(order="F"), st.up, gp, st.cumcnt, st.oracle_state())
    assert stt == O.ERR_CG_MAXITER


def test_sort_is_stable_counting_sort():
    st = State(nx=20, ny=10, ppc=7, field_amp=0.05)
    gp = st.gp.copy(order="F")
    O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
    O.bc_particle_x(st.par, st.d, gp, st.np2)
    np2 = st.np2.copy(order="F")
    assert O.bc_particle_y(st.par, st.d, gp, np2) == 0
    out, cum = st.d.alloc_up(), st.d.alloc_cumcnt()
    assert O.sort_bucket(st.par, st.d, out, gp, cum, np2) == 0
    for isp in range(2):
        for j in range(st.d.ny):
            n = np2[j, isp]
            cell = gp[0, :n, j, isp].astype(int)
            order = np.argsort(cell, kind="stable")
            assert np.array_equal(out[:, :n, j, isp].view(np.int64), gp[:, order, j, isp].view(np.int64))
            counts = np.bincount(cell - st.d.nxs, minlength=st.d.nx)
            assert np.array_equal(cum[:, j, isp], np.concatenate([[0], np.cumsum(counts)]))


def test_sort_reports_out_of_grid():
    st = State(nx=8, ny=8, ppc=2)
    bad = st.up.copy(order="F")
    bad[0, 0, 0, 0] = st.d.nxge + 3.0
    assert O.sort_bucket(st.par, st.d, st.d.alloc_up(), bad, st.d.alloc_cumcnt(), st.np2) == O.ERR_CELL


# ----------------------------------------------------------------- particle_y
def closed_form_particle_y(d, up, np2):
    """The GPU's particle_y formulation (slot P of every particle) in numpy, one species at a time."""
    out = up.copy(order="F")
    np2_new = np2.copy(order="F")
    ny = d.ny
    for isp in range(d.nsp):
        # classify with the wrap applied in place (round-down additions of ny*delx are exact here)
        dirs, ords, holes = [], [], []
        nup, ndown = np.zeros(ny, int), np.zeros(ny, int)
        for jr in range(ny):
            n = np2[jr, isp]
            y = out[1, :n, jr, isp]
            jpos = np.floor(y).astype(int)
            j = d.nys + jr
            dr = np.where(jpos == j + 1, 1, np.where(jpos == j - 1, 2, 0))
            assert np.all((jpos == j) | (dr != 0))
            wrap_lo, wrap_hi = jpos <= d.nygs - 1, jpos >= d.nyge + 1
            up_wrap = y + ny  # the reference adds in round-down mode: undo a round-up
            up_wrap = np.where(up_wrap - ny > y, np.nextafter(up_wrap, -np.inf), up_wrap)
            out[1, :n, jr, isp] = np.where(wrap_lo, up_wrap, np.where(wrap_hi, y - ny, y))
            leave = dr != 0
            L = np.cumsum(leave) - leave
            o = np.where(dr == 0, L, np.where(dr == 1, np.cumsum(dr == 1) - (dr == 1), np.cumsum(dr == 2) - (dr == 2)))
            dirs.append(dr)
            ords.append(o)
            holes.append(np.nonzero(leave)[0] + 1)
            nup[jr], ndown[jr] = np.sum(dr == 1), np.sum(dr == 2)

        def incoming(k):
            kin = 0
            if k > 0:
                kin += nup[k - 1]
            if k < ny - 1:
                kin += ndown[k + 1]
            if k == ny - 1:
                kin += ndown[0]
            if k == 0:
                kin += nup[ny - 1]
            return kin

        src = out[:, :, :, isp].copy(order="F")
        for jr in range(ny):
            N = np2[jr, isp]
            for s in range(N):
                dr, o = dirs[jr][s], ords[jr][s]
                if dr == 0:
                    k, m, kin = jr, nup[jr] + ndown[jr], incoming(jr)
                    P = s + 1
                    if kin < m and P > N + kin - m:
                        rr = (N - P) - (m - o) + 1
                        P = holes[jr][kin + rr - 1]
                else:
                    if dr == 1:
                        k, off = (jr + 1, 0) if jr < ny - 1 else (0, ndown[1] if ny > 1 else ndown[0])
                    else:
                        k, off = (jr - 1, nup[jr - 2] if jr - 1 > 0 else 0) if jr > 0 else (ny - 1, nup[ny - 2] if ny > 1 else 0)
                    t = off + o + 1
                    m = nup[k] + ndown[k]
                    P = holes[k][t - 1] if t <= m else np2[k, isp] + t - m
                out[:, P - 1, k, isp] = src[:, s, jr]
        for jr in range(ny):
            np2_new[jr, isp] = np2[jr, isp] + incoming(jr) - nup[jr] - ndown[jr]
    return out, np2_new


def _crafted_rows(ny, nrow, probs, seed, nx=8, np_slots=None):
    rng = np.random.default_rng(seed)
    np_slots = np_slots or 4 * nrow + 8
    d = Dims(nx=nx, ny=ny, np=np_slots)
    up = d.alloc_up()
    np2 = d.alloc_np2()
    for isp in range(2):
        for jr in range(ny):
            n = int(rng.integers(0, nrow + 1)) if probs is None else nrow
            p_up, p_dn = probs[jr % len(probs)] if probs is not None else rng.uniform(0, 0.5, 2)
            u = rng.random(n)
            move = np.where(u < p_up, 1, np.where(u < p_up + p_dn, -1, 0))
            j = d.nys + jr
            up[1, :n, jr, isp] = j + move + rng.uniform(0.001, 0.999, n)
            up[0, :n, jr, isp] = d.nxgs + d.nx * rng.random(n)
            up[2:5, :n, jr, isp] = rng.standard_normal((3, n))
            up[5, :n, jr, isp] = (-(1 + np.arange(n) + 1000 * jr + 10**6 * isp)).astype(np.int64).view(np.float64)
            np2[jr, isp] = n
    return d, up, np2


@pytest.mark.parametrize("ny", [1, 2, 3, 5, 8])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_particle_y_closed_form_matches_sequential_loop(ny, seed):
    d, up, np2 = _crafted_rows(ny, nrow=30, probs=None, seed=seed + 17 * ny)
    par = O.make_par(d, 0.5, [1.0, -1.0], [1.0, 1.0])
    ref, np2_ref = up.copy(order="F"), np2.copy(order="F")
    assert O.bc_particle_y(par, d, ref, np2_ref) == 0
    got, np2_got = closed_form_particle_y(d, up, np2)
    assert np.array_equal(np2_got, np2_ref)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))


@pytest.mark.parametrize("probs", [
    [(0.9, 0.05), (0.0, 0.0), (0.0, 0.9)],   # rows emptied, rows receiving many
    [(0.5, 0.5)],                            # everybody leaves
    [(0.0, 0.0)],                            # nobody moves
    [(0.3, 0.0), (0.0, 0.3)],                # imbalanced flux both ways
])
def test_particle_y_closed_form_extreme_flux(probs):
    d, up, np2 = _crafted_rows(6, nrow=40, probs=probs, seed=5)
    par = O.make_par(d, 0.5, [1.0, -1.0], [1.0, 1.0])
    ref, np2_ref = up.copy(order="F"), np2.copy(order="F")
    assert O.bc_particle_y(par, d, ref, np2_ref) == 0
    got, np2_got = closed_form_particle_y(d, up, np2)
    assert np.array_equal(np2_got, np2_ref)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))


def test_particle_y_overflow_is_reported():
    d, up, np2 = _crafted_rows(4, nrow=40, probs=[(0.9, 0.0), (0.0, 0.0)], seed=2, np_slots=48)
    par = O.make_par(d, 0.5, [1.0, -1.0], [1.0, 1.0])
    assert O.bc_particle_y(par, d, up, np2) == O.ERR_OVERFLOW


def test_particle_x_wraps_with_round_down():
    d = Dims(nx=256, ny=4, np=4)
    par = O.make_par(d, 0.5, [1.0, -1.0], [1.0, 1.0])
    up = d.alloc_up()
    np2 = d.alloc_np2()
    lo = np.nextafter(2.0, 0.0)
    up[0, 0, 0, 0] = lo
    up[0, 1, 0, 0] = 258.0
    up[0, 2, 0, 0] = 100.25
    np2[0, 0] = 3
    O.bc_particle_x(par, d, up, np2)
    assert up[0, 0, 0, 0] < 258.0 and int(up[0, 0, 0, 0]) == 257  # round-to-nearest would give 258.0
    assert up[0, 1, 0, 0] == 2.0 and up[0, 2, 0, 0] == 100.25


# ---------------------------------------------------------------- ghost patterns
def test_dfield_ghosts_are_periodic_copies():
    st = State(nx=10, ny=8, ppc=1)
    rng = np.random.default_rng(1)
    df = np.asfortranarray(rng.standard_normal((6, 14, 12)))
    O.bc_dfield(st.par, st.d, df)
    ref = df.copy()
    periodic_ghosts(ref, 10, 8)
    assert np.array_equal(df, ref)


def test_curre_fold_conserves_total_current():
    st = State(nx=10, ny=8, ppc=1)
    rng = np.random.default_rng(2)
    uj = np.asfortranarray(rng.standard_normal((3, 14, 12)))
    total = uj.sum(axis=(1, 2))
    O.bc_curre(st.par, st.d, uj)
    assert np.allclose(uj[:, 2:12, 2:10].sum(axis=(1, 2)), total, rtol=1e-13)
    ref = uj.copy()
    periodic_ghosts(ref, 10, 8)
    assert np.array_equal(uj, ref)


def test_mom_fold_conserves_total():
    st = State(nx=10, ny=8, ppc=1)
    rng = np.random.default_rng(4)
    mom = np.asfortranarray(rng.standard_normal((7, 12, 10, 2)))
    total = mom.sum(axis=(1, 2))
    O.bc_mom(st.par, st.d, mom)
    assert np.allclose(mom[:, 1:11, 1:9].sum(axis=(1, 2)), total, rtol=1e-13)


def test_energy_matches_numpy():
    st = State(nx=16, ny=12, ppc=5, field_amp=0.1)
    e = O.energy(st.par, st.d, st.up, st.uf, st.np2)
    ke = []
    for isp in range(2):
        u = np.concatenate([st.up[2:5, :st.np2[j, isp], j, isp] for j in range(st.d.ny)], axis=1)
        ke.append(st.cfg.mass[isp] * np.sum(np.sqrt(1 + np.sum(u * u, axis=0)) - 1))
    inner = st.uf[:, 2:-2, 2:-2]
    ee = np.sum(inner[3:6] ** 2) / (8 * np.pi)
    bb = np.sum(inner[0:3] ** 2) / (8 * np.pi)
    assert rel_err(e, np.array(ke + [ee, bb])) < 1e-13


def test_thread_count_does_not_change_particle_results():
    st = State(nx=24, ny=16, ppc=6, field_amp=0.05)
    outs = []
    for th in (1, 4):
        O.set_threads(th)
        gp = st.gp.copy(order="F")
        O.particle_solv(st.par, st.d, gp, st.up, st.uf, st.cumcnt)
        outs.append(gp)
    O.set_threads(1)
    assert np.array_equal(outs[0].view(np.int64), outs[1].view(np.int64))


def test_particle_x_round_down_at_any_thread_count():
    d = Dims(nx=256, ny=16, np=8)
    par = O.make_par(d, 0.5, [1.0, -1.0], [1.0, 1.0])
    up = d.alloc_up()
    np2 = d.alloc_np2()
    up[0, :4, :, :] = np.nextafter(2.0, 0.0)
    np2[:, :] = 4
    outs = []
    for th in (1, 4):
        O.set_threads(th)
        a = up.copy(order="F")
        O.bc_particle_x(par, d, a, np2)
        outs.append(a)
    O.set_threads(1)
    assert np.array_equal(outs[0], outs[1])
    assert np.all(outs[1][0, :4] < 258.0)
