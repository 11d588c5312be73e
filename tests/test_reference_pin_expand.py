"""The shock application's expanding box (proj/shock/app.f90:277 n_x_ini, :123-125 every
intvl_expand steps, relocate :613-690): the common-module routines run over nxs..nxe with nxe below
nxge and growing one cell per step.  The hand restatement (oracle/wm_oracle.c, par.bc = shock) and
the reference's own Fortran translated to C (oracle/f90c.py) are run on the same seeded state
through whole steps in the application's order (push, injection boundary, field solve,
particle_y, sort), each followed by the application's inject and relocate restated in
oracle/init.py on both arrays; the two agree bit for bit.  The relocate restatement itself is
checked for the layout the Fortran gives it (counts, cumcnt, ids, the new cell, the fields)."""
from dataclasses import replace

import numpy as np
import pytest

from oracle import init as I
from oracle import oracle as O
from oracle import reference as R
from wumingpic2d_gb300.shock import ShockConfig

STEPS = 6


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def config():
    return ShockConfig(nx=64, ny=12, n_ppc=6, l_damp_ini=8.0, slack=4.0, seed=23, n_x_ini=30, intvl_expand=1)


def initial(cfg):
    d = replace(cfg.dims(), nxe_act=cfg.dims().nxgs + cfg.n_x_ini)
    a = cfg.init_args()
    up0, uf, np2 = I.shock(d, *a[:-1], seed=a[-1])
    par = O.make_par(d, cfg.delt, cfg.charge, cfg.mass, bc="shock", u0=cfg.u0)
    up, cc = d.alloc_up(), d.alloc_cumcnt()
    assert O.sort_bucket(par, d, up, up0, cc, np2) == 0
    return d, par, up, uf, np2, cc


def app_tail(cfg, d, up, uf, np2, cc, it):
    """inject (app.f90:120) and, every intvl_expand steps, relocate (:123-125)."""
    a = cfg.init_args()
    I.inject(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], cfg.delt)
    if (it + 1) % cfg.intvl_expand == 0:
        d = I.relocate(d, up, uf, np2, cc, it, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7])
    return d


def test_relocate_layout():
    cfg = config()
    d, par, up, uf, np2, cc = initial(cfg)
    n0 = cfg.n_ppc
    np2_0, nxe0 = np2.copy(), d.nxe
    ids0 = {isp: set(up[5, :np2[0, isp], 0, isp].view(np.int64).tolist()) for isp in range(2)}
    a = cfg.init_args()
    d2 = I.relocate(d, up, uf, np2, cc, 0, a[-1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7])
    assert d2.nxe == nxe0 + 1
    assert np.array_equal(np2, np2_0 + n0)
    for isp in range(2):
        for j in range(d.ny):
            new = up[:, np2_0[j, isp]:np2[j, isp], j, isp]
            assert np.all((new[0] > nxe0) & (new[0] < nxe0 + 1))  # the new cell nxe_new - 1 = nxe_old
            assert np.all((new[1] >= d.nys + j) & (new[1] < d.nys + j + 1))
            assert cc[d2.nxe - d.nxgs, j, isp] == cc[d2.nxe - 1 - d.nxgs, j, isp] + n0
        new_ids = up[5, np2_0[0, isp]:np2[0, isp], 0, isp].view(np.int64)
        assert np.all(new_ids < 0) and not set(new_ids.tolist()) & ids0[isp]
    assert np.array_equal(up[1, np2_0[0, 0]:np2[0, 0], 0, 0], up[1, np2_0[0, 1]:np2[0, 1], 0, 1])  # y shared by the species
    i = d2.nxe - (d.nxgs - 2)
    assert np.all(uf[1, i - 1] == uf[1, i]) and np.all(uf[2, i - 1] == uf[2, i])


@pytest.mark.skipif(not R.available(), reason="reference translation unavailable")
def test_expanding_box_steps_match_the_reference():
    O.set_threads(1)
    try:
        cfg = config()
        d, par, up, uf, np2, cc = initial(cfg)
        A = [d, up, up.copy(order="F"), uf, cc, np2]
        B = [d, up.copy(order="F"), up.copy(order="F"), uf.copy(order="F"), cc.copy(order="F"), np2.copy(order="F")]
        ref = R.Reference(d, cfg.delt, cfg.charge, cfg.mass, bc="shock")
        S = O.OracleState(d)
        for it in range(STEPS):
            dA, upA, gpA, ufA, ccA, np2A = A
            status, _ = O.step(par, dA, upA, gpA, ufA, ccA, np2A, S)
            assert status == 0
            A[0] = app_tail(cfg, dA, upA, ufA, np2A, ccA, it)
            dB, upB, gpB, ufB, ccB, np2B = B
            ref.d = dB
            assert ref.particle_solv(gpB, upB, ufB, ccB) == 0
            assert ref.bc_injection(gpB, np2B, cfg.u0) == 0
            assert ref.field_fdtd_i(ufB, upB, gpB, ccB) == 0
            assert ref.bc_particle_y(gpB, np2B) == 0
            assert ref.sort_bucket(upB, gpB, ccB, np2B) == 0
            B[0] = app_tail(cfg, dB, upB, ufB, np2B, ccB, it)
        assert A[0].nxe == B[0].nxe == d.nxe + STEPS
        assert np.array_equal(A[5], B[5]) and np.array_equal(A[4], B[4])
        assert np.array_equal(bits(A[1]), bits(B[1]))
        assert np.array_equal(bits(A[3]), bits(B[3]))
        df_r, uj_r, _ = ref.get_work()
        assert np.array_equal(bits(S.df), bits(df_r)) and np.array_equal(bits(S.uj), bits(uj_r))
    finally:
        O.set_threads(O.num_threads())
