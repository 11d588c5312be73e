"""Oracle (test infrastructure only): the seeded initial conditions that the library generates on
the GPU (wm_sim_init_weibel / _harris / _shock), restated with numpy.

Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter = (particle index low,
high, call, generator tag), key = the seed; uniforms with 53 bits from two words; normals by the
Box-Muller transform of one draw.  The integer stream and the uniforms are bit-exact with the
device; the normals go through log, sqrt and sin/cos, so they agree to a few units in the last
place.  The physical set-ups follow the applications:

* weibel  -- the Weibel benchmark state of wumingpic2d_gb300/weibel.py (two electron beams along
  z, uniform random positions per row, ids 1..n per species);
* harris  -- proj/reconnection/app.f90:353-470 as wumingpic2d_gb300/harris.py states it;
* shock   -- proj/shock/app.f90:408-525 (evenly spaced x per row, Maxwellian boosted by
  vprofile, app.f90:881-891; ids negative, positive inside [xrs, xre]).
"""
from __future__ import annotations

import math

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)
TAG = {"weibel": 1, "harris": 2, "shock": 3, "inject": 4, "expand": 6}


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised over the counter words (uint32 arrays or scalars); the key is scalar."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) & MASK for x in (c0, c1, c2, c3))
    k0, k1 = int(k0) & 0xFFFFFFFF, int(k1) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        n0 = (p1 >> np.uint64(32)) ^ c1 ^ np.uint64(k0)
        n2 = (p0 >> np.uint64(32)) ^ c3 ^ np.uint64(k1)
        c1 = p1 & MASK
        c3 = p0 & MASK
        c0, c2 = n0, n2
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c0, c1, c2, c3


def uniform53(a, b):
    return ((a >> np.uint64(5)).astype(np.float64) * 67108864.0 + (b >> np.uint64(6)).astype(np.float64)) * (
        1.0 / 9007199254740992.0)


def uniform2(seed, idx, call, tag):
    idx = np.asarray(idx, dtype=np.int64).astype(np.uint64)
    r = philox4x32_10(idx & MASK, idx >> np.uint64(32), np.full(idx.shape, call, np.uint64),
                      np.full(idx.shape, tag, np.uint64), seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    return uniform53(r[0], r[1]), uniform53(r[2], r[3])


def normal2(seed, idx, call, tag):
    u1, u2 = uniform2(seed, idx, call, tag)
    r = np.sqrt(-2.0 * np.log(1.0 - u1))
    return r * np.cos(2.0 * np.pi * u2), r * np.sin(2.0 * np.pi * u2)


def _rows(d, n_row):
    """(slot, row) index grids and the particle index within a species' rows."""
    i = np.arange(n_row, dtype=np.int64)[:, None]
    jr = np.arange(d.ny, dtype=np.int64)[None, :]
    return i, jr, jr * n_row + i


def weibel(d, ppc, v_drift, vth_e, vth_i, seed, delx=1.0):
    """(up, uf, np2) in the reference layout, rows filled in slot order (not cell-sorted)."""
    n_row = ppc * d.nx
    i, jr, idx = _rows(d, n_row)
    t = TAG["weibel"]
    ux, uy = uniform2(seed, idx, 0, t)
    x = (d.nxgs + d.nx * ux) * delx
    y = (d.nys + jr + uy) * delx
    x = np.minimum(x, np.nextafter((d.nxge + 1.0) * delx, 0.0))
    y = np.minimum(y, np.nextafter((d.nys + jr + 1.0) * delx, 0.0))
    n1, n2 = normal2(seed, idx, 1, t)
    n3, n4 = normal2(seed, idx, 2, t)
    n5, n6 = normal2(seed, idx, 3, t)
    ud = v_drift / math.sqrt(1.0 - v_drift * v_drift)
    sign = np.where(i % 2 == 0, 1.0, -1.0)
    up, np2 = d.alloc_up(), d.alloc_np2()
    np2[:, :] = n_row
    pid = (1 + idx).view(np.float64)
    for isp, u in ((0, (vth_i * n1, vth_i * n2, vth_i * n3)), (1, (vth_e * n4, vth_e * n5, vth_e * n6 + sign * ud))):
        up[0, :n_row, :, isp] = x
        up[1, :n_row, :, isp] = y
        for k in range(3):
            up[2 + k, :n_row, :, isp] = u[k]
        up[5, :n_row, :, isp] = pid
    return up, d.alloc_uf(), np2


def harris_rows(nx, nbg, ncs, lcs):
    """Particles per row of proj/reconnection/app.f90:309 (nxge - nxgs = nx - 1)."""
    return int(nbg * (nx - 1) + ncs * 2 * lcs)


def harris(d, nbg, ncs, lcs, b0, e1, vte, vti, rtemp, q, seed, delx=1.0):
    n_row = harris_rows(d.nx, nbg, ncs, lcs)
    i, jr, idx = _rows(d, n_row)
    t = TAG["harris"]
    nxgs, nxge, nygs, nyge = d.nxgs, d.nxge, d.nygs, d.nyge
    x0 = 0.5 * (nxge + nxgs) * delx
    y0 = 0.5 * (nyge - nygs) * delx
    ibg = nbg * (nxge - nxgs - 2)
    ua, ub = uniform2(seed, idx, 0, t)
    xb = (nxgs + 1) * delx + ua * delx * (nxge - nxgs - 2)
    r1 = (2.0 * ua - 1.0) * math.tanh(0.5 * (nxge - nxgs - 2) * delx / lcs)
    xs = lcs * 0.5 * (np.log1p(r1) - np.log1p(-r1)) + x0
    x = np.where(i < ibg, xb, xs)
    y = (d.nys + jr) * delx + ub * delx
    y = np.minimum(y, np.nextafter((d.nys + jr + 1.0) * delx, 0.0))
    g = np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2)
    sech2 = np.cosh((x - x0) / lcs) ** (-2)
    jz = b0 / (4 * math.pi * lcs) * sech2 - 2 * e1 * b0 / (4 * math.pi * lcs) * (1.0 - ((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2) * g
    drift = jz / (ncs * sech2 + nbg)
    f = (1.0 / ((1.0 + rtemp) * q[0]), rtemp / ((1.0 + rtemp) * q[1]))
    n1, n2 = normal2(seed, idx, 1, t)
    n3, n4 = normal2(seed, idx, 2, t)
    n5, n6 = normal2(seed, idx, 3, t)
    up, np2 = d.alloc_up(), d.alloc_np2()
    np2[:, :] = n_row
    pid = (-(1 + idx)).view(np.float64)
    for isp, sd, u in ((0, vti / math.sqrt(2.0), (n1, n2, n3)), (1, vte / math.sqrt(2.0), (n4, n5, n6))):
        up[0, :n_row, :, isp] = x
        up[1, :n_row, :, isp] = y
        up[2, :n_row, :, isp] = sd * u[0]
        up[3, :n_row, :, isp] = sd * u[1]
        up[4, :n_row, :, isp] = sd * u[2] + f[isp] * drift
        up[5, :n_row, :, isp] = pid
    # fields at the integer index * delx on the ghosted grid (app.f90:397-410)
    uf = d.alloc_uf()
    ii = (np.arange(d.nx + 4) + nxgs - 2)[:, None] * delx
    jj = (np.arange(d.ny + 4) + nygs - 2)[None, :] * delx
    gg = np.exp(-((ii - x0) ** 2 + (jj - y0) ** 2) / (2 * lcs) ** 2)
    uf[0] = +e1 * b0 * ((jj - y0) / lcs) * gg
    uf[1] = b0 * np.tanh((ii - x0) / lcs) - e1 * b0 * ((ii - x0) / lcs) * gg
    return up, uf, np2


def vprofile(x, v0, l_damp_ini, nxgs, delx=1.0):
    """proj/shock/app.f90:881-891."""
    x0 = l_damp_ini + nxgs * delx
    xs = l_damp_ini * 0.1
    return 0.5 * v0 * (1 + np.tanh((x - x0) / xs))


def shock(d, n0, u0, vth_e, vth_i, b0, theta_bn, phi_bn, l_damp_ini, xrs, xre, seed, c=1.0, delx=1.0):
    """proj/shock/app.f90:408-525 with nxs = nxgs and nxe = d.nxe (nxge, or nxgs + n_x_ini for the
    expanding box of app.f90:277); the fields over the whole box (:416-426)."""
    nxs, nxe = d.nxgs, d.nxe
    n_row = n0 * (nxe - nxs - 1)  # app.f90:335
    i, jr, idx = _rows(d, n_row)
    t = TAG["shock"]
    gam0 = math.sqrt(1 + u0 * u0 / (c * c))
    v0 = u0 / gam0
    _, uy = uniform2(seed, idx, 0, t)
    # over the cells nxs+1..nxe-1 that np2 and the initial cumcnt fill (app.f90:335-349), not
    # [nxs, nxe) as app.f90:437 writes it (that puts a few particles behind the wall at nxs+1)
    x = np.broadcast_to(((nxs + 1) + (nxe - nxs - 1) * (i + 0.5) / n_row) * delx, (n_row, d.ny))
    y = (d.nys + jr + uy) * delx
    y = np.minimum(y, np.nextafter((d.nys + jr + 1.0) * delx, 0.0))
    n1, n2 = normal2(seed, idx, 1, t)
    n3, n4 = normal2(seed, idx, 2, t)
    n5, n6 = normal2(seed, idx, 3, t)
    v1 = vprofile(x, v0, l_damp_ini, d.nxgs, delx)
    gam1 = 1 / np.sqrt(1 - (v1 / c) ** 2)
    up, np2 = d.alloc_up(), d.alloc_np2()
    np2[:, :] = n_row
    pid = -(1 + idx)
    pid = np.where((x >= xrs) & (x <= xre), -pid, pid)
    for isp, sd, u in ((0, vth_i, (n1, n2, n3)), (1, vth_e, (n4, n5, n6))):
        ux, uyy, uz = sd * u[0], sd * u[1], sd * u[2]
        gamp = np.sqrt(1 + (ux ** 2 + uyy ** 2 + uz ** 2) / c ** 2)
        up[0, :n_row, :, isp] = x
        up[1, :n_row, :, isp] = y
        up[2, :n_row, :, isp] = gam1 * (ux + v1 * gamp)
        up[3, :n_row, :, isp] = uyy
        up[4, :n_row, :, isp] = uz
        up[5, :n_row, :, isp] = pid.view(np.float64)
    uf = d.alloc_uf()
    ii = (np.arange(d.nx + 4) + d.nxgs - 2)[:, None] * delx
    vp = vprofile(ii, v0, l_damp_ini, d.nxgs, delx)
    by = b0 * math.sin(theta_bn) * math.cos(phi_bn)
    bz = b0 * math.sin(theta_bn) * math.sin(phi_bn)
    uf[0] = b0 * math.cos(theta_bn)
    uf[1] = by
    uf[2] = bz
    uf[4] = +vp * bz / c
    uf[5] = -vp * by / c
    return up, uf, np2


def inject_counts(seed, it, pflux, ny):
    """Particles entering each row this step (proj/shock/app.f90:722-754, one rank): int(pflux),
    one more with probability frac(pflux); nginj // ny per row and one more in nginj % ny rows
    drawn at random (the rows whose Philox key ranks lowest)."""
    t = TAG["inject"] + 1
    u, _ = uniform2(seed, np.array([int(it) << 32]), 0, t)
    nginj = int(pflux) + (1 if u[0] < pflux - int(pflux) else 0)
    j = np.arange(ny, dtype=np.uint64)
    keys = philox4x32_10(j, np.full(ny, it, np.uint64), np.ones(ny, np.uint64), np.full(ny, t, np.uint64),
                         seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)[0]
    order = np.lexsort((np.arange(ny), keys))
    rank = np.empty(ny, np.int64)
    rank[order] = np.arange(ny)
    return (nginj // ny + (rank < nginj % ny)).astype(np.int64)


def inject(d, up, uf, np2, cumcnt, it, seed, n0, u0, vth_e, vth_i, b0, theta_bn, phi_bn, l_damp_ini, delt, c=1.0, delx=1.0):
    """proj/shock/app.f90:695-850 on reference-layout arrays, in place: the new particles behind each
    row, np2 and cumcnt(nxe) advanced (the row total column is left as the Fortran leaves it),
    the upstream field at columns nxe-1 and nxe (nxe = d.nxe)."""
    nxe = d.nxe
    gam0 = math.sqrt(1 + u0 * u0 / (c * c))
    v0 = u0 / gam0
    pflux = n0 * abs(v0) * delt * delx * (d.nyge - d.nygs + 1)
    x0 = abs(v0) * delt
    inj = inject_counts(seed, it, pflux, d.ny)
    ninc = np.concatenate(([0], np.cumsum(inj)[:-1]))
    nptot = [int(np2[:, isp].sum()) for isp in range(d.nsp)]
    t = TAG["inject"]
    for jr in range(d.ny):
        n = int(inj[jr])
        if n == 0:
            continue
        k = np.arange(n, dtype=np.int64)
        q = ninc[jr] + k
        uy_draw, _ = uniform2(seed, q, 4 * it + 0, t)
        n1, n2 = normal2(seed, q, 4 * it + 1, t)
        n3, n4 = normal2(seed, q, 4 * it + 2, t)
        n5, n6 = normal2(seed, q, 4 * it + 3, t)
        xb = nxe * delx + (k + 0.5) / n * x0
        y = (d.nys + jr + uy_draw) * delx
        for isp, sd, u in ((0, vth_i, (n1, n2, n3)), (1, vth_e, (n4, n5, n6))):
            ux, uyy, uz = sd * u[0], sd * u[1], sd * u[2]
            x = xb + (v0 + ux) * delt
            v1 = vprofile(x, v0, l_damp_ini, d.nxgs, delx)
            gam1 = 1 / np.sqrt(1 - (v1 / c) ** 2)
            gamp = np.sqrt(1 + (ux ** 2 + uyy ** 2 + uz ** 2) / c ** 2)
            s0 = int(np2[jr, isp])
            up[0, s0:s0 + n, jr, isp] = x
            up[1, s0:s0 + n, jr, isp] = y
            up[2, s0:s0 + n, jr, isp] = gam1 * (ux + v1 * gamp)
            up[3, s0:s0 + n, jr, isp] = uyy
            up[4, s0:s0 + n, jr, isp] = uz
            up[5, s0:s0 + n, jr, isp] = (-(k + 1 + ninc[jr] + nptot[isp])).view(np.float64)
    for isp in range(d.nsp):
        np2[:, isp] += inj.astype(np2.dtype)
        cumcnt[nxe - d.nxgs, :, isp] += inj.astype(cumcnt.dtype)
    by0 = b0 * math.sin(theta_bn) * math.cos(phi_bn)
    bz0 = b0 * math.sin(theta_bn) * math.sin(phi_bn)
    i1, i2 = nxe - 1 - (d.nxgs - 2), nxe - (d.nxgs - 2)
    uf[1, i1, :] = by0
    uf[2, i1, :] = bz0
    uf[4, i1, :] = +v0 * bz0 / c
    uf[5, i1, :] = -v0 * by0 / c
    uf[1, i2, :] = by0
    uf[2, i2, :] = bz0
    return inj


def relocate(d, up, uf, np2, cumcnt, it, seed, n0, u0, vth_e, vth_i, b0, theta_bn, phi_bn, l_damp_ini, c=1.0, delx=1.0):
    """proj/shock/app.f90:613-690 (relocate) on reference-layout arrays, in place, for one rank: the
    box grows by one cell (nxe -> nxe + 1, nothing while nxe = nxge); n0 particles per row and
    species enter cell nxe_new - 1 at x = (nxe_new - 1 + (ii - 1/2)/n0) dx, y = (j + U) dx shared by
    the species, Maxwellian in the fluid rest frame boosted by vprofile(x), behind the row's
    particles, ids -(ii + (j - nygs) n0 + the species' count); np2 += n0; cumcnt(nxe_new) =
    cumcnt(nxe_new - 1) + n0; the upstream field at columns nxe_new - 1 and nxe_new.  The draws
    (random_number in the Fortran) are the Philox stream of this library: counter (row * n0 + k,
    step), tag "expand".  Returns the Dims of the grown box."""
    from dataclasses import replace
    if d.nxe >= d.nxge:
        return d
    nxe = d.nxe + 1
    gam0 = math.sqrt(1 + u0 * u0 / (c * c))
    v0 = u0 / gam0
    nptot = [int(np2[:, isp].sum()) for isp in range(d.nsp)]
    t = TAG["expand"]
    k = np.arange(n0, dtype=np.int64)
    x = (nxe - 1) * delx + (k + 0.5) / n0 * delx
    v1 = vprofile(x, v0, l_damp_ini, d.nxgs, delx)
    gam1 = 1 / np.sqrt(1 - (v1 / c) ** 2)
    for jr in range(d.ny):
        q = jr * n0 + k
        uy_draw, _ = uniform2(seed, q, 4 * it + 0, t)
        n1, n2 = normal2(seed, q, 4 * it + 1, t)
        n3, n4 = normal2(seed, q, 4 * it + 2, t)
        n5, n6 = normal2(seed, q, 4 * it + 3, t)
        y = (d.nys + jr + uy_draw) * delx
        for isp, sd, u in ((0, vth_i, (n1, n2, n3)), (1, vth_e, (n4, n5, n6))):
            ux, uyy, uz = sd * u[0], sd * u[1], sd * u[2]
            gamp = np.sqrt(1 + (ux ** 2 + uyy ** 2 + uz ** 2) / c ** 2)
            s0 = int(np2[jr, isp])
            up[0, s0:s0 + n0, jr, isp] = x
            up[1, s0:s0 + n0, jr, isp] = y
            up[2, s0:s0 + n0, jr, isp] = gam1 * (ux + v1 * gamp)
            up[3, s0:s0 + n0, jr, isp] = uyy
            up[4, s0:s0 + n0, jr, isp] = uz
            up[5, s0:s0 + n0, jr, isp] = (-(k + 1 + jr * n0 + nptot[isp])).view(np.float64)
    for isp in range(d.nsp):
        np2[:, isp] += n0
        cumcnt[nxe - d.nxgs, :, isp] = cumcnt[nxe - 1 - d.nxgs, :, isp] + n0
    by0 = b0 * math.sin(theta_bn) * math.cos(phi_bn)
    bz0 = b0 * math.sin(theta_bn) * math.sin(phi_bn)
    i1, i2 = nxe - 1 - (d.nxgs - 2), nxe - (d.nxgs - 2)
    uf[1, i1, :] = by0
    uf[2, i1, :] = bz0
    uf[4, i1, :] = +v0 * bz0 / c
    uf[5, i1, :] = -v0 * by0 / c
    uf[1, i2, :] = by0
    uf[2, i2, :] = bz0
    return replace(d, nxe_act=nxe)
