// wm_init.cu -- seeded initial conditions generated on the GPU.
//
// One thread per (row, slot) writes that slot of both species into a reference-layout stage
// (6 doubles per slot, rows species-major), which the resident simulation then unpacks and
// cell-sorts like a host load -- no host round trip for the 5e8-particle states.  Random numbers
// are Philox4x32-10 draws keyed by the seed and counted by (particle, draw, generator), so a state
// does not depend on the launch shape (wm_rng.cuh).
//
//   weibel   the two-beam Weibel state of the benchmark (uniform positions per row, electrons
//            drifting +/- along z by slot parity)
//   harris   proj/reconnection/app.f90:353-470: background uniform in [nxgs+1, nxge-1), sheet
//            particles x0 + lcs atanh(r) (the logistic draw of :429-433), drifts jz/n split by
//            the temperature ratio (:440-446), fields tanh(x) By + the e1 perturbation
//   shock    proj/shock/app.f90:408-525 with the box at full size: x evenly spaced per row,
//            Maxwellian boosted along x by vprofile (:881-891), ids negative except in the
//            tracer window [xrs, xre]; uniform B and the motional E of vprofile
#include "wm_launch.cuh"
#include "wm_rng.cuh"

namespace {

__device__ __forceinline__ void put(double *a, double x, double y, double ux, double uy, double uz, long long pid)
{
    a[0] = x;
    a[1] = y;
    a[2] = ux;
    a[3] = uy;
    a[4] = uz;
    a[5] = __longlong_as_double(pid);
}

__device__ __forceinline__ double below(double v, double hi) { return fmin(v, nextafter(hi, 0.0)); }

// proj/shock/app.f90:881-891
__device__ __forceinline__ double vprofile(double x, double v0, double l_damp_ini, double nxgs_delx)
{
    const double x0 = l_damp_ini + nxgs_delx;
    const double xs = l_damp_ini * 0.1;
    return 0.5 * v0 * (1 + tanh((x - x0) / xs));
}
__device__ __forceinline__ double vprofile(double x, const WmInitArgs &a) { return vprofile(x, a.v0, a.l_damp_ini, a.nxgs_delx); }

__global__ void k_init_particles(WmGeom g, WmInitArgs a, double *__restrict__ stage)
{
    const long long n = (long long)a.n_row * g.ny;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int jr = (int)(t / a.n_row), i = (int)(t % a.n_row);
    const long long idx = (long long)jr * a.n_row + i;  // place in the species' rows
    const double delx = a.delx;
    const double jrow = (double)(g.nys + jr);
    double *s0 = stage + 6 * ((long long)jr * a.n_row + i);
    double *s1 = stage + 6 * ((long long)(g.ny + jr) * a.n_row + i);
    double n1, n2, n3, n4, n5, n6, ua, ub;
    wm_rng_uniform2(a.seed, idx, 0, a.tag, ua, ub);
    wm_rng_normal2(a.seed, idx, 1, a.tag, n1, n2);
    wm_rng_normal2(a.seed, idx, 2, a.tag, n3, n4);
    wm_rng_normal2(a.seed, idx, 3, a.tag, n5, n6);
    if (a.tag == WM_RNG_WEIBEL) {
        const double x = below((g.nxgs + g.nx * ua) * delx, (g.nxge + 1.0) * delx);
        const double y = below((jrow + ub) * delx, (jrow + 1.0) * delx);
        const double sign = (i % 2 == 0) ? 1.0 : -1.0;
        put(s0, x, y, a.vth_i * n1, a.vth_i * n2, a.vth_i * n3, 1 + idx);
        put(s1, x, y, a.vth_e * n4, a.vth_e * n5, a.vth_e * n6 + sign * a.ud, 1 + idx);
    } else if (a.tag == WM_RNG_HARRIS) {
        const int nxgs = g.nxgs, nxge = g.nxge;
        double x;
        if (i < a.ibg) {
            x = (nxgs + 1) * delx + ua * delx * (nxge - nxgs - 2);
        } else {
            const double r1 = (2.0 * ua - 1.0) * a.tanh_edge;
            x = a.lcs * 0.5 * (log1p(r1) - log1p(-r1)) + a.x0;
        }
        const double y = below(jrow * delx + ub * delx, (jrow + 1.0) * delx);
        const double dx = x - a.x0, dy = y - a.y0, w2 = (2 * a.lcs) * (2 * a.lcs);
        const double gg = exp(-(dx * dx + dy * dy) / w2);
        const double ch = cosh(dx / a.lcs);
        const double sech2 = 1.0 / (ch * ch);
        const double jz = a.b0 / (4 * WM_PI * a.lcs) * sech2 - 2 * a.e1 * a.b0 / (4 * WM_PI * a.lcs) * (1.0 - (dx * dx + dy * dy) / w2) * gg;
        const double drift = jz / (a.ncs * sech2 + a.nbg);
        const double sdi = a.vth_i / sqrt(2.0), sde = a.vth_e / sqrt(2.0);
        put(s0, x, y, sdi * n1, sdi * n2, sdi * n3 + a.f1 * drift, -(1 + idx));
        put(s1, x, y, sde * n4, sde * n5, sde * n6 + a.f2 * drift, -(1 + idx));
    } else {  // shock
        const int nxs = g.nxgs, nxe = g.nxgs + g.nxa - 1;  // nxe = nxgs + n_x_ini (proj/shock/app.f90:277)
        // evenly over the cells nxs+1..nxe-1 that np2 = n0 (nxe-nxs-1) and the initial cumcnt
        // (app.f90:335-349) give n0 each; app.f90:437 spreads them over [nxs, nxe), which puts a
        // few behind the wall at nxs+1, where the first reflection moves them by more than a cell
        const double x = ((nxs + 1) + (nxe - nxs - 1) * (i + 0.5) / a.n_row) * delx;
        const double y = below((jrow + ub) * delx, (jrow + 1.0) * delx);
        const double v1 = vprofile(x, a);
        const double gam1 = 1 / sqrt(1 - (v1 / a.c) * (v1 / a.c));
        long long pid = -(1 + idx);
        if (x >= a.xrs && x <= a.xre) pid = -pid;
        const double c2 = a.c * a.c;
        {
            const double ux = a.vth_i * n1, uy = a.vth_i * n2, uz = a.vth_i * n3;
            const double gamp = sqrt(1 + (ux * ux + uy * uy + uz * uz) / c2);
            put(s0, x, y, gam1 * (ux + v1 * gamp), uy, uz, pid);
        }
        {
            const double ux = a.vth_e * n4, uy = a.vth_e * n5, uz = a.vth_e * n6;
            const double gamp = sqrt(1 + (ux * ux + uy * uy + uz * uz) / c2);
            put(s1, x, y, gam1 * (ux + v1 * gamp), uy, uz, pid);
        }
    }
}

// Fields on the ghosted grid at the integer index * delx (planes of x-fastest rows).
__global__ void k_init_fields(WmGeom g, WmInitArgs a, FView<6, false> uf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nxw * g.nyw) return;
    const int ix = t % g.nxw, iy = t / g.nxw;
    const double xi = (ix + g.nxgs - 2) * a.delx, yj = (iy + g.nygs - 2) * a.delx;
    double f[6] = {0, 0, 0, 0, 0, 0};
    if (a.tag == WM_RNG_HARRIS) {  // proj/reconnection/app.f90:397-410
        const double dx = xi - a.x0, dy = yj - a.y0, w2 = (2 * a.lcs) * (2 * a.lcs);
        const double gg = exp(-(dx * dx + dy * dy) / w2);
        f[0] = +a.e1 * a.b0 * (dy / a.lcs) * gg;
        f[1] = a.b0 * tanh(dx / a.lcs) - a.e1 * a.b0 * (dx / a.lcs) * gg;
    } else if (a.tag == WM_RNG_SHOCK) {  // proj/shock/app.f90:416-426
        const double vp = vprofile(xi, a);
        f[0] = a.bx;
        f[1] = a.by;
        f[2] = a.bz;
        f[4] = +vp * a.bz / a.c;
        f[5] = -vp * a.by / a.c;
    }
    for (int k = 0; k < 6; ++k) uf(k, ix, iy) = f[k];
}

}  // namespace

int wm_launch_init_particles(const WmGeom &g, const WmInitArgs &a, double *stage, cudaStream_t st)
{
    k_init_particles<<<wm_div_up((long long)a.n_row * g.ny, 256), 256, 0, st>>>(g, a, stage);
    return wm_check_launch("k_init_particles");
}

int wm_launch_init_fields(const WmGeom &g, const WmInitArgs &a, FView<6, false> uf, cudaStream_t st)
{
    k_init_fields<<<wm_div_up((long long)g.nxw * g.nyw, 256), 256, 0, st>>>(g, a, uf);
    return wm_check_launch("k_init_fields");
}

// ============================================================ shock injection
// proj/shock/app.f90:695-850 for one rank: nginj = int(pflux) (+1 with probability frac(pflux))
// particles per species enter each step, nginj / ny per row and one more in nginj mod ny rows
// drawn at random; row j's particles sit at x = nxe dx + (k + 1/2)/n_j x0, y = (j + U) dx, then
// move by (v0 + u_x) dt and are boosted by vprofile; ids continue after the species' count.
namespace {

__global__ void k_inject_counts(WmGeom g, WmInjectArgs a, const int *__restrict__ np2, int *__restrict__ inj,
                                long long *__restrict__ ninc, long long *__restrict__ nptot, unsigned *status)
{
    extern __shared__ unsigned keys[];  // [ny]
    __shared__ unsigned long long tot[2];
    __shared__ long long s_nginj;
    const int ny = g.ny;
    if (threadIdx.x < 2) tot[threadIdx.x] = 0;
    __syncthreads();
    unsigned long long t0 = 0, t1 = 0;
    for (int r = threadIdx.x; r < ny; r += blockDim.x) {
        t0 += np2[r];
        t1 += np2[ny + r];
        keys[r] = wm_philox4x32_10((uint32_t)r, (uint32_t)a.it, 1u, WM_RNG_INJECT_COUNT, (uint32_t)a.seed, (uint32_t)(a.seed >> 32)).v[0];
    }
    atomicAdd(&tot[0], t0);
    atomicAdd(&tot[1], t1);
    if (threadIdx.x == 0) {
        double u, unused;
        wm_rng_uniform2(a.seed, (long long)a.it << 32, 0u, WM_RNG_INJECT_COUNT, u, unused);
        long long n = (long long)a.pflux;
        if (u < a.pflux - (double)(long long)a.pflux) ++n;
        s_nginj = n;
    }
    __syncthreads();
    long long nginj = s_nginj;
    if ((long long)(tot[0] + tot[1]) + 2 * (nginj + (long long)a.n_expand * ny) > a.cap) {  // no room: nothing enters, the step reports it
        if (threadIdx.x == 0) atomicOr(status, (unsigned)WMDEV_OVERFLOW);
        nginj = 0;
    }
    const long long base = nginj / ny, nlmod = nginj % ny;
    for (int j = threadIdx.x; j < ny; j += blockDim.x) {
        const unsigned kj = keys[j];
        int rank = 0;
        for (int k = 0; k < ny; ++k) rank += (keys[k] < kj) || (keys[k] == kj && k < j);
        inj[j] = (int)(base + (rank < nlmod ? 1 : 0));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long c = 0;
        for (int j = 0; j < ny; ++j) {
            ninc[j] = c;
            c += inj[j];
        }
        nptot[0] = (long long)tot[0];
        nptot[1] = (long long)tot[1];
    }
}

__global__ void k_inject_reserve(WmGeom g, const int *__restrict__ np2, const int *__restrict__ inj, int extra, int *__restrict__ tmp)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < g.nrows) tmp[r] = np2[r] + inj[r % g.ny] + extra;
}

__device__ __forceinline__ void put_particle(const SoAView &v, long long p, const WmGeom &, int, int, double x, double y, double ux, double uy,
                                             double uz, long long pid)
{
    v.X(p) = x;
    v.Y(p) = y;
    v.UX(p) = ux;
    v.UY(p) = uy;
    v.UZ(p) = uz;
    v.setpid(p, pid);
}

// mixed sets: offsets against the cell the particle is counted in (may reach past 1 for a
// particle beyond nxe, as the FP64 shape offset does in the reference)
__device__ __forceinline__ void put_particle(const MixedView &v, long long p, const WmGeom &g, int cell, int jr, double x, double y,
                                             double ux, double uy, double uz, long long pid)
{
    v.X(p) = (float)(x - (double)(g.nxgs + cell));
    float oy = (float)(y - (double)(g.nys + jr));
    if (oy >= 1.f) oy = 0x1.fffffep-1f;
    v.Y(p) = oy;
    v.UX(p) = (float)ux;
    v.UY(p) = (float)uy;
    v.UZ(p) = (float)uz;
    v.setpid(p, pid);
}

// perm != null (the mixed path's permuted state): the new particle of row slot np2+k goes to the
// fresh slot *phys0 + isp * (this step's count) + (its injection index) of dst's arrays -- past
// the slots the push output and the ids occupy -- and perm / idperm of its cell-sorted slot point there.
template <class PV>
__global__ void k_inject_particles(WmGeom g, WmInjectArgs a, PV dst, const int *__restrict__ np2, const int *__restrict__ inj,
                                   const long long *__restrict__ ninc, const long long *__restrict__ nptot, unsigned *__restrict__ perm,
                                   unsigned *__restrict__ idperm, const long long *__restrict__ phys0)
{
    const int jr = blockIdx.y;
    const int n = inj[jr];
    const long long step_total = ninc[g.ny - 1] + inj[g.ny - 1];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const long long q = ninc[jr] + k;  // this step's injection index
        double uy_draw, unused, n1, n2, n3, n4, n5, n6;
        wm_rng_uniform2(a.seed, q, (uint32_t)(4 * a.it + 0), WM_RNG_INJECT, uy_draw, unused);
        wm_rng_normal2(a.seed, q, (uint32_t)(4 * a.it + 1), WM_RNG_INJECT, n1, n2);
        wm_rng_normal2(a.seed, q, (uint32_t)(4 * a.it + 2), WM_RNG_INJECT, n3, n4);
        wm_rng_normal2(a.seed, q, (uint32_t)(4 * a.it + 3), WM_RNG_INJECT, n5, n6);
        const double delx = a.delx;
        const double xb = a.xe + (k + 0.5) / n * a.x0;
        const double y = (g.nys + jr + uy_draw) * delx;
        const double c2 = a.c * a.c;
        for (int isp = 0; isp < 2; ++isp) {
            const double sd = isp == 0 ? a.vth_i : a.vth_e;
            const double ux = sd * (isp == 0 ? n1 : n4), uy = sd * (isp == 0 ? n2 : n5), uz = sd * (isp == 0 ? n3 : n6);
            const double x = xb + (a.v0 + ux) * a.delt;
            const double v1 = vprofile(x, a.v0, a.l_damp_ini, a.nxgs_delx);
            const double gam1 = 1 / sqrt(1 - (v1 / a.c) * (v1 / a.c));
            const double gamp = sqrt(1 + (ux * ux + uy * uy + uz * uz) / c2);
            const int row = isp * g.ny + jr;
            long long p = dst.idx(row, np2[row] + k);
            if (perm) {
                const long long ph = *phys0 + isp * step_total + q;
                perm[p] = (unsigned)ph;
                idperm[p] = (unsigned)ph;
                p = ph;
            }
            put_particle(dst, p, g, a.cell, jr, x, y, gam1 * (ux + v1 * gamp), uy, uz, -(k + 1 + ninc[jr] + nptot[isp]));
        }
    }
}

__global__ void k_inject_finish(WmGeom g, WmInjectArgs a, int *__restrict__ np2, int *__restrict__ cumcnt, const int *__restrict__ inj)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.nrows) return;
    const int n = inj[r % g.ny];
    np2[r] += n;
    int *cc = cumcnt + (long long)r * (g.nx + 1);
    cc[a.cell + 1] += n;  // cumcnt(nxe): the new particles count in cell nxe-1 (app.f90:837)
    for (int ci = a.cell + 2; ci <= g.nx; ++ci) cc[ci] += n;  // and the row total with it
}

// proj/shock/app.f90:613-690 (relocate), the box growing by one cell (nxe -> nxe + 1), for one
// rank: n0 = a.n_expand particles per row and species in the cell nxe (interior cell a.cell + 1),
// x = nxe dx + (k + 1/2)/n0 dx, y = (j + U) dx shared by the species, a Maxwellian in the fluid
// rest frame boosted by vprofile(x); they go behind the row's sorted and injected particles
// (np2 already counts the injected ones) and are counted in that cell; the ids continue after the
// species' count including this step's injection.  The draws are Philox with counter
// (row * n0 + k, step) under their own tag.  perm != null: as k_inject_particles, past the
// injected particles' fresh slots.
template <class PV>
__global__ void k_expand_particles(WmGeom g, WmInjectArgs a, PV dst, const int *__restrict__ np2, const int *__restrict__ inj,
                                   const long long *__restrict__ ninc, const long long *__restrict__ nptot, unsigned *__restrict__ perm,
                                   unsigned *__restrict__ idperm, const long long *__restrict__ phys0)
{
    const int jr = blockIdx.y;
    const int n0 = a.n_expand;
    const long long step_inj = ninc[g.ny - 1] + inj[g.ny - 1];  // this step's injected particles per species
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n0; k += gridDim.x * blockDim.x) {
        const long long q = (long long)jr * n0 + k;
        double uy_draw, unused, n1, n2, n3, n4, n5, n6;
        wm_rng_uniform2(a.seed, q, (uint32_t)(4 * a.it + 0), WM_RNG_EXPAND, uy_draw, unused);
        wm_rng_normal2(a.seed, q, (uint32_t)(4 * a.it + 1), WM_RNG_EXPAND, n1, n2);
        wm_rng_normal2(a.seed, q, (uint32_t)(4 * a.it + 2), WM_RNG_EXPAND, n3, n4);
        wm_rng_normal2(a.seed, q, (uint32_t)(4 * a.it + 3), WM_RNG_EXPAND, n5, n6);
        const double delx = a.delx;
        const double x = a.xe + (k + 0.5) / n0 * delx;
        const double y = (g.nys + jr + uy_draw) * delx;
        const double c2 = a.c * a.c;
        const double v1 = vprofile(x, a.v0, a.l_damp_ini, a.nxgs_delx);
        const double gam1 = 1 / sqrt(1 - (v1 / a.c) * (v1 / a.c));
        for (int isp = 0; isp < 2; ++isp) {
            const double sd = isp == 0 ? a.vth_i : a.vth_e;
            const double ux = sd * (isp == 0 ? n1 : n4), uy = sd * (isp == 0 ? n2 : n5), uz = sd * (isp == 0 ? n3 : n6);
            const double gamp = sqrt(1 + (ux * ux + uy * uy + uz * uz) / c2);
            const int row = isp * g.ny + jr;
            long long p = dst.idx(row, np2[row] + k);
            if (perm) {
                const long long ph = *phys0 + 2 * step_inj + isp * (long long)g.ny * n0 + q;
                perm[p] = (unsigned)ph;
                idperm[p] = (unsigned)ph;
                p = ph;
            }
            put_particle(dst, p, g, a.cell + 1, jr, x, y, gam1 * (ux + v1 * gamp), uy, uz, -(k + 1 + (long long)jr * n0 + nptot[isp] + step_inj));
        }
    }
}

// np2 += n0; cumcnt(nxe + 1) = cumcnt(nxe) + n0 (app.f90:674) and the row total with it
__global__ void k_expand_finish(WmGeom g, WmInjectArgs a, int *__restrict__ np2, int *__restrict__ cumcnt)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.nrows) return;
    const int n = a.n_expand;
    np2[r] += n;
    int *cc = cumcnt + (long long)r * (g.nx + 1);
    for (int ci = a.cell + 2; ci <= g.nx; ++ci) cc[ci] += n;
}

__global__ void k_inject_fields(WmGeom g, WmInjectArgs a, FView<6, false> uf)
{
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    if (iy >= g.nyw) return;
    const int i1 = a.cell + 2, i2 = a.cell + 3;  // ghosted columns of nxe-1 and nxe
    uf(1, i1, iy) = a.by0;
    uf(2, i1, iy) = a.bz0;
    uf(4, i1, iy) = +a.v0 * a.bz0 / a.c;
    uf(5, i1, iy) = -a.v0 * a.by0 / a.c;
    uf(1, i2, iy) = a.by0;
    uf(2, i2, iy) = a.bz0;
}

}  // namespace

int wm_launch_inject_counts(const WmGeom &g, const WmInjectArgs &a, const int *np2, int *inj, long long *ninc, long long *nptot,
                            unsigned *status, cudaStream_t st)
{
    if (g.ny > WM_INJECT_MAX_ROWS) return WM_ERR_UNSUPPORTED;
    k_inject_counts<<<1, 1024, sizeof(unsigned) * g.ny, st>>>(g, a, np2, inj, ninc, nptot, status);
    return wm_check_launch("k_inject_counts");
}

int wm_launch_inject_reserve(const WmGeom &g, const WmInjectArgs &a, const int *np2, const int *inj, int *tmp, cudaStream_t st)
{
    k_inject_reserve<<<wm_div_up(g.nrows, 256), 256, 0, st>>>(g, np2, inj, a.n_expand, tmp);
    return wm_check_launch("k_inject_reserve");
}

template <class PV>
int wm_launch_inject_particles(const WmGeom &g, const WmInjectArgs &a, PV dst, int *np2, int *cumcnt, const int *inj,
                               const long long *ninc, const long long *nptot, cudaStream_t st, unsigned *perm, unsigned *idperm,
                               const long long *phys0)
{
    k_inject_particles<PV><<<dim3(1, g.ny), 128, 0, st>>>(g, a, dst, np2, inj, ninc, nptot, perm, idperm, phys0);
    WM_TRY(wm_check_launch("k_inject_particles"));
    k_inject_finish<<<wm_div_up(g.nrows, 256), 256, 0, st>>>(g, a, np2, cumcnt, inj);
    return wm_check_launch("k_inject_finish");
}
template int wm_launch_inject_particles<SoAView>(const WmGeom &, const WmInjectArgs &, SoAView, int *, int *, const int *,
                                                 const long long *, const long long *, cudaStream_t, unsigned *, unsigned *,
                                                 const long long *);
template int wm_launch_inject_particles<MixedView>(const WmGeom &, const WmInjectArgs &, MixedView, int *, int *, const int *,
                                                   const long long *, const long long *, cudaStream_t, unsigned *, unsigned *,
                                                   const long long *);

template <class PV>
int wm_launch_expand_particles(const WmGeom &g, const WmInjectArgs &a, PV dst, int *np2, int *cumcnt, const int *inj, const long long *ninc,
                               const long long *nptot, cudaStream_t st, unsigned *perm, unsigned *idperm, const long long *phys0)
{
    if (a.n_expand < 1 || a.cell + 2 > g.nx) return WM_ERR_BAD_ARG;
    k_expand_particles<PV><<<dim3(1, g.ny), 128, 0, st>>>(g, a, dst, np2, inj, ninc, nptot, perm, idperm, phys0);
    WM_TRY(wm_check_launch("k_expand_particles"));
    k_expand_finish<<<wm_div_up(g.nrows, 256), 256, 0, st>>>(g, a, np2, cumcnt);
    return wm_check_launch("k_expand_finish");
}
template int wm_launch_expand_particles<SoAView>(const WmGeom &, const WmInjectArgs &, SoAView, int *, int *, const int *, const long long *,
                                                 const long long *, cudaStream_t, unsigned *, unsigned *, const long long *);
template int wm_launch_expand_particles<MixedView>(const WmGeom &, const WmInjectArgs &, MixedView, int *, int *, const int *, const long long *,
                                                   const long long *, cudaStream_t, unsigned *, unsigned *, const long long *);

int wm_launch_inject_fields(const WmGeom &g, const WmInjectArgs &a, FView<6, false> uf, cudaStream_t st)
{
    k_inject_fields<<<wm_div_up(g.nyw, 128), 128, 0, st>>>(g, a, uf);
    return wm_check_launch("k_inject_fields");
}
