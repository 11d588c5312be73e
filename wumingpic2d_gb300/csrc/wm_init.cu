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

__device__ __forceinline__ double vprofile(double x, const WmInitArgs &a)
{
    // proj/shock/app.f90:881-891
    const double x0 = a.l_damp_ini + a.nxgs_delx;
    const double xs = a.l_damp_ini * 0.1;
    return 0.5 * a.v0 * (1 + tanh((x - x0) / xs));
}

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
        const int nxs = g.nxgs, nxe = g.nxge;
        const double x = (nxs + (nxe - nxs) * (i + 0.5) / a.n_row) * delx;
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
