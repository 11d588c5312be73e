// wm_field.cu -- implicit field update of common/field.f90:66-186 on sm_103a, FP64.
//
// The three delta-B components are solved together: every CG kernel walks the grid once and
// handles each component that is still iterating, so one launch serves three solves.  Each
// component follows the reference's sequence exactly (field.f90:347-459): lagged stop test on
// the residual norm before the update, first test against ||b||^2, ite_max limit.  The global
// sums are deterministic: each CTA reduces its cells in a fixed order, writes one partial, and
// the last CTA to finish (an atomic ticket, no spin-wait) adds the partials in index order and
// updates the per-component scalars (alpha, beta, counters) in device memory, so no host round
// trip is needed between kernels.  Periodic halos of the CG vectors are index wraps
// (boundary_periodic__phi, :511-568); the field ghost layers are filled by the same copy
// pattern as boundary_periodic__dfield (:251-354) and __curre (:357-508).
#include <algorithm>

#include "wm_launch.cuh"

struct CgScal {
    double sum_g, eps, sumr, sum2, sum1, av, bv, pad;
    int ite, active, status, pad2;
};

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int CG_THREADS = 256;
constexpr int CG_BLOCKS = 152 * 4;  // one wave: 4 CTAs of 256 threads on each of the 152 SMs
// k_cg_phase: 5 CTAs per SM (measured at 2048^2 x 64 ppc: CG iterations 3.09 ms per step with 4, 2.86
// with 5, 3.19 with 3); the set-up kernels keep 4 (0.67 ms against 0.73 with 5)
constexpr int CG_PHASE_BLOCKS = 152 * 5;

// ------------------------------------------------------------ ghost patterns
template <class FV>
__global__ void k_curre_bc_y(WmGeom g, FV uj)
{
    const int nxr = g.nxa + 4;  // columns nxs-2 .. nxe+2
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nxr * 3) return;
    const int ix = t % nxr, k = t / nxr;
    // rows relative to nys-2: nys-2 -> 0, nys-1 -> 1, nys -> 2, nys+1 -> 3, nye-1 -> ny, nye -> ny+1, nye+1 -> ny+2, nye+2 -> ny+3
    const int rs2 = 0, rs1 = 1, rs = 2, rs_1 = 3, re1m = g.ny, re = g.ny + 1, re1 = g.ny + 2, re2 = g.ny + 3;
    const double a = uj(k, ix, rs2), b = uj(k, ix, rs1);
    uj(k, ix, re1m) = uj(k, ix, re1m) + a;
    uj(k, ix, re) = uj(k, ix, re) + b;
    const double c = uj(k, ix, re1), d = uj(k, ix, re2);
    uj(k, ix, rs) = uj(k, ix, rs) + c;
    uj(k, ix, rs_1) = uj(k, ix, rs_1) + d;
    uj(k, ix, re1) = uj(k, ix, rs);
    uj(k, ix, re2) = uj(k, ix, rs_1);
    uj(k, ix, rs2) = uj(k, ix, re1m);
    uj(k, ix, rs1) = uj(k, ix, re);
}

template <class FV>
__global__ void k_curre_bc_x(WmGeom g, FV uj)
{
    const int nyr = g.ny + 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nyr * 3) return;
    const int iy = t % nyr, k = t / nyr;
    const int cs2 = 0, cs1 = 1, cs = 2, cs_1 = 3, ce1m = g.nx, ce = g.nx + 1, ce1 = g.nx + 2, ce2 = g.nx + 3;
    uj(k, ce1m, iy) = uj(k, ce1m, iy) + uj(k, cs2, iy);
    uj(k, ce, iy) = uj(k, ce, iy) + uj(k, cs1, iy);
    uj(k, cs, iy) = uj(k, cs, iy) + uj(k, ce1, iy);
    uj(k, cs_1, iy) = uj(k, cs_1, iy) + uj(k, ce2, iy);
    uj(k, cs2, iy) = uj(k, ce1m, iy);
    uj(k, cs1, iy) = uj(k, ce, iy);
    uj(k, ce1, iy) = uj(k, cs, iy);
    uj(k, ce2, iy) = uj(k, cs_1, iy);
}

template <class FV>
__global__ void k_dfield_bc_y(WmGeom g, FV df)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nxa * 6) return;
    const int ix = 2 + t % g.nxa, k = t / g.nxa;  // interior columns nxs..nxe only (:263-345)
    df(k, ix, g.ny + 2) = df(k, ix, 2);
    df(k, ix, g.ny + 3) = df(k, ix, 3);
    df(k, ix, 0) = df(k, ix, g.ny);
    df(k, ix, 1) = df(k, ix, g.ny + 1);
}

template <class FV>
__global__ void k_dfield_bc_x(WmGeom g, FV df)
{
    const int nyr = g.ny + 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nyr * 6) return;
    const int iy = t % nyr, k = t / nyr;
    if (g.bc == WM_BC_PERIODIC) {
        df(k, 0, iy) = df(k, g.nx, iy);
        df(k, 1, iy) = df(k, g.nx + 1, iy);
        df(k, g.nx + 2, iy) = df(k, 2, iy);
        df(k, g.nx + 3, iy) = df(k, 3, iy);
        return;
    }
    // conducting wall at nxs (boundary_reconnection.f90:351-360, boundary_shock.f90:397-406):
    // column nxs-1 (ghosted 1) from nxs (2) or nxs+1 (3)
    if (k == 0 || k >= 4) df(k, 1, iy) = -df(k, 2, iy);
    else df(k, 1, iy) = df(k, 3, iy);
    if (g.bc == WM_BC_RECONNECTION) {  // conducting wall at nxe (ghosted nx+1), mirror of the left
        if (k == 0 || k >= 4) df(k, g.nx + 1, iy) = -df(k, g.nx, iy);
        else df(k, g.nx + 2, iy) = df(k, g.nx, iy);
    } else {  // shock: zero beyond the injection boundary, column nxe+1
        df(k, g.nxa + 2, iy) = 0.0;
    }
}

// phi(nxs-1:nxe+1, nys-1:nye+1), x fastest
__global__ void k_phi_bc_y(int nx, int ny, double *phi)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nx) return;
    const int pw = nx + 2, ix = 1 + t;
    phi[ix + (long long)pw * (ny + 1)] = phi[ix + (long long)pw * 1];
    phi[ix + 0] = phi[ix + (long long)pw * ny];
}
__global__ void k_phi_bc_x(int nx, int ny, double *phi, int bc, int l)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ny + 2) return;
    const int pw = nx + 2;
    if (bc == WM_BC_PERIODIC) {
        phi[0 + (long long)pw * t] = phi[nx + (long long)pw * t];
        phi[nx + 1 + (long long)pw * t] = phi[1 + (long long)pw * t];
    } else {  // walls (boundary_reconnection.f90:557-577): Bx odd about nxs-1/2, By, Bz even about nxs; zero at nxe+1
        phi[0 + (long long)pw * t] = (l == 1) ? -phi[1 + (long long)pw * t] : phi[2 + (long long)pw * t];
        phi[nx + 1 + (long long)pw * t] = 0.0;
    }
}

// mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp), reference layout
__global__ void k_mom_bc_x(WmGeom g, double *mom)
{
    const int mx = g.nx + 2, my = g.ny + 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= my * g.nsp * 7) return;
    const int k = t % 7, jy = (t / 7) % my, isp = t / (7 * my);
    double *rowp = mom + 7 * (long long)mx * (jy + (long long)my * isp);
    const bool walls = g.bc != WM_BC_PERIODIC;  // boundary_reconnection.f90:590-593: onto the own edge
    rowp[k + 7 * 1] = rowp[k + 7 * 1] + rowp[k + 7 * (walls ? 0 : mx - 1)];
    rowp[k + 7 * (mx - 2)] = rowp[k + 7 * (mx - 2)] + rowp[k + 7 * (walls ? mx - 1 : 0)];
}
__global__ void k_mom_bc_y(WmGeom g, double *mom)
{
    const int mx = g.nx + 2, my = g.ny + 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= mx * g.nsp * 7) return;
    const int k = t % 7, ix = (t / 7) % mx, isp = t / (7 * mx);
    double *col = mom + k + 7 * (ix + (long long)mx * (long long)my * isp);
    const long long rs = (long long)7 * mx;
    col[rs * (my - 2)] = col[rs * (my - 2)] + col[rs * 0];
    col[rs * 1] = col[rs * 1] + col[rs * (my - 1)];
}

// ------------------------------------------------------------ transposes
// ref (AoS, component fastest) <-> planes (SoA)
template <int NC>
__global__ void k_aos_to_soa(long long npts, const double *__restrict__ a, double *__restrict__ s)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < npts * NC; e += (long long)gridDim.x * blockDim.x) {
        const long long pt = e / NC;
        const int k = (int)(e - pt * NC);
        s[(long long)k * npts + pt] = a[e];
    }
}
template <int NC>
__global__ void k_soa_to_aos(long long npts, const double *__restrict__ s, double *__restrict__ a)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < npts * NC; e += (long long)gridDim.x * blockDim.x) {
        const long long pt = e / NC;
        const int k = (int)(e - pt * NC);
        a[e] = s[(long long)k * npts + pt];
    }
}

// Grid-stride walk over the elements e = r * n + c of an (rows x n) grid: the column and row
// advance by the stride's quotient and remainder, so the loop divides only once per thread.
struct GridCell {
    long long e, stride;
    int c, r, dc, dr, n;
    __device__ explicit GridCell(int n_) : n(n_)
    {
        e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        stride = (long long)gridDim.x * blockDim.x;
        c = (int)(e % n);
        r = (int)(e / n);
        dc = (int)(stride % n);
        dr = (int)(stride / n);
    }
    __device__ __forceinline__ void next()
    {
        e += stride;
        c += dc;
        r += dr;
        if (c >= n) {
            c -= n;
            ++r;
        }
    }
};

// ------------------------------------------------------------- reductions
__device__ __forceinline__ void block_sum3(double &a, double &b, double &c)
{
    __shared__ double sh[3][CG_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(FULL, a, o);
        b += __shfl_down_sync(FULL, b, o);
        c += __shfl_down_sync(FULL, c, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) {
        sh[0][w] = a;
        sh[1][w] = b;
        sh[2][w] = c;
    }
    __syncthreads();
    if (w == 0) {
        a = (l < CG_THREADS / 32) ? sh[0][l] : 0.0;
        b = (l < CG_THREADS / 32) ? sh[1][l] : 0.0;
        c = (l < CG_THREADS / 32) ? sh[2][l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(FULL, a, o);
            b += __shfl_down_sync(FULL, b, o);
            c += __shfl_down_sync(FULL, c, o);
        }
    }
}

// Writes this CTA's three partials; returns true in thread 0 of the last CTA to finish, with
// tot[] = the partials summed in index order.
__device__ bool last_block_reduce3(double a, double b, double c, double *partial, unsigned *ticket, double tot[3])
{
    __shared__ bool is_last;
    block_sum3(a, b, c);
    if (threadIdx.x == 0) {
        partial[0 * gridDim.x + blockIdx.x] = a;
        partial[1 * gridDim.x + blockIdx.x] = b;
        partial[2 * gridDim.x + blockIdx.x] = c;
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
        s0 += __ldcg(&partial[0 * gridDim.x + i]);
        s1 += __ldcg(&partial[1 * gridDim.x + i]);
        s2 += __ldcg(&partial[2 * gridDim.x + i]);
    }
    block_sum3(s0, s1, s2);
    if (threadIdx.x == 0) {
        tot[0] = s0;
        tot[1] = s1;
        tot[2] = s2;
        *ticket = 0u;
    }
    return threadIdx.x == 0;
}

struct FieldK {
    double f1, f2, f3, f4, f5, gfac, pi4dt, err;
    int itemax;
};

__device__ __forceinline__ int wrapm(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// The x neighbours of interior cell ci (0-based) of component l (0 = Bx) of a CG vector, read
// through at(c) = value at interior column c of the same row: periodic wrap, or the walls' halo
// (boundary_reconnection__phi / boundary_shock__phi): Bx odd about nxs - 1/2, By and Bz even
// about nxs, zero beyond nxe (the last active cell, nxa - 1).
//
// Cells past nxe (ci >= nxa: the shock's expanding box) are outside the solve of field.f90:319-461,
// which runs over nxs..nxe: the kernels below give them b = r = ap = delta-E = 0, so every CG vector
// and dfield stays zero there and the fields past nxe + 1 keep their values, as in the reference.
template <class F>
__device__ __forceinline__ void x_neighbours(const WmGeom &g, int l, int ci, const F &at, double &left, double &right)
{
    if (g.bc == WM_BC_PERIODIC) {
        left = at(wrapm(ci - 1, g.nx));
        right = at(wrapm(ci + 1, g.nx));
        return;
    }
    left = ci > 0 ? at(ci - 1) : (l == 0 ? -at(0) : at(1));
    right = ci < g.nxa - 1 ? at(ci + 1) : 0.0;
}

// gkl (field.f90:125-146), b = f5*gkl and ||b||^2 (:351-364).
template <class FV6, class FV3>
__global__ void __launch_bounds__(CG_THREADS) k_cg_rhs(WmGeom g, FieldK fk, FV6 uf, FV3 uj, double *__restrict__ b,
                                                       double *partial, unsigned *ticket, CgScal *scal)
{
    const long long ncell = (long long)g.nx * g.ny;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const long long e = q.e;
        const int ci = q.c, cj = q.r;
        const int x = ci + 2, y = cj + 2;
        const double g1 = +fk.f2 * (+uf(0, x, y - 1) + uf(0, x - 1, y) - 4. * uf(0, x, y) + uf(0, x + 1, y) + uf(0, x, y + 1)
                                    + fk.f3 * (-uj(2, x, y - 1) + uj(2, x, y)))
                          - fk.f1 * (-uf(5, x, y - 1) + uf(5, x, y));
        const double g2 = +fk.f2 * (+uf(1, x, y - 1) + uf(1, x - 1, y) - 4. * uf(1, x, y) + uf(1, x + 1, y) + uf(1, x, y + 1)
                                    - fk.f3 * (-uj(2, x - 1, y) + uj(2, x, y)))
                          + fk.f1 * (-uf(5, x - 1, y) + uf(5, x, y));
        const double g3 = +fk.f2 * (+uf(2, x, y - 1) + uf(2, x - 1, y) - 4. * uf(2, x, y) + uf(2, x + 1, y) + uf(2, x, y + 1)
                                    + fk.f3 * (-uj(1, x - 1, y) + uj(1, x, y) + uj(0, x, y - 1) - uj(0, x, y)))
                          - fk.f1 * (-uf(4, x - 1, y) + uf(4, x, y) + uf(3, x, y - 1) - uf(3, x, y));
        const bool on = ci < g.nxa;
        const double b1 = on ? fk.f5 * g1 : 0.0, b2 = on ? fk.f5 * g2 : 0.0, b3 = on ? fk.f5 * g3 : 0.0;
        b[0 * ncell + e] = b1;
        b[1 * ncell + e] = b2;
        b[2 * ncell + e] = b3;
        a0 += b1 * b1;
        a1 += b2 * b2;
        a2 += b3 * b3;
    }
    double tot[3];
    if (last_block_reduce3(a0, a1, a2, partial, ticket, tot)) {
        for (int l = 0; l < 3; ++l) {
            scal[l].sum_g = tot[l];
            scal[l].eps = sqrt(tot[l]) * fk.err;
        }
    }
}

// r = b + (phi neighbours) - f4 phi, p = r, ||r||^2 (:366-385); phi = df(l) interior.
template <class FV6>
__global__ void __launch_bounds__(CG_THREADS) k_cg_resid(WmGeom g, FieldK fk, FV6 df, const double *__restrict__ b,
                                                         double *__restrict__ r, double *__restrict__ p, double *partial,
                                                         unsigned *ticket, CgScal *scal)
{
    const long long ncell = (long long)g.nx * g.ny;
    double acc[3] = {0.0, 0.0, 0.0};
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const long long e = q.e;
        const int ci = q.c, cj = q.r;
        const int ym = wrapm(cj - 1, g.ny) + 2, yp = wrapm(cj + 1, g.ny) + 2, x = ci + 2, y = cj + 2;
#pragma unroll
        for (int l = 0; l < 3; ++l) {
            double xl, xr;
            x_neighbours(g, l, ci, [&](int c) { return df(l, c + 2, y); }, xl, xr);
            const double rv = ci < g.nxa ? b[l * ncell + e] + df(l, x, ym) + xl - fk.f4 * df(l, x, y) + xr + df(l, x, yp) : 0.0;
            r[l * ncell + e] = rv;
            p[l * ncell + e] = rv;
            acc[l] += rv * rv;
        }
    }
    double tot[3];
    if (last_block_reduce3(acc[0], acc[1], acc[2], partial, ticket, tot)) {
        for (int l = 0; l < 3; ++l) {
            scal[l].sumr = tot[l];
            scal[l].ite = 0;
            scal[l].status = 0;
            scal[l].active = (sqrt(tot[l]) > scal[l].eps) && (scal[l].sum_g > scal[l].eps);
        }
    }
}

// Candidate guess stored as [3][nx*ny] (x fastest), read through ghosted indices like df.
struct PlaneView {
    const double *p;
    int nx, ny;
    __device__ __forceinline__ double operator()(int l, int ix, int iy) const
    {
        return p[((long long)l * ny + (iy - 2)) * nx + (ix - 2)];
    }
};

// |b - A x|^2 per component for both initial guesses in one pass over b: the network's candidate
// (cand, [3][nx*ny]) into out6[0..2] and the previous step's dB (df) into out6[3..5] (the residual
// of k_cg_resid).  Six partials per CTA, summed in CTA order by the last CTA.
template <class FV6>
__global__ void __launch_bounds__(CG_THREADS) k_guess_resid2(WmGeom g, FieldK fk, PlaneView cand, FV6 df, const double *__restrict__ b,
                                                             double *partial, unsigned *ticket, double *out6)
{
    __shared__ bool is_last;
    const long long ncell = (long long)g.nx * g.ny;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const long long e = q.e;
        const int ci = q.c, cj = q.r;
        const int ym = wrapm(cj - 1, g.ny) + 2, yp = wrapm(cj + 1, g.ny) + 2, xx = ci + 2, yy = cj + 2;
#pragma unroll
        for (int l = 0; l < 3; ++l) {
            const double bl = b[l * ncell + e];
            double xl, xr;
            x_neighbours(g, l, ci, [&](int c) { return cand(l, c + 2, yy); }, xl, xr);
            const double rc = bl + cand(l, xx, ym) + xl - fk.f4 * cand(l, xx, yy) + xr + cand(l, xx, yp);
            x_neighbours(g, l, ci, [&](int c) { return df(l, c + 2, yy); }, xl, xr);
            const double rp = bl + df(l, xx, ym) + xl - fk.f4 * df(l, xx, yy) + xr + df(l, xx, yp);
            const bool on = ci < g.nxa;
            acc[l] += on ? rc * rc : 0.0;
            acc[3 + l] += on ? rp * rp : 0.0;
        }
    }
    block_sum3(acc[0], acc[1], acc[2]);
    block_sum3(acc[3], acc[4], acc[5]);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k) partial[k * gridDim.x + blockIdx.x] = acc[k];
        __threadfence();
        is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < 6; ++k) t[k] += __ldcg(&partial[k * gridDim.x + i]);
    block_sum3(t[0], t[1], t[2]);
    block_sum3(t[3], t[4], t[5]);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k) out6[k] = t[k];
        *ticket = 0u;
    }
}

// k_cg_resid for a solve that starts from the better of two guesses: component l starts from the
// network's candidate where its residual (stats[l]) is below the previous step's (stats[3 + l]),
// which is then copied into df(l); the residual, p and ||r||^2 are those of k_cg_resid on the
// chosen start.  A component reads only cand or only df, so the copy races with no read.
// stats[6 + l] = 1 where the candidate was taken, stats[9 + l] = ||b_l||^2.
template <class FV6>
__global__ void __launch_bounds__(CG_THREADS) k_cg_resid_pick(WmGeom g, FieldK fk, FV6 df, PlaneView cand, const double *__restrict__ b,
                                                              double *__restrict__ r, double *__restrict__ p, double *partial,
                                                              unsigned *ticket, CgScal *scal, double *stats)
{
    const long long ncell = (long long)g.nx * g.ny;
    bool take[3];
#pragma unroll
    for (int l = 0; l < 3; ++l) take[l] = stats[l] < stats[3 + l];
    double acc[3] = {0.0, 0.0, 0.0};
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const long long e = q.e;
        const int ci = q.c, cj = q.r;
        const int ym = wrapm(cj - 1, g.ny) + 2, yp = wrapm(cj + 1, g.ny) + 2, x = ci + 2, y = cj + 2;
#pragma unroll
        for (int l = 0; l < 3; ++l) {
            const bool tk = take[l];
            auto at = [&](int ix, int iy) { return tk ? cand(l, ix, iy) : df(l, ix, iy); };
            double xl, xr;
            x_neighbours(g, l, ci, [&](int c) { return at(c + 2, y); }, xl, xr);
            const double centre = at(x, y);
            const double rv = ci < g.nxa ? b[l * ncell + e] + at(x, ym) + xl - fk.f4 * centre + xr + at(x, yp) : 0.0;
            if (tk) df(l, x, y) = centre;
            r[l * ncell + e] = rv;
            p[l * ncell + e] = rv;
            acc[l] += rv * rv;
        }
    }
    double tot[3];
    if (last_block_reduce3(acc[0], acc[1], acc[2], partial, ticket, tot)) {
        for (int l = 0; l < 3; ++l) {
            scal[l].sumr = tot[l];
            scal[l].ite = 0;
            scal[l].status = 0;
            scal[l].active = (sqrt(tot[l]) > scal[l].eps) && (scal[l].sum_g > scal[l].eps);
            stats[6 + l] = take[l] ? 1.0 : 0.0;
            stats[9 + l] = scal[l].sum_g;
        }
    }
}

// One launch of the CG iterations (field.f90:395-450), the three components staggered: component
// l runs phase (t - l) mod 3 of its iteration at launch t (it starts at launch l), so that each
// launch mixes one component's FP64-bound stencil with the other two's HBM-bound updates.
//   phase 0 (:395-415): ap = A p and p.ap, then av = sumr / p.ap;
//   phase 1 (:417-443): phi += av p, r -= av ap, ||r||^2, the lagged stop test and bv;
//   phase 2 (:444-450): p = r + bv p.
// A component that stopped in phase 1 skips the rest.  Per component the arithmetic, its order
// and the reduction tree (fixed grid, fixed per-thread cells) do not depend on the staggering.
// Registers are bounded for one CTA per SM more than the grid places, so that the mixed step's
// rebin kernels, which run on a second stream beside the field solve, find room on every SM.
template <class FV6>
__global__ void __launch_bounds__(CG_THREADS, CG_PHASE_BLOCKS / 152 + 1) k_cg_phase(WmGeom g, FieldK fk, FV6 df, double *__restrict__ p, double *__restrict__ r,
                                                         double *__restrict__ ap, double *partial, unsigned *ticket, CgScal *scal, int t)
{
    const long long ncell = (long long)g.nx * g.ny;
    int ph[3];
    bool act[3];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
        ph[l] = t >= l ? (t - l) % 3 : -1;
        act[l] = ph[l] >= 0 && scal[l].active != 0;
    }
    if (!act[0] && !act[1] && !act[2]) return;  // uniform across the grid: no CTA takes a ticket
    const double av[3] = {scal[0].av, scal[1].av, scal[2].av}, bv[3] = {scal[0].bv, scal[1].bv, scal[2].bv};
    double acc[3] = {0.0, 0.0, 0.0};
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const long long e = q.e;
        const int ci = q.c, cj = q.r;
#pragma unroll
        for (int l = 0; l < 3; ++l) {
            if (!act[l]) continue;
            const long long o = l * ncell + e;
            if (ph[l] == 0) {
                const double *pl = p + l * ncell;
                const long long row = (long long)cj * g.nx;
                const long long es = (long long)wrapm(cj - 1, g.ny) * g.nx + ci, en = (long long)wrapm(cj + 1, g.ny) * g.nx + ci;
                const double pc = pl[e];
                double xl, xr;
                x_neighbours(g, l, ci, [&](int c) { return pl[row + c]; }, xl, xr);
                const double a = ci < g.nxa ? -pl[es] - xl + fk.f4 * pc - xr - pl[en] : 0.0;
                ap[o] = a;
                acc[l] += pc * a;
            } else if (ph[l] == 1) {
                df(l, ci + 2, cj + 2) = df(l, ci + 2, cj + 2) + av[l] * p[o];
                const double rv = r[o] - av[l] * ap[o];
                r[o] = rv;
                acc[l] += rv * rv;
            } else {
                p[o] = r[o] + bv[l] * p[o];
            }
        }
    }
    if ((act[0] && ph[0] < 2) || (act[1] && ph[1] < 2) || (act[2] && ph[2] < 2)) {
        double tot[3];
        if (last_block_reduce3(acc[0], acc[1], acc[2], partial, ticket, tot)) {
            for (int l = 0; l < 3; ++l) {
                if (!act[l]) continue;
                CgScal &s = scal[l];
                if (ph[l] == 0) {
                    s.sum2 = tot[l];
                    s.av = s.sumr / tot[l];
                    s.ite += 1;
                } else if (ph[l] == 1) {
                    s.sum1 = tot[l];
                    s.sum_g = sqrt(s.sumr);
                    if (s.ite >= fk.itemax) {
                        s.status = WM_ERR_CG_MAXITER;
                        s.active = 0;
                    } else {
                        s.bv = tot[l] / s.sumr;
                        s.sumr = tot[l];
                        s.active = (s.sum_g > s.eps);
                    }
                }
            }
        }
    }
}

// delta-E (field.f90:154-171)
template <class FV6, class FV3>
__global__ void k_efield(WmGeom g, FieldK fk, FV6 df, FV6 uf, FV3 uj)
{
    const long long ncell = (long long)g.nx * g.ny;
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const int x = q.c + 2, y = q.r + 2;
        if (q.c >= g.nxa) {  // past nxe: no field update (:156)
            df(3, x, y) = 0.0;
            df(4, x, y) = 0.0;
            df(5, x, y) = 0.0;
            continue;
        }
        df(3, x, y) = +fk.f1 * (+fk.gfac * (-df(2, x, y) + df(2, x, y + 1)) + (-uf(2, x, y) + uf(2, x, y + 1))) - fk.pi4dt * uj(0, x, y);
        df(4, x, y) = -fk.f1 * (+fk.gfac * (-df(2, x, y) + df(2, x + 1, y)) + (-uf(2, x, y) + uf(2, x + 1, y))) - fk.pi4dt * uj(1, x, y);
        df(5, x, y) = +fk.f1 * (+fk.gfac * (-df(1, x, y) + df(1, x + 1, y) + df(0, x, y) - df(0, x, y + 1))
                                + (-uf(1, x, y) + uf(1, x + 1, y) + uf(0, x, y) - uf(0, x, y + 1)))
                      - fk.pi4dt * uj(2, x, y);
    }
}

// uf += df over the ghosted grid (:176-184)
template <class FV6>
__global__ void k_field_add(WmGeom g, FV6 uf, FV6 df)
{
    const long long n = (long long)g.nxw * g.nyw;
    for (GridCell q(g.nxw); q.e < n; q.next()) {
        const int ix = q.c, iy = q.r;
#pragma unroll
        for (int k = 0; k < 6; ++k) uf(k, ix, iy) = uf(k, ix, iy) + df(k, ix, iy);
    }
}

// E^2, B^2 over the interior (proj/weibel/app.f90:521-528): partial[2][blocks]
template <class FV6>
__global__ void __launch_bounds__(CG_THREADS) k_energy_fields(WmGeom g, FV6 uf, double *partial)
{
    const long long ncell = (long long)g.nx * g.ny;
    double be = 0.0, ee = 0.0, z = 0.0;
    for (GridCell q(g.nx); q.e < ncell; q.next()) {
        const int x = q.c + 2, y = q.r + 2;
        be += uf(0, x, y) * uf(0, x, y) + uf(1, x, y) * uf(1, x, y) + uf(2, x, y) * uf(2, x, y);
        ee += uf(3, x, y) * uf(3, x, y) + uf(4, x, y) * uf(4, x, y) + uf(5, x, y) * uf(5, x, y);
    }
    block_sum3(be, ee, z);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = be;
        partial[gridDim.x + blockIdx.x] = ee;
    }
}

__global__ void k_sum_partials(const double *partial, int nparts, int nsets, double *out)
{
    // one thread per set, index order: deterministic
    const int s = threadIdx.x;
    if (s >= nsets) return;
    double acc = 0.0;
    for (int i = 0; i < nparts; ++i) acc += partial[(long long)s * nparts + i];
    out[s] = acc;
}

}  // namespace

// ========================================================================== host
static unsigned grid_for(long long n, int threads) { return (unsigned)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, 152LL * 16)); }

template <class FV>
int wm_launch_curre_bc(const WmGeom &g, FV uj, cudaStream_t st)
{
    k_curre_bc_y<FV><<<wm_div_up((g.nx + 4) * 3, 128), 128, 0, st>>>(g, uj);
    WM_TRY(wm_check_launch("k_curre_bc_y"));
    if (g.bc != WM_BC_PERIODIC) return WM_OK;  // walls: no x fold (boundary_reconnection.f90:364-502)
    k_curre_bc_x<FV><<<wm_div_up((g.ny + 4) * 3, 128), 128, 0, st>>>(g, uj);
    return wm_check_launch("k_curre_bc_x");
}

template <class FV>
int wm_launch_dfield_bc(const WmGeom &g, FV df, cudaStream_t st)
{
    k_dfield_bc_y<FV><<<wm_div_up(g.nx * 6, 128), 128, 0, st>>>(g, df);
    WM_TRY(wm_check_launch("k_dfield_bc_y"));
    k_dfield_bc_x<FV><<<wm_div_up((g.ny + 4) * 6, 128), 128, 0, st>>>(g, df);
    return wm_check_launch("k_dfield_bc_x");
}

int wm_launch_phi_bc(int nx, int ny, double *phi, int bc, int l, cudaStream_t st)
{
    k_phi_bc_y<<<wm_div_up(nx, 128), 128, 0, st>>>(nx, ny, phi);
    WM_TRY(wm_check_launch("k_phi_bc_y"));
    k_phi_bc_x<<<wm_div_up(ny + 2, 128), 128, 0, st>>>(nx, ny, phi, bc, l);
    return wm_check_launch("k_phi_bc_x");
}

int wm_launch_mom_bc(const WmGeom &g, double *mom, cudaStream_t st)
{
    k_mom_bc_x<<<wm_div_up((g.ny + 2) * g.nsp * 7, 128), 128, 0, st>>>(g, mom);
    WM_TRY(wm_check_launch("k_mom_bc_x"));
    k_mom_bc_y<<<wm_div_up((g.nx + 2) * g.nsp * 7, 128), 128, 0, st>>>(g, mom);
    return wm_check_launch("k_mom_bc_y");
}

int wm_launch_aos_to_soa(int nc, long long npts, const double *a, double *s, cudaStream_t st)
{
    if (nc == 6) k_aos_to_soa<6><<<grid_for(npts * 6, 256), 256, 0, st>>>(npts, a, s);
    else if (nc == 3) k_aos_to_soa<3><<<grid_for(npts * 3, 256), 256, 0, st>>>(npts, a, s);
    else return WM_ERR_BAD_ARG;
    return wm_check_launch("k_aos_to_soa");
}

int wm_launch_soa_to_aos(int nc, long long npts, const double *s, double *a, cudaStream_t st)
{
    if (nc == 6) k_soa_to_aos<6><<<grid_for(npts * 6, 256), 256, 0, st>>>(npts, s, a);
    else if (nc == 3) k_soa_to_aos<3><<<grid_for(npts * 3, 256), 256, 0, st>>>(npts, s, a);
    else return WM_ERR_BAD_ARG;
    return wm_check_launch("k_soa_to_aos");
}

// --------------------------------------------------------------- field solve
int wm_field_cg_blocks() { return CG_BLOCKS > CG_PHASE_BLOCKS ? CG_BLOCKS : CG_PHASE_BLOCKS; }  // the partials of the largest grid
size_t wm_field_scal_bytes() { return sizeof(CgScal) * 3; }

static FieldK make_fk(const WmConst &k)
{
    const double pi = 3.14159265358979311599796346854418516;
    FieldK fk;
    fk.f1 = k.c * k.delt / k.delx;
    fk.f2 = k.gfac * fk.f1 * fk.f1;
    fk.f3 = 4.0 * pi * k.delx / k.c;
    const double t = k.delx / (k.c * k.delt * k.gfac);
    fk.f4 = 4.0 + t * t;
    fk.f5 = t * t;
    fk.gfac = k.gfac;
    fk.pi4dt = 4. * pi * k.delt;
    fk.err = k.cg_err;
    fk.itemax = k.cg_itemax;
    return fk;
}


// field__fdtd_i after the deposit: curre BC, RHS, CG, dfield BC, delta-E, dfield BC, uf += df.
// iters[3] and the status are read back at the end.  cg_batch = CG iterations enqueued between
// host checks of the "still iterating" flags.
int wm_field_solve(const WmGeom &g, const WmConst &k, FView<6, false> uf, FView<3, false> uj, FView<6, false> df, WmFieldWork &w,
                   int *iters, int cg_batch, cudaStream_t st, wm_mark_fn mark, void *mctx, long long *launches, const WmGuess *guess)
{
    const FieldK fk = make_fk(k);
    long long nl = 0;
    auto M = [&](const char *n) {
        if (mark) mark(mctx, n);
    };
    WM_TRY(wm_launch_curre_bc(g, uj, st));
    nl += 2;
    M("curre_bc");
    k_cg_rhs<FView<6, false>, FView<3, false>><<<CG_BLOCKS, CG_THREADS, 0, st>>>(g, fk, uf, uj, w.b, w.partial, w.ticket, w.scal);
    WM_TRY(wm_check_launch("k_cg_rhs"));
    if (guess) {
        M("cg_setup");
        WM_TRY(guess->run(guess->ctx, st));
        M("guess_net");
        const PlaneView cv{guess->cand, g.nx, g.ny};
        k_guess_resid2<FView<6, false>><<<CG_BLOCKS, CG_THREADS, 0, st>>>(g, fk, cv, df, w.b, w.partial, w.ticket, guess->stats);
        WM_TRY(wm_check_launch("k_guess_resid2"));
        k_cg_resid_pick<FView<6, false>><<<CG_BLOCKS, CG_THREADS, 0, st>>>(g, fk, df, cv, w.b, w.r, w.p, w.partial, w.ticket, w.scal,
                                                                            guess->stats);
        WM_TRY(wm_check_launch("k_cg_resid_pick"));
        nl += 1;
    } else {
        k_cg_resid<FView<6, false>><<<CG_BLOCKS, CG_THREADS, 0, st>>>(g, fk, df, w.b, w.r, w.p, w.partial, w.ticket, w.scal);
        WM_TRY(wm_check_launch("k_cg_resid"));
    }
    nl += 2;
    M("cg_setup");
    // cg_batch iterations (3 launches each) between host checks of the "still iterating" flags;
    // launch t runs phase (t - l) mod 3 of component l
    const int t_max = 3 * (fk.itemax + 1) + 2;
    for (int t = 0;;) {
        WM_CUDA(cudaMemcpyAsync(w.scal_host, w.scal, sizeof(CgScal) * 3, cudaMemcpyDeviceToHost, st));
        WM_CUDA(cudaStreamSynchronize(st));
        const bool any = w.scal_host[0].active || w.scal_host[1].active || w.scal_host[2].active;
        if (!any || t >= t_max) break;
        for (int b = 0; b < 3 * cg_batch; ++b, ++t) {
            k_cg_phase<FView<6, false>><<<CG_PHASE_BLOCKS, CG_THREADS, 0, st>>>(g, fk, df, w.p, w.r, w.ap, w.partial, w.ticket, w.scal, t);
            ++nl;
        }
        WM_TRY(wm_check_launch("cg iteration"));
    }
    M("cg_iterate");
    int status = WM_OK;
    for (int l = 0; l < 3; ++l) {
        if (iters) iters[l] = w.scal_host[l].ite;
        if (w.scal_host[l].status) status = WM_ERR_CG_MAXITER;
    }
    if (status != WM_OK) return status;
    WM_TRY(wm_launch_dfield_bc(g, df, st));
    k_efield<FView<6, false>, FView<3, false>><<<grid_for((long long)g.nx * g.ny, 256), 256, 0, st>>>(g, fk, df, uf, uj);
    WM_TRY(wm_check_launch("k_efield"));
    WM_TRY(wm_launch_dfield_bc(g, df, st));
    k_field_add<FView<6, false>><<<grid_for((long long)g.nxw * g.nyw, 256), 256, 0, st>>>(g, uf, df);
    WM_TRY(wm_check_launch("k_field_add"));
    nl += 6;
    M("efield_update");
    if (launches) *launches += nl;
    return WM_OK;
}

int wm_launch_energy_fields(const WmGeom &g, FView<6, false> uf, double *partial, int nblocks, cudaStream_t st)
{
    k_energy_fields<FView<6, false>><<<nblocks, CG_THREADS, 0, st>>>(g, uf, partial);
    return wm_check_launch("k_energy_fields");
}

int wm_launch_sum_partials(const double *partial, int nparts, int nsets, double *out, cudaStream_t st)
{
    k_sum_partials<<<1, 32, 0, st>>>(partial, nparts, nsets, out);
    return wm_check_launch("k_sum_partials");
}

template int wm_launch_curre_bc<FView<3, false>>(const WmGeom &, FView<3, false>, cudaStream_t);
template int wm_launch_curre_bc<FView<3, true>>(const WmGeom &, FView<3, true>, cudaStream_t);
template int wm_launch_dfield_bc<FView<6, false>>(const WmGeom &, FView<6, false>, cudaStream_t);
template int wm_launch_dfield_bc<FView<6, true>>(const WmGeom &, FView<6, true>, cudaStream_t);
