// wm_particles.cu -- FP64 particle kernels for sm_103a.
//
//   k_push            particle__solv (common/particle.f90:48-177) and mom_calc__accl
//                     (common/mom_calc.f90:48-164): one thread per particle, one CTA per
//                     (row, 32-cell tile); the cell-centred fields of the tile and its one-cell
//                     halo are staged in shared memory (particle.f90:68-81).
//   k_deposit_cells   ele_cur (common/field.f90:189-316): one thread per cell walks the cell's
//                     particles in the reference's order and keeps the 5x5 partial currents
//                     pjx/pjy/pjz in registers; they are written per cell.
//   k_deposit_fold    adds the per-cell partial currents into uj node by node in the order of
//                     the reference's (j, i) cell loop, so the sum order is fixed and the result
//                     does not depend on scheduling.
//   k_mom_nvt         mom_calc__nvt (common/mom_calc.f90:167-249), CIC deposit of 7 moments.
//   k_energy_*        energy sums of proj/weibel/app.f90:507-534.
//
// The FP64 path is bound by the FP64 pipe, not by HBM: its kernels minimise FP64 instructions
// (fused multiply-adds, precomputed weights) and use integer/FP32 pipes for index work.
#include "wm_launch.cuh"

namespace {

constexpr int PUSH_TW = 32;      // cells per push tile
constexpr int PUSH_THREADS = 256;

template <class PV, class FV>
__global__ void __launch_bounds__(PUSH_THREADS) k_push(WmGeom g, WmConst kc, PV up, PV gp, FV uf,
                                                       const int *__restrict__ cumcnt, int half_step, int copy_pid)
{
    __shared__ double tmp[6][3][PUSH_TW + 2];
    __shared__ int cc[WM_MAX_SP][PUSH_TW + 1];
    const int j = g.nys + blockIdx.y;
    const int i0 = g.nxgs + blockIdx.x * PUSH_TW;
    const int ncell = min(PUSH_TW, g.nxgs + g.nxa - i0);  // cells nxs..nxe (particle.f90:86)
    if (ncell <= 0) return;                             // past nxe: the shock's box has not reached this tile
    const int tw = ncell + 2;

    // cell-centred fields tmp(1:6, i0-1:i0+ncell, j-1:j+1), particle.f90:68-81
    for (int e = threadIdx.x; e < 3 * tw; e += blockDim.x) {
        const int a = e % tw, b = e / tw;
        const int ix = (i0 - 1 + a) - (g.nxgs - 2), iy = (j - 1 + b) - (g.nys - 2);
        tmp[0][b][a] = 0.5 * (+uf(0, ix, iy) + uf(0, ix, iy + 1));
        tmp[1][b][a] = 0.5 * (+uf(1, ix, iy) + uf(1, ix + 1, iy));
        tmp[2][b][a] = 0.25 * (+uf(2, ix, iy) + uf(2, ix + 1, iy) + uf(2, ix, iy + 1) + uf(2, ix + 1, iy + 1));
        tmp[3][b][a] = 0.5 * (+uf(3, ix, iy) + uf(3, ix + 1, iy));
        tmp[4][b][a] = 0.5 * (+uf(4, ix, iy) + uf(4, ix, iy + 1));
        tmp[5][b][a] = uf(5, ix, iy);
    }
    for (int e = threadIdx.x; e < g.nsp * (ncell + 1); e += blockDim.x) {
        const int isp = e / (ncell + 1), c = e % (ncell + 1);
        const int row = isp * g.ny + (j - g.nys);
        cc[isp][c] = cumcnt[(i0 + c - g.nxgs) + (long long)(g.nx + 1) * row];
    }
    __syncthreads();
    // Each cell's particles are cumcnt(i)+1 .. cumcnt(i+1) (particle.f90:86-88), none where that
    // range is reversed: the shock application's injection raises cumcnt(nxe) alone, and past a
    // growing nxe the entry cumcnt(nxe+1) is not maintained.  The running maximum turns the
    // starts into one ascending sequence with the same cells.
    if (threadIdx.x < g.nsp)
        for (int c = 1; c <= ncell; ++c) cc[threadIdx.x][c] = max(cc[threadIdx.x][c], cc[threadIdx.x][c - 1]);
    __syncthreads();

    const double d_delx = 1. / kc.delx;
    const double delt = half_step ? kc.delt * 0.5 : kc.delt;
    const double c = kc.c;
    for (int isp = 0; isp < g.nsp; ++isp) {
        const int row = isp * g.ny + (j - g.nys);
        const double fac1 = kc.q[isp] / kc.r[isp] * 0.5 * delt;
        const double txxx = fac1 * fac1;
        const double fac2 = kc.q[isp] * delt / kc.r[isp];
        const int start = cc[isp][0], end = cc[isp][ncell];
        for (int s = start + threadIdx.x; s < end; s += blockDim.x) {
            int lo = 0, hi = ncell - 1;  // last cell whose start is <= s
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (cc[isp][mid] <= s) lo = mid;
                else hi = mid - 1;
            }
            const int i = i0 + lo;
            const long long p = up.idx(row, s);
            const double x = up.X(p), y = up.Y(p);
            double dh = x * d_delx - 0.5 - i;
            const double shx0 = 0.5 * (0.5 - dh) * (0.5 - dh), shx1 = 0.75 - dh * dh, shx2 = 0.5 * (0.5 + dh) * (0.5 + dh);
            dh = y * d_delx - 0.5 - j;
            const double shy0 = 0.5 * (0.5 - dh) * (0.5 - dh), shy1 = 0.75 - dh * dh, shy2 = 0.5 * (0.5 + dh) * (0.5 + dh);
            double f[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const double *t0 = &tmp[k][0][lo], *t1 = &tmp[k][1][lo], *t2 = &tmp[k][2][lo];
                f[k] = (+t0[0] * shx0 + t0[1] * shx1 + t0[2] * shx2) * shy0 + (+t1[0] * shx0 + t1[1] * shx1 + t1[2] * shx2) * shy1
                       + (+t2[0] * shx0 + t2[1] * shx1 + t2[2] * shx2) * shy2;
            }
            const double bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
            double uvm1 = up.UX(p) + fac1 * epx;
            double uvm2 = up.UY(p) + fac1 * epy;
            double uvm3 = up.UZ(p) + fac1 * epz;
            const double gam = sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
            const double igam = 1. / gam;
            const double fac1r = fac1 * igam;
            const double fac2r = fac2 / (gam + txxx * (bpx * bpx + bpy * bpy + bpz * bpz) * igam);
            const double uvm4 = uvm1 + fac1r * (+uvm2 * bpz - uvm3 * bpy);
            const double uvm5 = uvm2 + fac1r * (+uvm3 * bpx - uvm1 * bpz);
            const double uvm6 = uvm3 + fac1r * (+uvm1 * bpy - uvm2 * bpx);
            uvm1 = uvm1 + fac2r * (+uvm5 * bpz - uvm6 * bpy);
            uvm2 = uvm2 + fac2r * (+uvm6 * bpx - uvm4 * bpz);
            uvm3 = uvm3 + fac2r * (+uvm4 * bpy - uvm5 * bpx);
            const double u1 = uvm1 + fac1 * epx, u2 = uvm2 + fac1 * epy, u3 = uvm3 + fac1 * epz;
            gp.UX(p) = u1;
            gp.UY(p) = u2;
            gp.UZ(p) = u3;
            if (half_step) {
                gp.X(p) = x;
                gp.Y(p) = y;
            } else {
                const double ig = 1. / sqrt(1.0 + (+u1 * u1 + u2 * u2 + u3 * u3) / (c * c));
                gp.X(p) = x + u1 * delt * ig;
                gp.Y(p) = y + u2 * delt * ig;
                if (copy_pid) gp.setpid(p, up.getpid(p));
            }
        }
    }
}

__global__ void k_pid_copy_aos(double *__restrict__ gp, const double *__restrict__ up, long long nslots)
{
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nslots; s += (long long)gridDim.x * blockDim.x)
        gp[6 * s + 5] = up[6 * s + 5];
}

// ------------------------------------------------------------------ deposit
constexpr int DEP_THREADS = 128;

// pj layout: [75][ncell]; component c in 0..74 = comp*25 + (jp+2)*5 + (ip+2).
template <class PV>
__global__ void __launch_bounds__(DEP_THREADS) k_deposit_cells(WmGeom g, WmConst kc, PV up, PV gp,
                                                               const int *__restrict__ cumcnt, double *__restrict__ pj,
                                                               unsigned *status)
{
    const int ncell = g.nx * g.ny;
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncell) return;
    const int ci = cell % g.nx, cj = cell / g.nx;
    const int i = g.nxgs + ci, j = g.nys + cj;
    const double d_delx = 1. / kc.delx, d_delt = 1. / kc.delt;
    const double fac = 1.0 / 3.0;
    const double c2 = kc.c * kc.c;

    double ax[5][4];  // pjx(ip=-1..2, jp=-2..2): [jp+2][ip+1]
    double ay[4][5];  // pjy(ip=-2..2, jp=-1..2): [jp+1][ip+2]
    double az[5][5];  // pjz(ip, jp): [jp+2][ip+2]
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            ax[a][b] = 0.0;
            ay[b][a] = 0.0;
        }
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) az[a][b] = 0.0;

    unsigned bad = 0;
    for (int isp = 0; isp < g.nsp; ++isp) {
        const int row = isp * g.ny + cj;
        const long long ccb = (long long)(g.nx + 1) * row;
        // cells nxs..nxe (field.f90:213); past nxe cumcnt is not maintained (the shock's box)
        const int s_beg = ci < g.nxa ? cumcnt[ccb + ci] : 0, s_end = ci < g.nxa ? cumcnt[ccb + ci + 1] : 0;
        const double qs = kc.q[isp];
        const double mqdd = -(qs * kc.delx * d_delt);
        for (int s = s_beg; s < s_end; ++s) {
            const long long p = up.idx(row, s);
            const double x0 = up.X(p), y0 = up.Y(p);
            const double x1 = gp.X(p), y1 = gp.Y(p);
            const double u3 = gp.UX(p), u4 = gp.UY(p), u5 = gp.UZ(p);
            double s0x[5], s0y[5], dsx[5], dsy[5];
            double dh = x0 * d_delx - 0.5 - i;
            s0x[0] = 0.0;
            s0x[1] = 0.5 * (0.5 - dh) * (0.5 - dh);
            s0x[2] = 0.75 - dh * dh;
            s0x[3] = 0.5 * (0.5 + dh) * (0.5 + dh);
            s0x[4] = 0.0;
            dh = y0 * d_delx - 0.5 - j;
            s0y[0] = 0.0;
            s0y[1] = 0.5 * (0.5 - dh) * (0.5 - dh);
            s0y[2] = 0.75 - dh * dh;
            s0y[3] = 0.5 * (0.5 + dh) * (0.5 + dh);
            s0y[4] = 0.0;
            // new shape, shifted by inc = i2 - i in {-1,0,1} (field.f90:238-266)
            int i2 = (int)(x1 * d_delx);
            dh = x1 * d_delx - 0.5 - i2;
            int inc = i2 - i;
            bad |= (inc < -1 || inc > 1);
            {
                const double a0 = 0.5 * (0.5 - dh) * (0.5 - dh), a1 = 0.75 - dh * dh, a2 = 0.5 * (0.5 + dh) * (0.5 + dh);
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const int o = m - 2 - inc;  // offset into (a0,a1,a2) at -1..1
                    const double s1 = (o == -1) ? a0 : (o == 0) ? a1 : (o == 1) ? a2 : 0.0;
                    dsx[m] = s1 - s0x[m];
                }
            }
            i2 = (int)(y1 * d_delx);
            dh = y1 * d_delx - 0.5 - i2;
            inc = i2 - j;
            bad |= (inc < -1 || inc > 1);
            {
                const double a0 = 0.5 * (0.5 - dh) * (0.5 - dh), a1 = 0.75 - dh * dh, a2 = 0.5 * (0.5 + dh) * (0.5 + dh);
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const int o = m - 2 - inc;
                    const double s1 = (o == -1) ? a0 : (o == 0) ? a1 : (o == 1) ? a2 : 0.0;
                    dsy[m] = s1 - s0y[m];
                }
            }
            const double gvz = u5 / sqrt(1. + (+u3 * u3 + u4 * u4 + u5 * u5) / c2);
            const double qg = qs * gvz;
            // Jx: pjx(ip+1,jp) = pjx(ip,jp) - q dx/dt ds_x(ip) (s0y + ds_y/2)  -> prefix sums of ds_x
            double wy[5], wx[5], z2[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                wy[m] = s0y[m] + 0.5 * dsy[m];
                wx[m] = s0x[m] + 0.5 * dsx[m];
                z2[m] = qg * (0.5 * s0y[m] + fac * dsy[m]);
            }
            double cx[4], cy[4];
            cx[0] = dsx[0];
            cx[1] = cx[0] + dsx[1];
            cx[2] = cx[1] + dsx[2];
            cx[3] = cx[2] + dsx[3];
            cy[0] = dsy[0];
            cy[1] = cy[0] + dsy[1];
            cy[2] = cy[1] + dsy[2];
            cy[3] = cy[2] + dsy[3];
#pragma unroll
            for (int jp = 0; jp < 5; ++jp) {
                const double fy = mqdd * wy[jp];
#pragma unroll
                for (int k = 0; k < 4; ++k) ax[jp][k] = fma(fy, cx[k], ax[jp][k]);
            }
#pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                const double fx = mqdd * wx[ip];
#pragma unroll
                for (int k = 0; k < 4; ++k) ay[k][ip] = fma(fx, cy[k], ay[k][ip]);
            }
#pragma unroll
            for (int jp = 0; jp < 5; ++jp) {
                const double z1 = qg * wy[jp];
#pragma unroll
                for (int ip = 0; ip < 5; ++ip) az[jp][ip] = fma(s0x[ip], z1, fma(dsx[ip], z2[jp], az[jp][ip]));
            }
        }
    }
    if (bad) atomicOr(status, (unsigned)WMDEV_CELL);
    // write the 5x5x3 partial currents of this cell (zeros where the reference's pj is 0)
#pragma unroll
    for (int jp = 0; jp < 5; ++jp)
#pragma unroll
        for (int ip = 0; ip < 5; ++ip) {
            pj[(long long)(0 * 25 + jp * 5 + ip) * ncell + cell] = (ip == 0) ? 0.0 : ax[jp][ip - 1];
            pj[(long long)(1 * 25 + jp * 5 + ip) * ncell + cell] = (jp == 0) ? 0.0 : ay[jp - 1][ip];
            pj[(long long)(2 * 25 + jp * 5 + ip) * ncell + cell] = az[jp][ip];
        }
}

// uj(k, I, J) over the whole ghosted grid = sum over cells (j, i) with |I-i|,|J-j| <= 2 of
// pj_k(I-i, J-j), in the (j ascending, i ascending) order of the reference's cell loop.
template <class FV3>
__global__ void k_deposit_fold(WmGeom g, FV3 uj, const double *__restrict__ pj)
{
    const int ncell = g.nx * g.ny;
    const long long n = (long long)g.nxw * g.nyw;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(e % g.nxw), iy = (int)(e / g.nxw);
        // node (I,J) = (ix + nxgs-2, iy + nys-2); contributing interior cells ci in [ix-4, ix], cj in [iy-4, iy]
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int cj = iy - 4; cj <= iy; ++cj) {
            if (cj < 0 || cj >= g.ny) continue;
            const int jp = iy - 2 - cj;  // J - j in -2..2
            for (int ci = ix - 4; ci <= ix; ++ci) {
                if (ci < 0 || ci >= g.nx) continue;
                const int ip = ix - 2 - ci;
                const int cell = cj * g.nx + ci;
                const int o = (jp + 2) * 5 + (ip + 2);
                s0 = s0 + pj[(long long)(0 * 25 + o) * ncell + cell];
                s1 = s1 + pj[(long long)(1 * 25 + o) * ncell + cell];
                s2 = s2 + pj[(long long)(2 * 25 + o) * ncell + cell];
            }
        }
        uj(0, ix, iy) = s0;
        uj(1, ix, iy) = s1;
        uj(2, ix, iy) = s2;
    }
}

// ------------------------------------------------------------------ moments
// mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp) in the reference layout on the device.
template <class PV>
__global__ void k_mom_nvt(WmGeom g, WmConst kc, PV up, const int *__restrict__ np2, double *__restrict__ mom)
{
    const int row = blockIdx.y;
    const int isp = row / g.ny;
    const int n = np2[row];
    const double d_delx = 1. / kc.delx, c2 = kc.c * kc.c;
    const int mx = g.nx + 2, my = g.ny + 2;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const long long p = up.idx(row, s);
        const double x = up.X(p), y = up.Y(p), u3 = up.UX(p), u4 = up.UY(p), u5 = up.UZ(p);
        const int ih = (int)(x * d_delx - 0.5);
        const int jh = (int)(y * d_delx - 0.5);
        const double dx = x * d_delx - 0.5 - ih, dxm = 1. - dx;
        const double dy = y * d_delx - 0.5 - jh, dym = 1. - dy;
        const double gam = 1. / sqrt(1.0 + (+u3 * u3 + u4 * u4 + u5 * u5) / c2);
        const int bx = ih - (g.nxgs - 1), by = jh - (g.nys - 1);
        if (bx < 0 || bx + 1 >= mx || by < 0 || by + 1 >= my) continue;
        double *m00 = mom + 7 * (bx + (long long)mx * (by + (long long)my * isp));
        double *m10 = m00 + 7;
        double *m01 = m00 + 7 * mx;
        double *m11 = m01 + 7;
        const double w00 = dxm * dym, w10 = dx * dym, w01 = dxm * dy, w11 = dx * dy;
        atomicAdd(m00, w00);
        atomicAdd(m10, w10);
        atomicAdd(m01, w01);
        atomicAdd(m11, w11);
        const double v[6] = {u3, u4, u5, u3 * u3, u4 * u4, u5 * u5};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double vg = v[k] * gam;
            atomicAdd(m00 + 1 + k, vg * dxm * dym);
            atomicAdd(m10 + 1 + k, vg * dx * dym);
            atomicAdd(m01 + 1 + k, vg * dxm * dy);
            atomicAdd(m11 + 1 + k, vg * dx * dy);
        }
    }
}

// --------------------------------------------------------------- energy sums
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double sh[RED_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = (l < RED_THREADS / 32) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;  // valid in thread 0
}

// partial[isp * gridDim.x + block] = sum over the block's particles of r (gamma - 1)
template <class PV>
__global__ void __launch_bounds__(RED_THREADS) k_energy_particles(WmGeom g, WmConst kc, PV up, const int *__restrict__ np2,
                                                                  double *__restrict__ partial)
{
    const double c2 = kc.c * kc.c;
    for (int isp = 0; isp < g.nsp; ++isp) {
        double acc = 0.0;
        for (int rj = 0; rj < g.ny; ++rj) {
            const int row = isp * g.ny + rj;
            const int n = np2[row];
            for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
                const long long p = up.idx(row, s);
                const double u3 = up.UX(p), u4 = up.UY(p), u5 = up.UZ(p);
                const double u2 = u3 * u3 + u4 * u4 + u5 * u5;
                acc += kc.r[isp] * (sqrt(1 + u2 / c2) - 1);
            }
        }
        acc = block_sum(acc);
        if (threadIdx.x == 0) partial[isp * gridDim.x + blockIdx.x] = acc;
    }
}

}  // namespace

// ======================================================================= launchers
template <class PV, class FV>
int wm_launch_push(const WmGeom &g, const WmConst &k, PV up, PV gp, FV uf, const int *cumcnt, int half_step, int copy_pid,
                   cudaStream_t st)
{
    dim3 grid(wm_div_up(g.nx, PUSH_TW), g.ny);
    k_push<PV, FV><<<grid, PUSH_THREADS, 0, st>>>(g, k, up, gp, uf, cumcnt, half_step, copy_pid);
    return wm_check_launch("k_push");
}

int wm_launch_pid_copy_aos(double *gp, const double *up, long long nslots, cudaStream_t st)
{
    k_pid_copy_aos<<<1216, 256, 0, st>>>(gp, up, nslots);
    return wm_check_launch("k_pid_copy_aos");
}

template <class PV>
int wm_launch_deposit_cells(const WmGeom &g, const WmConst &k, PV up, PV gp, const int *cumcnt, double *pjcell,
                            unsigned *status, cudaStream_t st)
{
    const int ncell = g.nx * g.ny;
    k_deposit_cells<PV><<<wm_div_up(ncell, DEP_THREADS), DEP_THREADS, 0, st>>>(g, k, up, gp, cumcnt, pjcell, status);
    return wm_check_launch("k_deposit_cells");
}

template <class FV3>
int wm_launch_deposit_fold(const WmGeom &g, FV3 uj, const double *pjcell, cudaStream_t st)
{
    const long long n = (long long)g.nxw * g.nyw;
    const unsigned blocks = (unsigned)std::min<long long>(wm_div_up(n, 256), 152 * 16);
    k_deposit_fold<FV3><<<blocks, 256, 0, st>>>(g, uj, pjcell);
    return wm_check_launch("k_deposit_fold");
}

template <class PV>
int wm_launch_mom_nvt(const WmGeom &g, const WmConst &k, PV up, const int *np2, double *mom, int max_row_count, cudaStream_t st)
{
    const size_t bytes = sizeof(double) * 7 * (size_t)(g.nx + 2) * (size_t)(g.ny + 2) * (size_t)g.nsp;
    WM_CUDA(cudaMemsetAsync(mom, 0, bytes, st));
    if (max_row_count <= 0) return WM_OK;
    dim3 grid(std::min(wm_div_up(max_row_count, 256), 64u), g.nrows);
    k_mom_nvt<PV><<<grid, 256, 0, st>>>(g, k, up, np2, mom);
    return wm_check_launch("k_mom_nvt");
}

template <class PV>
int wm_launch_energy_particles(const WmGeom &g, const WmConst &k, PV up, const int *np2, double *partial, int nblocks,
                               cudaStream_t st)
{
    k_energy_particles<PV><<<nblocks, RED_THREADS, 0, st>>>(g, k, up, np2, partial);
    return wm_check_launch("k_energy_particles");
}

// explicit instantiations
template int wm_launch_push<SoAView, FView<6, false>>(const WmGeom &, const WmConst &, SoAView, SoAView, FView<6, false>,
                                                     const int *, int, int, cudaStream_t);
template int wm_launch_push<AoSView, FView<6, true>>(const WmGeom &, const WmConst &, AoSView, AoSView, FView<6, true>,
                                                    const int *, int, int, cudaStream_t);
template int wm_launch_push<AoSView, FView<6, false>>(const WmGeom &, const WmConst &, AoSView, AoSView, FView<6, false>,
                                                     const int *, int, int, cudaStream_t);
template int wm_launch_deposit_cells<SoAView>(const WmGeom &, const WmConst &, SoAView, SoAView, const int *, double *,
                                              unsigned *, cudaStream_t);
template int wm_launch_deposit_cells<AoSView>(const WmGeom &, const WmConst &, AoSView, AoSView, const int *, double *,
                                              unsigned *, cudaStream_t);
template int wm_launch_deposit_fold<FView<3, false>>(const WmGeom &, FView<3, false>, const double *, cudaStream_t);
template int wm_launch_deposit_fold<FView<3, true>>(const WmGeom &, FView<3, true>, const double *, cudaStream_t);
template int wm_launch_mom_nvt<SoAView>(const WmGeom &, const WmConst &, SoAView, const int *, double *, int, cudaStream_t);
template int wm_launch_mom_nvt<AoSView>(const WmGeom &, const WmConst &, AoSView, const int *, double *, int, cudaStream_t);
template int wm_launch_energy_particles<SoAView>(const WmGeom &, const WmConst &, SoAView, const int *, double *, int,
                                                 cudaStream_t);
template int wm_launch_energy_particles<AoSView>(const WmGeom &, const WmConst &, AoSView, const int *, double *, int,
                                                 cudaStream_t);
template int wm_launch_energy_particles<MixedView>(const WmGeom &, const WmConst &, MixedView, const int *, double *, int,
                                                   cudaStream_t);
