// wm_mixed.cu -- the mixed-precision particle kernels (FP32 push and deposit) for sm_103a.
//
// Particles carry their position as (cell, FP32 offset in [0,1)) -- the cell is implicit in the
// cell-sorted rows -- and FP32 momenta.  k_mixed_push_deposit does, for one (species, row, 32-cell
// tile): the cell-centred fields of particle.f90:68-81 staged in shared memory as FP32, the
// Buneman-Boris push of particle.f90:96-161 in FP32, the Esirkepov deposit of field.f90:224-298 in
// FP32, the periodic wrap of boundary_periodic.f90:61-96 and :143-165 as integer cell arithmetic,
// and the destination cell key and row direction the rebin needs.  Eight lanes share a cell and
// read its particles in 32-byte runs straight from global memory; each lane keeps the cell's 5x5x3
// partial currents in registers (the cell's particles all deposit on the same 5x5 nodes), the
// eight lanes add theirs with shuffles, and the tile's node currents are summed from the per-cell
// partials in a fixed order.  Tile currents go to a per-tile buffer; k_mixed_jfold adds them into
// the FP64 global J node by node in a fixed order, so the result is deterministic and no atomics
// touch the currents.
#include <algorithm>

#include "wm_launch.cuh"

namespace {

constexpr int MX_TW = 32;   // cells per tile (one row, one species)
constexpr int MX_LPC = 8;   // lanes per cell
constexpr int MX_THREADS = MX_TW * MX_LPC;
constexpr int MX_JW = MX_TW + 4;
constexpr unsigned FULL = 0xffffffffu;

struct MxConst {
    float fac1[WM_MAX_SP], txxx[WM_MAX_SP], fac2[WM_MAX_SP], mqdd[WM_MAX_SP], q[WM_MAX_SP];
    float dt_dx, inv_c2, c2;
};

__device__ __forceinline__ void shape3(float h, float &a0, float &a1, float &a2)
{
    a0 = 0.5f * (0.5f - h) * (0.5f - h);
    a1 = 0.75f - h * h;
    a2 = 0.5f * (0.5f + h) * (0.5f + h);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// One CTA per (tile of 32 cells, row, species); 8 lanes per cell read the cell's particles in
// 32-byte runs straight from global memory.  Each lane keeps the cell's 5x5x3 partial currents in
// registers; the 8 lanes of a cell add theirs with shuffles, and the tile's node currents are then
// summed from the per-cell partials in a fixed order (no atomics on the currents).
__global__ void __launch_bounds__(MX_THREADS, 2)
    k_mixed_push_deposit(WmGeom g, MxConst kc, MixedView a, MixedView b, FView<6, false> uf, const int *__restrict__ cumcnt,
                         int *__restrict__ key, unsigned char *__restrict__ dir, int *__restrict__ cellcnt,
                         float *__restrict__ jtile, unsigned *status)
{
    __shared__ float tmp[6][3][MX_TW + 2];
    __shared__ float cellpj[65][MX_TW + 1];
    __shared__ int cc[MX_TW + 1];
    __shared__ float spc[5];
    const int tile = blockIdx.x, jr = blockIdx.y, isp = blockIdx.z;
    const int row = isp * g.ny + jr;
    const int c0 = tile * MX_TW;
    const int ncell = min(MX_TW, g.nx - c0);
    const int tid = threadIdx.x, lane = tid & 31;

    // fields at cell centres (i+1/2, j+1/2) for cells c0-1 .. c0+ncell and rows jr-1 .. jr+1
    const int tw = ncell + 2;
    for (int e = tid; e < 3 * tw; e += MX_THREADS) {
        const int aa = e % tw, bb = e / tw;
        const int ix = c0 - 1 + aa + 2, iy = jr - 1 + bb + 2;
        tmp[0][bb][aa] = (float)(0.5 * (uf(0, ix, iy) + uf(0, ix, iy + 1)));
        tmp[1][bb][aa] = (float)(0.5 * (uf(1, ix, iy) + uf(1, ix + 1, iy)));
        tmp[2][bb][aa] = (float)(0.25 * (uf(2, ix, iy) + uf(2, ix + 1, iy) + uf(2, ix, iy + 1) + uf(2, ix + 1, iy + 1)));
        tmp[3][bb][aa] = (float)(0.5 * (uf(3, ix, iy) + uf(3, ix + 1, iy)));
        tmp[4][bb][aa] = (float)(0.5 * (uf(4, ix, iy) + uf(4, ix, iy + 1)));
        tmp[5][bb][aa] = (float)uf(5, ix, iy);
    }
    const int *ccrow = cumcnt + (long long)(g.nx + 1) * row;
    for (int e = tid; e <= ncell; e += MX_THREADS) cc[e] = ccrow[c0 + e];
    if (tid == 0) {  // this species' constants (static indices: no local-memory copy)
#pragma unroll
        for (int s = 0; s < WM_MAX_SP; ++s)
            if (s == isp) {
                spc[0] = kc.fac1[s];
                spc[1] = kc.txxx[s];
                spc[2] = kc.fac2[s];
                spc[3] = kc.mqdd[s];
                spc[4] = kc.q[s];
            }
    }
    __syncthreads();

    const float fac1 = spc[0], txxx = spc[1], fac2 = spc[2], mqdd = spc[3], qs = spc[4];
    const int c = tid / MX_LPC, sub = tid % MX_LPC;
    const bool has_cell = c < ncell;
    const int s_beg = has_cell ? cc[c] : 0, s_end = has_cell ? cc[c + 1] : 0;
    const int nmine = (s_end - s_beg > sub) ? (s_end - s_beg - sub + MX_LPC - 1) / MX_LPC : 0;
    int nwarp = nmine;  // trip count of the warp: the largest over its lanes
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nwarp = max(nwarp, __shfl_xor_sync(FULL, nwarp, o));
    const long long rbase = a.rowbase[row];
    const int cl = has_cell ? c : 0;  // safe index for lanes without a cell

    float ax[5][4], ay[4][5], az[5][5];
#pragma unroll
    for (int jp = 0; jp < 5; ++jp)
#pragma unroll
        for (int ip = 0; ip < 5; ++ip) {
            if (ip < 4) ax[jp][ip] = 0.f;
            if (jp < 4) ay[jp][ip] = 0.f;
            az[jp][ip] = 0.f;
        }
    unsigned bad = 0;
    for (int it = 0; it < nwarp; ++it) {
        const bool valid = it < nmine;
        int kk = -1;
        if (valid) {
            const long long p = rbase + s_beg + sub + (long long)it * MX_LPC;
            const float dx = a.x[p], dy = a.y[p];
            float u1 = a.ux[p], u2 = a.uy[p], u3 = a.uz[p];
            float sx0, sx1, sx2, sy0, sy1, sy2;
            shape3(dx - 0.5f, sx0, sx1, sx2);
            shape3(dy - 0.5f, sy0, sy1, sy2);
            float f[6];
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                const float *t0 = &tmp[m][0][cl], *t1 = &tmp[m][1][cl], *t2 = &tmp[m][2][cl];
                f[m] = (t0[0] * sx0 + t0[1] * sx1 + t0[2] * sx2) * sy0 + (t1[0] * sx0 + t1[1] * sx1 + t1[2] * sx2) * sy1
                       + (t2[0] * sx0 + t2[1] * sx1 + t2[2] * sx2) * sy2;
            }
            // Buneman-Boris
            float v1 = u1 + fac1 * f[3], v2 = u2 + fac1 * f[4], v3 = u3 + fac1 * f[5];
            const float g2 = kc.c2 + v1 * v1 + v2 * v2 + v3 * v3;
            const float igam = rsqrtf(g2);
            const float gam = g2 * igam;
            const float fac1r = fac1 * igam;
            const float fac2r = fac2 / (gam + txxx * (f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) * igam);
            const float w4 = v1 + fac1r * (v2 * f[2] - v3 * f[1]);
            const float w5 = v2 + fac1r * (v3 * f[0] - v1 * f[2]);
            const float w6 = v3 + fac1r * (v1 * f[1] - v2 * f[0]);
            v1 = v1 + fac2r * (w5 * f[2] - w6 * f[1]);
            v2 = v2 + fac2r * (w6 * f[0] - w4 * f[2]);
            v3 = v3 + fac2r * (w4 * f[1] - w5 * f[0]);
            u1 = v1 + fac1 * f[3];
            u2 = v2 + fac1 * f[4];
            u3 = v3 + fac1 * f[5];
            const float ig = rsqrtf(1.f + (u1 * u1 + u2 * u2 + u3 * u3) * kc.inv_c2);
            // move in cell units; a step crosses at most one cell (c dt < dx)
            float nx1 = dx + u1 * kc.dt_dx * ig, ny1 = dy + u2 * kc.dt_dx * ig;
            int incx = (int)floorf(nx1), incy = (int)floorf(ny1);
            nx1 -= (float)incx;
            ny1 -= (float)incy;
            if (nx1 >= 1.f) {
                nx1 -= 1.f;
                ++incx;
            }
            if (ny1 >= 1.f) {
                ny1 -= 1.f;
                ++incy;
            }
            bad |= (incx < -1 || incx > 1 || incy < -1 || incy > 1);
            // Esirkepov: old shape about the old cell, new shape about the new cell shifted by inc
            float dsx[5], dsy[5];
            const float s0x[5] = {0.f, sx0, sx1, sx2, 0.f}, s0y[5] = {0.f, sy0, sy1, sy2, 0.f};
            {
                float b0, b1, b2;
                shape3(nx1 - 0.5f, b0, b1, b2);
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const int o = m - 2 - incx;
                    dsx[m] = ((o == -1) ? b0 : (o == 0) ? b1 : (o == 1) ? b2 : 0.f) - s0x[m];
                }
                shape3(ny1 - 0.5f, b0, b1, b2);
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const int o = m - 2 - incy;
                    dsy[m] = ((o == -1) ? b0 : (o == 0) ? b1 : (o == 1) ? b2 : 0.f) - s0y[m];
                }
            }
            const float qg = qs * u3 * ig;
            float cx[4], cy[4];
            cx[0] = dsx[0];
            cy[0] = dsy[0];
#pragma unroll
            for (int m = 1; m < 4; ++m) {
                cx[m] = cx[m - 1] + dsx[m];
                cy[m] = cy[m - 1] + dsy[m];
            }
#pragma unroll
            for (int jp = 0; jp < 5; ++jp) {
                const float wy = s0y[jp] + 0.5f * dsy[jp];
                const float fy = mqdd * wy;
#pragma unroll
                for (int m = 0; m < 4; ++m) ax[jp][m] = fmaf(fy, cx[m], ax[jp][m]);
                const float z1 = qg * wy;
                const float z2 = qg * (0.5f * s0y[jp] + (1.f / 3.f) * dsy[jp]);
#pragma unroll
                for (int ip = 0; ip < 5; ++ip) az[jp][ip] = fmaf(s0x[ip], z1, fmaf(dsx[ip], z2, az[jp][ip]));
            }
#pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                const float fx = mqdd * (s0x[ip] + 0.5f * dsx[ip]);
#pragma unroll
                for (int m = 0; m < 4; ++m) ay[m][ip] = fmaf(fx, cy[m], ay[m][ip]);
            }
            b.x[p] = nx1;
            b.y[p] = ny1;
            b.ux[p] = u1;
            b.uy[p] = u2;
            b.uz[p] = u3;
            int ci = c0 + c + incx;
            ci = ci < 0 ? ci + g.nx : (ci >= g.nx ? ci - g.nx : ci);
            int kr = jr + incy;
            kr = kr < 0 ? kr + g.ny : (kr >= g.ny ? kr - g.ny : kr);
            kk = (isp * g.ny + kr) * g.nx + ci;
            key[p] = kk;
            dir[p] = (unsigned char)(incy == 1 ? 1 : (incy == -1 ? 2 : 0));
        }
        // cell counts for the sort, aggregated over the lanes that share a destination
        const unsigned m = __ballot_sync(FULL, valid);
        if (valid) {
            const unsigned peers = __match_any_sync(m, kk);
            if ((peers & lanemask_lt()) == 0) atomicAdd(&cellcnt[kk], __popc(peers));
        }
    }
    if (bad) atomicOr(status, (unsigned)WMDEV_CELL);

    // the 8 lanes of a cell add their partial currents; lane 0 of the cell keeps the sum
#pragma unroll
    for (int jp = 0; jp < 5; ++jp)
#pragma unroll
        for (int ip = 0; ip < 5; ++ip) {
#pragma unroll
            for (int o = 1; o < MX_LPC; o <<= 1) {
                if (ip < 4) ax[jp][ip] += __shfl_xor_sync(FULL, ax[jp][ip], o);
                if (jp < 4) ay[jp][ip] += __shfl_xor_sync(FULL, ay[jp][ip], o);
                az[jp][ip] += __shfl_xor_sync(FULL, az[jp][ip], o);
            }
        }
    if (sub == 0 && has_cell) {
#pragma unroll
        for (int jp = 0; jp < 5; ++jp)
#pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                if (ip < 4) cellpj[jp * 4 + ip][c] = ax[jp][ip];
                if (jp < 4) cellpj[20 + jp * 5 + ip][c] = ay[jp][ip];
                cellpj[40 + jp * 5 + ip][c] = az[jp][ip];
            }
    }
    __syncthreads();
    // node currents of the tile footprint (5 rows x (32+4) columns), cells in ascending order;
    // per-tile buffer [isp][jr][tile][3][5][MX_JW]
    float *out = jtile + ((((long long)isp * g.ny + jr) * gridDim.x + tile) * 3) * 5 * MX_JW;
    for (int e = tid; e < 3 * 5 * MX_JW; e += MX_THREADS) {
        const int k = e / (5 * MX_JW), ly = (e / MX_JW) % 5, lx = e % MX_JW;
        float sum = 0.f;
        for (int cc2 = max(0, lx - 4); cc2 <= min(ncell - 1, lx); ++cc2) {
            const int ip = lx - cc2;
            if (k == 0) {
                if (ip >= 1) sum += cellpj[ly * 4 + ip - 1][cc2];
            } else if (k == 1) {
                if (ly >= 1) sum += cellpj[20 + (ly - 1) * 5 + ip][cc2];
            } else {
                sum += cellpj[40 + ly * 5 + ip][cc2];
            }
        }
        out[e] = sum;
    }
}


// uj(k, ix, iy) over the ghosted grid = sum of the tile currents that cover the node, in the
// order (species, cell row, tile), accumulated in FP64.
__global__ void k_mixed_jfold(WmGeom g, int ntiles, const float *__restrict__ jtile, FView<3, false> uj)
{
    const long long n = (long long)g.nxw * g.nyw;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(e % g.nxw), iy = (int)(e / g.nxw);
        double s[3] = {0.0, 0.0, 0.0};
        const int t_lo = max(0, (ix - MX_JW + 1 + MX_TW - 1) / MX_TW), t_hi = min(ntiles - 1, ix / MX_TW);
        for (int isp = 0; isp < g.nsp; ++isp)
            for (int cj = max(0, iy - 4); cj <= min(g.ny - 1, iy); ++cj) {
                const int ly = iy - cj;
                for (int t = t_lo; t <= t_hi; ++t) {
                    const int lx = ix - t * MX_TW;
                    if (lx < 0 || lx >= MX_JW) continue;
                    const float *base = jtile + ((((long long)isp * g.ny + cj) * ntiles + t) * 3) * 5 * MX_JW;
#pragma unroll
                    for (int k = 0; k < 3; ++k) s[k] += (double)base[(k * 5 + ly) * MX_JW + lx];
                }
            }
        uj(0, ix, iy) = s[0];
        uj(1, ix, iy) = s[1];
        uj(2, ix, iy) = s[2];
    }
}

// FP64 reference-layout staging (pitch slots per row) -> mixed set; key = row * nx + cell for the
// load-time sort.  Offsets are taken against the particle's own cell int(x) and its row.
__global__ void k_mixed_unpack(WmGeom g, const double *__restrict__ stage, int pitch, const int *__restrict__ np2, MixedView dst,
                               int *__restrict__ key, int *__restrict__ cellcnt, unsigned *status)
{
    const int row = blockIdx.y;
    const int jr = row % g.ny;
    const int n = np2[row];
    unsigned bad = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const double *a = stage + 6 * ((long long)row * pitch + s);
        const long long p = dst.idx(row, s);
        const int ci = (int)a[0] - g.nxgs;
        float ox = (float)(a[0] - (double)(g.nxgs + ci));
        float oy = (float)(a[1] - (double)(g.nys + jr));
        if (ox >= 1.f) ox = 0x1.fffffep-1f;  // rounding up to 1 would leave the cell
        if (oy >= 1.f) oy = 0x1.fffffep-1f;
        if (ci < 0 || ci >= g.nx || !(oy >= 0.f)) {
            bad = 1;
            key[p] = 0;
            continue;
        }
        dst.X(p) = ox;
        dst.Y(p) = oy;
        dst.UX(p) = (float)a[2];
        dst.UY(p) = (float)a[3];
        dst.UZ(p) = (float)a[4];
        dst.setpid(p, __double_as_longlong(a[5]));
        const int k = row * g.nx + ci;
        key[p] = k;
        atomicAdd(&cellcnt[k], 1);
    }
    if (bad) atomicOr(status, (unsigned)WMDEV_CELL);
}

// mixed set -> FP64 reference-layout staging; the cell of each particle comes from cumcnt.
__global__ void k_mixed_pack(WmGeom g, MixedView src, const int *__restrict__ np2, const int *__restrict__ cumcnt, int pitch,
                             double *__restrict__ stage)
{
    const int row = blockIdx.y;
    const int jr = row % g.ny;
    const int n = np2[row];
    const int *cc = cumcnt + (long long)(g.nx + 1) * row;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < pitch; s += gridDim.x * blockDim.x) {
        double *a = stage + 6 * ((long long)row * pitch + s);
        if (s < n) {
            int lo = 0, hi = g.nx - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (cc[mid] <= s) lo = mid;
                else hi = mid - 1;
            }
            const long long p = src.idx(row, s);
            a[0] = (double)(g.nxgs + lo) + (double)src.X(p);
            a[1] = (double)(g.nys + jr) + (double)src.Y(p);
            a[2] = src.UX(p);
            a[3] = src.UY(p);
            a[4] = src.UZ(p);
            a[5] = __longlong_as_double(src.getpid(p));
        } else {
            for (int k = 0; k < 6; ++k) a[k] = 0.0;
        }
    }
}

}  // namespace

int wm_mixed_ntiles(const WmGeom &g) { return (g.nx + MX_TW - 1) / MX_TW; }
size_t wm_mixed_jtile_floats(const WmGeom &g) { return (size_t)g.nsp * g.ny * wm_mixed_ntiles(g) * 3 * 5 * MX_JW; }

int wm_launch_mixed_push_deposit(const WmGeom &g, const WmConst &k, MixedView a, MixedView b, FView<6, false> uf,
                                 const int *cumcnt, const WmRebinScratch &sc, float *jtile, cudaStream_t st)
{
    MxConst kc;
    for (int s = 0; s < WM_MAX_SP; ++s) {
        const double qm = k.q[s] / k.r[s];
        kc.fac1[s] = (float)(qm * 0.5 * k.delt);
        kc.txxx[s] = kc.fac1[s] * kc.fac1[s];
        kc.fac2[s] = (float)(k.q[s] * k.delt / k.r[s]);
        kc.mqdd[s] = (float)(-(k.q[s] * k.delx / k.delt));
        kc.q[s] = (float)k.q[s];
    }
    kc.dt_dx = (float)(k.delt / k.delx);
    kc.inv_c2 = (float)(1.0 / (k.c * k.c));
    kc.c2 = (float)(k.c * k.c);
    WM_CUDA(cudaMemsetAsync(sc.cellcnt, 0, sizeof(int) * (size_t)g.nrows * g.nx, st));
    dim3 grid(wm_mixed_ntiles(g), g.ny, g.nsp);
    k_mixed_push_deposit<<<grid, MX_THREADS, 0, st>>>(g, kc, a, b, uf, cumcnt, sc.key, sc.dir, sc.cellcnt, jtile, sc.status);
    return wm_check_launch("k_mixed_push_deposit");
}

int wm_launch_mixed_jfold(const WmGeom &g, const float *jtile, FView<3, false> uj, cudaStream_t st)
{
    const long long n = (long long)g.nxw * g.nyw;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_mixed_jfold<<<blocks, 256, 0, st>>>(g, wm_mixed_ntiles(g), jtile, uj);
    return wm_check_launch("k_mixed_jfold");
}

int wm_launch_mixed_unpack(const WmGeom &g, const double *stage, int pitch, const int *np2, MixedView dst, const WmRebinScratch &sc,
                           cudaStream_t st)
{
    WM_CUDA(cudaMemsetAsync(sc.cellcnt, 0, sizeof(int) * (size_t)g.nrows * g.nx, st));
    dim3 grid(std::min(wm_div_up(std::max(pitch, 1), 256), 64u), g.nrows);
    k_mixed_unpack<<<grid, 256, 0, st>>>(g, stage, pitch, np2, dst, sc.key, sc.cellcnt, sc.status);
    return wm_check_launch("k_mixed_unpack");
}

int wm_launch_mixed_pack(const WmGeom &g, MixedView src, const int *np2, const int *cumcnt, int pitch, double *stage, cudaStream_t st)
{
    dim3 grid(std::min(wm_div_up(std::max(pitch, 1), 256), 64u), g.nrows);
    k_mixed_pack<<<grid, 256, 0, st>>>(g, src, np2, cumcnt, pitch, stage);
    return wm_check_launch("k_mixed_pack");
}
