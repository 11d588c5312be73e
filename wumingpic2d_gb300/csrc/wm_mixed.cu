// wm_mixed.cu -- the mixed-precision particle kernels (FP32 push and deposit) for sm_103a.
//
// Particles carry their position as (cell, FP32 offset in [0,1)) -- the cell is implicit in the
// cell-sorted rows -- and FP32 momenta.  k_mixed_push_deposit does, for one (species, row, 64-cell
// tile): the cell-centred fields of particle.f90:68-81 staged in shared memory as FP32, the
// Buneman-Boris push of particle.f90:96-161 in FP32, the Esirkepov deposit of field.f90:224-298 in
// FP32, the periodic wrap of boundary_periodic.f90:61-96 and :143-165 as integer cell arithmetic,
// and the destination cell key and row direction the rebin needs.  Particles are staged through
// shared memory in chunks so that global loads and stores are coalesced while each thread walks
// 8 consecutive particles; a thread adds its particles' 5x5x3 currents into registers while they
// stay in one cell and flushes them to the tile's FP32 current accumulator (shared-memory atomics)
// when the cell changes.  Tile currents go to a per-tile buffer; k_mixed_jfold adds them into the
// FP64 global J node by node in a fixed order, so the result is deterministic.
#include <algorithm>

#include "wm_launch.cuh"

namespace {

constexpr int MX_TW = 64;  // cells per tile
constexpr int MX_THREADS = 256;
constexpr int MX_PER = 8;  // consecutive particles per thread per chunk
constexpr int MX_CHUNK = MX_THREADS * MX_PER;
constexpr int MX_PAD = MX_PER + 1;  // padded stride: conflict-free shared-memory access
constexpr int MX_JW = MX_TW + 4;

struct MxConst {
    float fac1[WM_MAX_SP], txxx[WM_MAX_SP], fac2[WM_MAX_SP], mqdd[WM_MAX_SP], q[WM_MAX_SP];
    float dt_dx, inv_c2, c2;
};

struct MxSmem {
    float tmp[6][3][MX_TW + 2];
    float jacc[3][5][MX_JW];
    int cc[MX_TW + 1];
    float buf[5][MX_THREADS * MX_PAD];
    int keyb[MX_THREADS * MX_PAD];
    unsigned char dirb[MX_THREADS * MX_PAD];
};

__device__ __forceinline__ void shape3(float h, float &a0, float &a1, float &a2)
{
    a0 = 0.5f * (0.5f - h) * (0.5f - h);
    a1 = 0.75f - h * h;
    a2 = 0.5f * (0.5f + h) * (0.5f + h);
}

__global__ void __launch_bounds__(MX_THREADS, 2)
    k_mixed_push_deposit(WmGeom g, MxConst kc, MixedView a, MixedView b, FView<6, false> uf, const int *__restrict__ cumcnt,
                         int *__restrict__ key, unsigned char *__restrict__ dir, int *__restrict__ cellcnt,
                         float *__restrict__ jtile, unsigned *status)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MxSmem &S = *reinterpret_cast<MxSmem *>(smem_raw);
    const int tile = blockIdx.x, jr = blockIdx.y, isp = blockIdx.z;
    const int row = isp * g.ny + jr;
    const int c0 = tile * MX_TW;  // first interior cell of the tile
    const int ncell = min(MX_TW, g.nx - c0);
    const int tid = threadIdx.x;

    // fields at cell centres (i+1/2, j+1/2) for cells c0-1 .. c0+ncell and rows jr-1 .. jr+1
    const int tw = ncell + 2;
    for (int e = tid; e < 3 * tw; e += MX_THREADS) {
        const int aa = e % tw, bb = e / tw;
        const int ix = c0 - 1 + aa + 2, iy = jr - 1 + bb + 2;
        S.tmp[0][bb][aa] = (float)(0.5 * (uf(0, ix, iy) + uf(0, ix, iy + 1)));
        S.tmp[1][bb][aa] = (float)(0.5 * (uf(1, ix, iy) + uf(1, ix + 1, iy)));
        S.tmp[2][bb][aa] = (float)(0.25 * (uf(2, ix, iy) + uf(2, ix + 1, iy) + uf(2, ix, iy + 1) + uf(2, ix + 1, iy + 1)));
        S.tmp[3][bb][aa] = (float)(0.5 * (uf(3, ix, iy) + uf(3, ix + 1, iy)));
        S.tmp[4][bb][aa] = (float)(0.5 * (uf(4, ix, iy) + uf(4, ix, iy + 1)));
        S.tmp[5][bb][aa] = (float)uf(5, ix, iy);
    }
    for (int e = tid; e < 3 * 5 * MX_JW; e += MX_THREADS) (&S.jacc[0][0][0])[e] = 0.f;
    __shared__ float spc[5];  // this species' constants (static indices: no local-memory copy)
    if (tid == 0) {
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
    const int *ccrow = cumcnt + (long long)(g.nx + 1) * row;
    for (int e = tid; e <= ncell; e += MX_THREADS) S.cc[e] = ccrow[c0 + e];
    __syncthreads();

    const float fac1 = spc[0], txxx = spc[1], fac2 = spc[2], mqdd = spc[3], qs = spc[4];
    const int start = S.cc[0], end = S.cc[ncell];
    const long long rbase = a.rowbase[row];
    unsigned bad = 0;

    for (int cbeg = start; cbeg < end; cbeg += MX_CHUNK) {
        const int nchunk = min(MX_CHUNK, end - cbeg);
        // coalesced load into the padded per-thread layout
        for (int e = tid; e < nchunk; e += MX_THREADS) {
            const long long p = rbase + cbeg + e;
            const int sidx = (e / MX_PER) * MX_PAD + (e % MX_PER);
            S.buf[0][sidx] = a.x[p];
            S.buf[1][sidx] = a.y[p];
            S.buf[2][sidx] = a.ux[p];
            S.buf[3][sidx] = a.uy[p];
            S.buf[4][sidx] = a.uz[p];
        }
        __syncthreads();

        const int q0 = tid * MX_PER;
        int c = -1;  // cell (within the tile) of the current run
        float ax[5][4], ay[4][5], az[5][5];
        int run_key = -1, run_cnt = 0;
        for (int k = 0; k < MX_PER; ++k) {
            const int q = q0 + k;
            if (q >= nchunk) break;
            const int slot = cbeg + q;
            int cn = c;
            if (cn < 0) {  // first particle of the chunk: last cell whose start is <= slot
                int lo = 0, hi = ncell - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (S.cc[mid] <= slot) lo = mid;
                    else hi = mid - 1;
                }
                cn = lo;
            } else {
                while (cn + 1 < ncell && S.cc[cn + 1] <= slot) ++cn;
            }
            if (cn != c) {
                if (c >= 0) {  // flush the finished cell
#pragma unroll
                    for (int jp = 0; jp < 5; ++jp)
#pragma unroll
                        for (int ip = 0; ip < 5; ++ip) {
                            if (ip > 0) atomicAdd(&S.jacc[0][jp][c + ip], ax[jp][ip - 1]);
                            if (jp > 0) atomicAdd(&S.jacc[1][jp][c + ip], ay[jp - 1][ip]);
                            atomicAdd(&S.jacc[2][jp][c + ip], az[jp][ip]);
                        }
                }
                c = cn;
#pragma unroll
                for (int jp = 0; jp < 5; ++jp)
#pragma unroll
                    for (int ip = 0; ip < 5; ++ip) {
                        if (ip < 4) ax[jp][ip] = 0.f;
                        if (jp < 4) ay[jp][ip] = 0.f;
                        az[jp][ip] = 0.f;
                    }
            }
            const int sidx = tid * MX_PAD + k;
            const float dx = S.buf[0][sidx], dy = S.buf[1][sidx];
            float u1 = S.buf[2][sidx], u2 = S.buf[3][sidx], u3 = S.buf[4][sidx];
            // gather (TSC weights about the cell centre)
            float sx0, sx1, sx2, sy0, sy1, sy2;
            shape3(dx - 0.5f, sx0, sx1, sx2);
            shape3(dy - 0.5f, sy0, sy1, sy2);
            float f[6];
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                const float *t0 = &S.tmp[m][0][c], *t1 = &S.tmp[m][1][c], *t2 = &S.tmp[m][2][c];
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
            float s0x[5], s0y[5], dsx[5], dsy[5];
            s0x[0] = 0.f;
            s0x[4] = 0.f;
            s0y[0] = 0.f;
            s0y[4] = 0.f;
            s0x[1] = sx0;
            s0x[2] = sx1;
            s0x[3] = sx2;
            s0y[1] = sy0;
            s0y[2] = sy1;
            s0y[3] = sy2;
            {
                float b0, b1, b2;
                shape3(nx1 - 0.5f, b0, b1, b2);
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const int o = m - 2 - incx;
                    const float s1 = (o == -1) ? b0 : (o == 0) ? b1 : (o == 1) ? b2 : 0.f;
                    dsx[m] = s1 - s0x[m];
                }
                shape3(ny1 - 0.5f, b0, b1, b2);
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const int o = m - 2 - incy;
                    const float s1 = (o == -1) ? b0 : (o == 0) ? b1 : (o == 1) ? b2 : 0.f;
                    dsy[m] = s1 - s0y[m];
                }
            }
            const float qg = qs * u3 * ig;
            float wy[5], wx[5], z2[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                wy[m] = s0y[m] + 0.5f * dsy[m];
                wx[m] = s0x[m] + 0.5f * dsx[m];
                z2[m] = qg * (0.5f * s0y[m] + (1.f / 3.f) * dsy[m]);
            }
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
                const float fy = mqdd * wy[jp];
#pragma unroll
                for (int m = 0; m < 4; ++m) ax[jp][m] = fmaf(fy, cx[m], ax[jp][m]);
            }
#pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                const float fx = mqdd * wx[ip];
#pragma unroll
                for (int m = 0; m < 4; ++m) ay[m][ip] = fmaf(fx, cy[m], ay[m][ip]);
            }
#pragma unroll
            for (int jp = 0; jp < 5; ++jp) {
                const float z1 = qg * wy[jp];
#pragma unroll
                for (int ip = 0; ip < 5; ++ip) az[jp][ip] = fmaf(s0x[ip], z1, fmaf(dsx[ip], z2[jp], az[jp][ip]));
            }
            // new state, destination cell (periodic wrap as integer arithmetic) and row direction
            S.buf[0][sidx] = nx1;
            S.buf[1][sidx] = ny1;
            S.buf[2][sidx] = u1;
            S.buf[3][sidx] = u2;
            S.buf[4][sidx] = u3;
            int ci = c0 + c + incx;
            ci = ci < 0 ? ci + g.nx : (ci >= g.nx ? ci - g.nx : ci);
            int kr = jr + incy;
            kr = kr < 0 ? kr + g.ny : (kr >= g.ny ? kr - g.ny : kr);
            const int kk = (isp * g.ny + kr) * g.nx + ci;
            S.keyb[sidx] = kk;
            S.dirb[sidx] = (unsigned char)(incy == 1 ? 1 : (incy == -1 ? 2 : 0));
            if (kk != run_key) {
                if (run_cnt) atomicAdd(&cellcnt[run_key], run_cnt);
                run_key = kk;
                run_cnt = 0;
            }
            ++run_cnt;
        }
        if (run_cnt) atomicAdd(&cellcnt[run_key], run_cnt);
        if (c >= 0) {
#pragma unroll
            for (int jp = 0; jp < 5; ++jp)
#pragma unroll
                for (int ip = 0; ip < 5; ++ip) {
                    if (ip > 0) atomicAdd(&S.jacc[0][jp][c + ip], ax[jp][ip - 1]);
                    if (jp > 0) atomicAdd(&S.jacc[1][jp][c + ip], ay[jp - 1][ip]);
                    atomicAdd(&S.jacc[2][jp][c + ip], az[jp][ip]);
                }
        }
        __syncthreads();
        for (int e = tid; e < nchunk; e += MX_THREADS) {
            const long long p = rbase + cbeg + e;
            const int sidx = (e / MX_PER) * MX_PAD + (e % MX_PER);
            b.x[p] = S.buf[0][sidx];
            b.y[p] = S.buf[1][sidx];
            b.ux[p] = S.buf[2][sidx];
            b.uy[p] = S.buf[3][sidx];
            b.uz[p] = S.buf[4][sidx];
            key[p] = S.keyb[sidx];
            dir[p] = S.dirb[sidx];
        }
        __syncthreads();
    }
    if (bad) atomicOr(status, (unsigned)WMDEV_CELL);
    // tile currents -> per-tile buffer [isp][jr][tile][3][5][MX_JW]
    const int ntiles = gridDim.x;
    float *out = jtile + ((((long long)isp * g.ny + jr) * ntiles + tile) * 3) * 5 * MX_JW;
    for (int e = tid; e < 3 * 5 * MX_JW; e += MX_THREADS) out[e] = (&S.jacc[0][0][0])[e];
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
    static bool attr_set = false;
    const size_t smem = sizeof(MxSmem);
    if (!attr_set) {
        WM_CUDA(cudaFuncSetAttribute(k_mixed_push_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
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
    k_mixed_push_deposit<<<grid, MX_THREADS, smem, st>>>(g, kc, a, b, uf, cumcnt, sc.key, sc.dir, sc.cellcnt, jtile, sc.status);
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
