// wm_rebin.cu -- periodic particle boundaries and the per-cell counting sort on sm_103a.
//
// The reference moves particles between rows in boundary_periodic__particle_y
// (common/boundary_periodic.f90:99-248) and then counting-sorts every row by cell, stably, in
// sort__bucket (common/sort.f90:36-82).  Both define an exact permutation that these kernels
// reproduce bit for bit without running the sequential hole-filling loop.
//
// particle_y in closed form.  For a row with N particles, leaver slots h_1 < ... < h_m (holes)
// and an incoming list B of length kin (order: scan entries from lower rows first, then the
// two self-exchanges of the single-rank MPI_SENDRECV pair, :173-189):
//   * incoming number t <= m fills hole h_t, t > m is appended at slot N + t - m;
//   * if kin < m the row shrinks to N' = N + kin - m: the still-valid particles in slots
//     (N', N] (never incoming ones) move, highest slot first, into the remaining holes
//     h_{kin+1}, h_{kin+2}, ... in ascending order; for a stayer at slot s > N' that is hole
//     h_{kin+r} with r = (N - s) - (m - L(s)) + 1, L(s) = number of leavers at slots <= s;
//   * every other stayer keeps its slot.
// This is the loop at :193-225 unrolled; tests compare it with the sequential oracle.
//
// Sort.  With P = the slot after particle_y, sort__bucket orders particles by (cell, P) within
// each row.  k_count builds per-cell counts with warp-aggregated atomics, k_scan_cells turns
// them into the reference's cumcnt, k_scatter_pairs drops (P, particle) pairs into their cell's
// range in arbitrary order and k_cellsort_gather ranks each cell's pairs by P (one warp per cell)
// and moves the particles to their final slots.
#include <algorithm>

#include "wm_launch.cuh"

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------------------ walls in x
// Reflecting walls, boundary_reconnection.f90:61-99 (= boundary_shock.f90:62-100): a particle in
// cell ipos < nxs+1 is mirrored about x = nxs+1, one in ipos >= nxe-1 about nxe-1, its momentum
// reversed.  inject != 0: boundary_shock.f90:255-297 instead -- the same left wall, and beyond
// xend = nxe*delx + u0/sqrt(1+u0^2/c^2)*delt the particle is mirrored into the inflow
// (u_x -> 2 u0 - u_x).  `2.*(nxs+1)` is a default-real (FP32) product, exact here.
template <class PV>
__device__ __forceinline__ void walls_x_one(const PV &v, long long p, double delx, double xl, double xr, double xend, int nxs, int nxe,
                                            int inject, double u0)
{
    const double x = v.X(p);
    const int ipos = (int)(x / delx);
    if (ipos < nxs + 1) {
        v.X(p) = xl - x;
        v.UX(p) = -v.UX(p);
        v.UY(p) = -v.UY(p);
        v.UZ(p) = -v.UZ(p);
    } else if (!inject && ipos >= nxe - 1) {
        v.X(p) = xr - x;
        v.UX(p) = -v.UX(p);
        v.UY(p) = -v.UY(p);
        v.UZ(p) = -v.UZ(p);
    } else if (inject && x > xend) {
        v.X(p) = 2.0 * xend - x;
        v.UX(p) = 2.0 * u0 - v.UX(p);
        v.UY(p) = -v.UY(p);
        v.UZ(p) = -v.UZ(p);
    }
}

struct WallsX {
    double delx, xl, xr, xend, u0;
    int nxs, nxe, inject;
};

WallsX walls_x_params(const WmGeom &g, double delx, double delt, double c, int inject, double u0)
{
    WallsX w;
    w.delx = delx;
    w.nxs = g.nxgs;
    w.nxe = g.nxgs + g.nxa - 1;  // the active nxe (nxge but while the shock's box expands)
    w.xl = (double)(2.0f * (float)(w.nxs + 1)) * delx;
    w.xr = (double)(2.0f * (float)(w.nxe - 1)) * delx;
    w.xend = w.nxe * delx + u0 / sqrt(1 + (u0 * u0) / (c * c)) * delt;
    w.u0 = u0;
    w.inject = inject;
    return w;
}

template <class PV>
__global__ void k_walls_x(WmGeom g, WallsX w, PV v, const int *__restrict__ np2)
{
    const int row = blockIdx.y;
    const int n = np2[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        walls_x_one(v, v.idx(row, s), w.delx, w.xl, w.xr, w.xend, w.nxs, w.nxe, w.inject, w.u0);
}

// ------------------------------------------------------- wrap + classify + key
// mode bits: 1 = particle_x wrap, 2 = particle_y wrap + dir, 4 = sort key + cell count
// (key from the wrapped row), 8 = sort key from the current row (sort__bucket alone),
// 16 = particle_x of the walls (reflect at nxs+1 and nxe-1) instead of the wrap.
template <class PV>
__global__ void k_wrap_classify(WmGeom g, double delx, PV v, const int *__restrict__ np2, int mode,
                                unsigned char *__restrict__ dir, int *__restrict__ key, int *__restrict__ cellcnt,
                                unsigned *status)
{
    const int row = blockIdx.y;
    const int isp = row / g.ny, jr = row % g.ny;
    const int j = g.nys + jr;
    const int n = np2[row];
    const int lane = threadIdx.x & 31;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const double xlen = __dmul_rd((double)(g.nxge - g.nxgs + 1), delx);
    const double ylen = __dmul_rd((double)(g.nyge - g.nygs + 1), delx);
    // x / 1.0 is exact in every rounding mode, so with unit cells the FP64 division (a long
    // software sequence on this GPU) is skipped without changing any result.
    const bool unit = (delx == 1.0);
    unsigned bad = 0;
    for (int sb = warp_global * 32; sb < n; sb += nwarps * 32) {
        const int s = sb + lane;
        const bool valid = s < n;
        int k = -1;
        if (valid) {
            const long long p = v.idx(row, s);
            if (mode & 16) {
                const double xl = (double)(2.0f * (float)(g.nxgs + 1)) * delx, xr = (double)(2.0f * (float)(g.nxge - 1)) * delx;
                walls_x_one(v, p, delx, xl, xr, 0.0, g.nxgs, g.nxge, 0, 0.0);
            }
            double x = v.X(p);
            if (mode & 1) {  // boundary_periodic.f90:82-88, rounding mode downward
                const int ipos = unit ? (int)x : (int)__ddiv_rd(x, delx);
                if (ipos < g.nxgs) {
                    x = __dadd_rd(x, xlen);
                    v.X(p) = x;
                } else if (ipos >= g.nxge + 1) {
                    x = __dsub_rd(x, xlen);
                    v.X(p) = x;
                }
            }
            int kr = jr;
            if (mode & 2) {  // boundary_periodic.f90:147-165
                const double y = v.Y(p);
                const int jpos = unit ? (int)y : (int)__ddiv_rd(y, delx);
                unsigned char d = 0;
                if (jpos != j) {
                    if (jpos <= g.nygs - 1) v.Y(p) = __dadd_rd(y, ylen);
                    else if (jpos >= g.nyge + 1) v.Y(p) = __dsub_rd(y, ylen);
                    if (jpos == j + 1) {
                        d = 1;
                        kr = (jr == g.ny - 1) ? 0 : jr + 1;
                    } else if (jpos == j - 1) {
                        d = 2;
                        kr = (jr == 0) ? g.ny - 1 : jr - 1;
                    } else {
                        bad |= WMDEV_ROWJUMP;
                        d = 0;
                    }
                }
                dir[p] = d;
            }
            if (mode & 12) {  // sort.f90:60,72: i = int(x), no division by delx
                const int ci = (int)x - g.nxgs;
                if (ci < 0 || ci >= g.nx) {
                    bad |= WMDEV_CELL;
                    k = -1;
                } else {
                    k = (isp * g.ny + kr) * g.nx + ci;
                }
                key[p] = k;
            }
        }
        if (mode & 12) {
            const unsigned m = __ballot_sync(FULL, valid && k >= 0);
            if (valid && k >= 0) {
                const unsigned peers = __match_any_sync(m, k);
                if ((peers & lanemask_lt()) == 0) atomicAdd(&cellcnt[k], __popc(peers));
            }
        }
    }
    if (bad) atomicOr(status, bad);
}

// -------------------------------------------------------------------- rowscan
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_PER = 4;

// Exclusive block scan of a 64-bit value; returns the exclusive prefix, *total = block total.
__device__ __forceinline__ unsigned long long block_exscan_u64(unsigned long long v, unsigned long long *total)
{
    __shared__ unsigned long long wsum[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        unsigned long long s = (lane < SCAN_THREADS / 32) ? wsum[lane] : 0ull;
        unsigned long long si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(FULL, si, o);
            if (lane >= o) si += t;
        }
        if (lane < SCAN_THREADS / 32) wsum[lane] = si - s;  // exclusive warp offsets
        const unsigned long long tot = __shfl_sync(FULL, si, SCAN_THREADS / 32 - 1);
        if (lane == 0) *total = tot;
    }
    __syncthreads();
    const unsigned long long res = wsum[w] + inc - v;
    __syncthreads();
    return res;
}

// One CTA per row: leaver prefix counts, per-direction ordinals, the hole list and row totals.
// ord = up ordinal (dir 1), down ordinal (dir 2), L(s) = leavers before the slot (dir 0).
template <class PV>
__global__ void __launch_bounds__(SCAN_THREADS) k_rowscan(WmGeom g, PV v, const int *__restrict__ np2,
                                                          const unsigned char *__restrict__ dir, int *__restrict__ ord,
                                                          int *__restrict__ holes, int *__restrict__ nup,
                                                          int *__restrict__ ndown)
{
    __shared__ unsigned long long carry_s, total_s;
    const int row = blockIdx.x;
    const int n = np2[row];
    if (threadIdx.x == 0) carry_s = 0ull;
    __syncthreads();
    for (int cb = 0; cb < n; cb += SCAN_THREADS * SCAN_PER) {
        const int s0 = cb + threadIdx.x * SCAN_PER;
        unsigned char d[SCAN_PER];
        unsigned nu = 0, nd = 0;
#pragma unroll
        for (int e = 0; e < SCAN_PER; ++e) {
            const int s = s0 + e;
            d[e] = (s < n) ? dir[v.idx(row, s)] : (unsigned char)0;
            nu += (d[e] == 1);
            nd += (d[e] == 2);
        }
        const unsigned long long mine = ((unsigned long long)nu << 32) | nd;
        const unsigned long long ex = block_exscan_u64(mine, &total_s) + carry_s;
        unsigned cu = (unsigned)(ex >> 32), cd = (unsigned)(ex & 0xffffffffu);
#pragma unroll
        for (int e = 0; e < SCAN_PER; ++e) {
            const int s = s0 + e;
            if (s < n) {
                const long long p = v.idx(row, s);
                if (d[e] == 0) {
                    ord[p] = (int)(cu + cd);
                } else {
                    holes[v.idx(row, (int)(cu + cd))] = s + 1;
                    if (d[e] == 1) {
                        ord[p] = (int)cu;
                        ++cu;
                    } else {
                        ord[p] = (int)cd;
                        ++cd;
                    }
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) carry_s += total_s;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        nup[row] = (int)(carry_s >> 32);
        ndown[row] = (int)(carry_s & 0xffffffffu);
    }
}

// Incoming count of row kr (0-based within the species block starting at base).
__device__ __forceinline__ int incoming(const int *nup, const int *ndown, int base, int kr, int ny)
{
    int kin = 0;
    if (kr > 0) kin += nup[base + kr - 1];
    if (kr < ny - 1) kin += ndown[base + kr + 1];
    if (kr == ny - 1) kin += ndown[base + 0];
    if (kr == 0) kin += nup[base + ny - 1];
    return kin;
}

// Slot after particle_y (1-based, Pv) and destination row (kr, 0-based in the species block) of
// the particle at slot s of row (isp, jr).
template <class PV>
__device__ __forceinline__ void place_one(const WmGeom &g, const PV &v, int row, int jr, int base, int s, unsigned char d, int o,
                                          const int *__restrict__ np2, const int *__restrict__ holes,
                                          const int *__restrict__ nup, const int *__restrict__ ndown, int &kr, int &Pv)
{
    if (d == 0) {
        kr = jr;
        const int N = np2[row], m = nup[row] + ndown[row];
        const int kin = incoming(nup, ndown, base, kr, g.ny);
        Pv = s + 1;
        if (kin < m) {
            const int Np = N + kin - m;
            if (Pv > Np) {
                const int rr = (N - Pv) - (m - o) + 1;
                Pv = holes[v.idx(row, kin + rr - 1)];
            }
        }
    } else {
        int off;
        if (d == 1) {
            if (jr < g.ny - 1) {
                kr = jr + 1;
                off = 0;
            } else {
                kr = 0;
                off = (g.ny > 1) ? ndown[base + 1] : ndown[base + 0];
            }
        } else {
            if (jr > 0) {
                kr = jr - 1;
                off = (kr > 0) ? nup[base + kr - 1] : 0;
            } else {
                kr = g.ny - 1;
                off = (g.ny > 1) ? nup[base + g.ny - 2] : 0;
            }
        }
        const int krow = base + kr;
        const int t = off + o + 1;
        const int m = nup[krow] + ndown[krow];
        Pv = (t <= m) ? holes[v.idx(krow, t - 1)] : np2[krow] + t - m;
    }
}

// particle_y slot fused with the sort's scatter: with the new cumcnt already built from the
// destination cell counts, every particle drops its (P, index) pair into its destination cell's
// range right away (cursor atomics aggregated over the lanes that share a cell).
template <class PV>
__global__ void k_place_scatter(WmGeom g, PV v, PV dst, const int *__restrict__ np2, const unsigned char *__restrict__ dir,
                                const int *__restrict__ ord, const int *__restrict__ holes, const int *__restrict__ nup,
                                const int *__restrict__ ndown, const int *__restrict__ key, const int *__restrict__ cumcnt,
                                int *__restrict__ cursor, unsigned long long *__restrict__ pairs)
{
    const int row = blockIdx.y;
    const int jr = row % g.ny, base = (row / g.ny) * g.ny;
    const int n = np2[row];
    const int lane = threadIdx.x & 31;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int sb = warp_global * 32; sb < n; sb += nwarps * 32) {
        const int s = sb + lane;
        const bool valid = s < n;
        long long p = 0;
        int k = -1, Pv = 0;
        if (valid) {
            p = v.idx(row, s);
            int kr;
            place_one(g, v, row, jr, base, s, dir[p], ord[p], np2, holes, nup, ndown, kr, Pv);
            k = key[p];
        }
        const unsigned m = __ballot_sync(FULL, valid && k >= 0);
        if (valid && k >= 0) {
            const unsigned peers = __match_any_sync(m, k);
            const int leader = __ffs(peers) - 1;
            int basev = 0;
            if (lane == leader) basev = atomicAdd(&cursor[k], __popc(peers));
            basev = __shfl_sync(peers, basev, leader);
            const int slot = basev + __popc(peers & lanemask_lt());
            const int krow = k / g.nx, ci = k - krow * g.nx;
            const int cstart = cumcnt[(long long)krow * (g.nx + 1) + ci];
            pairs[dst.idx(krow, cstart + slot)] = ((unsigned long long)(unsigned)Pv << 32) | (unsigned long long)(unsigned)p;
        }
    }
}

// P (1-based slot after particle_y) of every particle.
template <class PV>
__global__ void k_place(WmGeom g, PV v, const int *__restrict__ np2, const unsigned char *__restrict__ dir,
                        const int *__restrict__ ord, const int *__restrict__ holes, const int *__restrict__ nup,
                        const int *__restrict__ ndown, int *__restrict__ P, int *__restrict__ drow)
{
    const int row = blockIdx.y;
    const int isp = row / g.ny, jr = row % g.ny, base = isp * g.ny;
    const int n = np2[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const long long p = v.idx(row, s);
        const unsigned char d = dir[p];
        const int o = ord[p];
        int kr, Pv;
        if (d == 0) {
            kr = jr;
            const int N = np2[row], m = nup[row] + ndown[row];
            const int kin = incoming(nup, ndown, base, kr, g.ny);
            Pv = s + 1;
            if (kin < m) {
                const int Np = N + kin - m;
                if (Pv > Np) {
                    const int rr = (N - Pv) - (m - o) + 1;
                    Pv = holes[v.idx(row, kin + rr - 1)];
                }
            }
        } else {
            int off;
            if (d == 1) {
                if (jr < g.ny - 1) {
                    kr = jr + 1;
                    off = 0;
                } else {
                    kr = 0;
                    off = (g.ny > 1) ? ndown[base + 1] : ndown[base + 0];
                }
            } else {
                if (jr > 0) {
                    kr = jr - 1;
                    off = (kr > 0) ? nup[base + kr - 1] : 0;
                } else {
                    kr = g.ny - 1;
                    off = (g.ny > 1) ? nup[base + g.ny - 2] : 0;
                }
            }
            const int krow = base + kr;
            const int t = off + o + 1;
            const int m = nup[krow] + ndown[krow];
            Pv = (t <= m) ? holes[v.idx(krow, t - 1)] : np2[krow] + t - m;
        }
        P[p] = Pv;
        if (drow) drow[p] = base + kr;
    }
}

// Row counts after particle_y (np2 += cnt, boundary_periodic.f90:228-235).
__global__ void k_np2_after_y(WmGeom g, const int *__restrict__ np2, const int *__restrict__ nup, const int *__restrict__ ndown,
                              int *__restrict__ np2_new, int np_limit, unsigned *status)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= g.nrows) return;
    const int isp = row / g.ny, kr = row % g.ny, base = isp * g.ny;
    const int v = np2[row] + incoming(nup, ndown, base, kr, g.ny) - (nup[row] + ndown[row]);
    np2_new[row] = v;
    if (np_limit > 0 && v > np_limit) atomicOr(status, (unsigned)WMDEV_OVERFLOW);
}

// particle_y alone: dst slot P-1 of the destination row gets the particle.
template <class PV>
__global__ void k_scatter_by_P(WmGeom g, PV src, PV dst, const int *__restrict__ np2, const int *__restrict__ P,
                               const int *__restrict__ drow, int np_limit, unsigned *status)
{
    const int row = blockIdx.y;
    const int n = np2[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const long long p = src.idx(row, s);
        const int Pv = P[p];
        if (np_limit > 0 && Pv > np_limit) {
            atomicOr(status, (unsigned)WMDEV_OVERFLOW);
            continue;
        }
        copy_particle(dst, dst.idx(drow[p], Pv - 1), src, p);
    }
}

// P = slot (sort__bucket alone)
template <class PV>
__global__ void k_slot_as_P(WmGeom g, PV v, const int *__restrict__ np2, int *__restrict__ P)
{
    const int row = blockIdx.y;
    const int n = np2[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) P[v.idx(row, s)] = s + 1;
}

// ---------------------------------------------------------------- cell scan
// One CTA per row: cumcnt(nxs..nxe+1) = exclusive prefix of cell counts, np2 = total; the
// counts are reset to zero for reuse as scatter cursors.
constexpr int CSCAN_THREADS = 512;
__global__ void __launch_bounds__(CSCAN_THREADS) k_scan_cells(WmGeom g, int *__restrict__ cellcnt, int *__restrict__ cumcnt,
                                                              int *__restrict__ np2_out)
{
    __shared__ int wsum[CSCAN_THREADS / 32];
    __shared__ int carry;
    const int row = blockIdx.x;
    int *cnt = cellcnt + (long long)row * g.nx;
    int *cc = cumcnt + (long long)row * (g.nx + 1);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int cb = 0; cb < g.nx; cb += CSCAN_THREADS) {
        const int c = cb + threadIdx.x;
        const int v = (c < g.nx) ? cnt[c] : 0;
        int inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        if (w == 0) {
            const int s = (lane < CSCAN_THREADS / 32) ? wsum[lane] : 0;
            int si = s;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(FULL, si, o);
                if (lane >= o) si += t;
            }
            if (lane < CSCAN_THREADS / 32) wsum[lane] = si - s;
        }
        __syncthreads();
        const int ex = carry + wsum[w] + inc - v;
        if (c < g.nx) {
            cc[c] = ex;
            cnt[c] = 0;
        }
        __syncthreads();
        if (threadIdx.x == CSCAN_THREADS - 1) carry = ex + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        cc[g.nx] = carry;
        np2_out[row] = carry;
    }
}

// rowbase[r] = sum of np2[0..r), one CTA.
__global__ void k_rowbase(int nrows, const int *__restrict__ np2, long long *__restrict__ rowbase)
{
    __shared__ long long wsum[32];
    __shared__ long long carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int cb = 0; cb < nrows; cb += blockDim.x) {
        const int r = cb + threadIdx.x;
        const long long v = (r < nrows) ? np2[r] : 0;
        long long inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        if (w == 0) {
            const long long s = (lane < nw) ? wsum[lane] : 0;
            long long si = s;
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(FULL, si, o);
                if (lane >= o) si += t;
            }
            if (lane < nw) wsum[lane] = si - s;
        }
        __syncthreads();
        const long long ex = carry + wsum[w] + inc - v;
        if (r < nrows) rowbase[r] = ex;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = ex + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) rowbase[nrows] = carry;
}

// ---------------------------------------------------------- scatter pairs
// pairs[dst.idx(row, cumcnt(cell) + cursor)] = (P << 32) | src particle index
template <class PV>
__global__ void k_scatter_pairs(WmGeom g, PV src, PV dst, const int *__restrict__ np2, const int *__restrict__ key,
                                const int *__restrict__ P, const int *__restrict__ cumcnt, int *__restrict__ cursor,
                                unsigned long long *__restrict__ pairs)
{
    const int row = blockIdx.y;
    const int n = np2[row];
    const int lane = threadIdx.x & 31;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int sb = warp_global * 32; sb < n; sb += nwarps * 32) {
        const int s = sb + lane;
        const bool valid = s < n;
        long long p = 0;
        int k = -1;
        if (valid) {
            p = src.idx(row, s);
            k = key[p];
        }
        const unsigned m = __ballot_sync(FULL, valid && k >= 0);
        if (valid && k >= 0) {
            const unsigned peers = __match_any_sync(m, k);
            const int leader = __ffs(peers) - 1;
            int basev = 0;
            if (lane == leader) basev = atomicAdd(&cursor[k], __popc(peers));
            basev = __shfl_sync(peers, basev, leader);
            const int slot = basev + __popc(peers & lanemask_lt());
            const int krow = k / g.nx, ci = k - krow * g.nx;
            const int cstart = cumcnt[(long long)krow * (g.nx + 1) + ci];
            pairs[dst.idx(krow, cstart + slot)] = ((unsigned long long)(unsigned)P[p] << 32) | (unsigned long long)(unsigned)p;
        }
    }
}

// ------------------------------------------------------ per-cell rank + move
constexpr int CS_WARPS = 8;
constexpr int CS_SMEM = 256;  // pairs per warp held in shared memory

template <class PV>
__global__ void __launch_bounds__(CS_WARPS * 32) k_cellsort_gather(WmGeom g, PV src, PV dst, const int *__restrict__ cumcnt,
                                                                   const unsigned long long *__restrict__ pairs)
{
    __shared__ unsigned sP[CS_WARPS][CS_SMEM];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long ncells = (long long)g.nrows * g.nx;
    for (long long cell = (long long)blockIdx.x * CS_WARPS + w; cell < ncells; cell += (long long)gridDim.x * CS_WARPS) {
        const int row = (int)(cell / g.nx), ci = (int)(cell - (long long)row * g.nx);
        const int *cc = cumcnt + (long long)row * (g.nx + 1);
        const int c0 = cc[ci], n = cc[ci + 1] - c0;
        if (n == 0) continue;
        const long long pb = dst.idx(row, c0);
        if (n <= CS_SMEM) {
            for (int e = lane; e < n; e += 32) sP[w][e] = (unsigned)(pairs[pb + e] >> 32);
            __syncwarp();
            for (int e = lane; e < n; e += 32) {
                const unsigned myP = sP[w][e];
                int rank = 0;
                for (int f = 0; f < n; ++f) rank += (sP[w][f] < myP);
                const long long ps = (long long)(unsigned)(pairs[pb + e] & 0xffffffffull);
                copy_particle(dst, dst.idx(row, c0 + rank), src, ps);
            }
            __syncwarp();
        } else {
            for (int e = lane; e < n; e += 32) {
                const unsigned long long pr = pairs[pb + e];
                const unsigned myP = (unsigned)(pr >> 32);
                int rank = 0;
                for (int f = 0; f < n; ++f) rank += ((unsigned)(pairs[pb + f] >> 32) < myP);
                copy_particle(dst, dst.idx(row, c0 + rank), src, (long long)(unsigned)(pr & 0xffffffffull));
            }
        }
    }
}

}  // namespace

// ======================================================================= host side
static dim3 row_grid(const WmGeom &g, int max_row_count, int threads, int cap_blocks = 64)
{
    const unsigned bx = std::max(1u, std::min(wm_div_up(std::max(max_row_count, 1), threads), (unsigned)cap_blocks));
    return dim3(bx, g.nrows);
}

template <class PV>
int wm_launch_wrap_classify(const WmGeom &g, double delx, PV v, const int *np2, int max_row_count, int mode,
                            const WmRebinScratch &sc, cudaStream_t st)
{
    if (mode & 12) WM_CUDA(cudaMemsetAsync(sc.cellcnt, 0, sizeof(int) * (size_t)g.nrows * g.nx, st));
    k_wrap_classify<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, delx, v, np2, mode, sc.dir, sc.key, sc.cellcnt,
                                                                         sc.status);
    return wm_check_launch("k_wrap_classify");
}

// particle_y ordinals and P; drow receives the destination row of every particle.
template <class PV>
int wm_launch_place(const WmGeom &g, PV v, const int *np2, int max_row_count, const WmRebinScratch &sc, int *drow,
                    cudaStream_t st)
{
    k_rowscan<PV><<<g.nrows, SCAN_THREADS, 0, st>>>(g, v, np2, sc.dir, sc.ord, sc.holes, sc.nup, sc.ndown);
    WM_TRY(wm_check_launch("k_rowscan"));
    k_place<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, v, np2, sc.dir, sc.ord, sc.holes, sc.nup, sc.ndown, sc.P,
                                                                 drow);
    return wm_check_launch("k_place");
}

// The fused step's rebin once the destination cumcnt and row bases exist: row prefix counts,
// particle_y slots with the pair scatter, then the per-cell ranking and gather src -> dst.
template <class PV>
int wm_launch_place_sort(const WmGeom &g, PV src, PV dst, const int *np2, int max_row_count, const int *cumcnt,
                         const WmRebinScratch &sc, cudaStream_t st)
{
    k_rowscan<PV><<<g.nrows, SCAN_THREADS, 0, st>>>(g, src, np2, sc.dir, sc.ord, sc.holes, sc.nup, sc.ndown);
    WM_TRY(wm_check_launch("k_rowscan"));
    k_place_scatter<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, src, dst, np2, sc.dir, sc.ord, sc.holes, sc.nup,
                                                                        sc.ndown, sc.key, cumcnt, sc.cellcnt, sc.pairs);
    WM_TRY(wm_check_launch("k_place_scatter"));
    const long long ncells = (long long)g.nrows * g.nx;
    const unsigned blocks = (unsigned)std::min<long long>((ncells + CS_WARPS - 1) / CS_WARPS, 152LL * 64);
    k_cellsort_gather<PV><<<blocks, CS_WARPS * 32, 0, st>>>(g, src, dst, cumcnt, sc.pairs);
    return wm_check_launch("k_cellsort_gather");
}

int wm_launch_np2_after_y(const WmGeom &g, const int *np2, const WmRebinScratch &sc, int *np2_new, int np_limit,
                          cudaStream_t st)
{
    k_np2_after_y<<<wm_div_up(g.nrows, 256), 256, 0, st>>>(g, np2, sc.nup, sc.ndown, np2_new, np_limit, sc.status);
    return wm_check_launch("k_np2_after_y");
}

template <class PV>
int wm_launch_scatter_by_P(const WmGeom &g, PV src, PV dst, const int *np2, int max_row_count, const WmRebinScratch &sc,
                           const int *drow, int np_limit, cudaStream_t st)
{
    k_scatter_by_P<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, src, dst, np2, sc.P, drow, np_limit, sc.status);
    return wm_check_launch("k_scatter_by_P");
}

template <class PV>
int wm_launch_slot_as_P(const WmGeom &g, PV v, const int *np2, int max_row_count, const WmRebinScratch &sc, cudaStream_t st)
{
    k_slot_as_P<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, v, np2, sc.P);
    return wm_check_launch("k_slot_as_P");
}

int wm_launch_scan_cells(const WmGeom &g, const WmRebinScratch &sc, int *cumcnt, int *np2_out, cudaStream_t st)
{
    k_scan_cells<<<g.nrows, CSCAN_THREADS, 0, st>>>(g, sc.cellcnt, cumcnt, np2_out);
    return wm_check_launch("k_scan_cells");
}

int wm_launch_rowbase(int nrows, const int *np2, long long *rowbase, cudaStream_t st)
{
    k_rowbase<<<1, 1024, 0, st>>>(nrows, np2, rowbase);
    return wm_check_launch("k_rowbase");
}

// src rows: src_np2 particles, keys in sc.key, P in sc.P; dst has cumcnt and its row bases.
template <class PV>
int wm_launch_sort_move(const WmGeom &g, PV src, PV dst, const int *src_np2, int max_row_count, const int *cumcnt,
                        const WmRebinScratch &sc, cudaStream_t st)
{
    k_scatter_pairs<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, src, dst, src_np2, sc.key, sc.P, cumcnt, sc.cellcnt,
                                                                         sc.pairs);
    WM_TRY(wm_check_launch("k_scatter_pairs"));
    const long long ncells = (long long)g.nrows * g.nx;
    const unsigned blocks = (unsigned)std::min<long long>((ncells + CS_WARPS - 1) / CS_WARPS, 152LL * 64);
    k_cellsort_gather<PV><<<blocks, CS_WARPS * 32, 0, st>>>(g, src, dst, cumcnt, sc.pairs);
    return wm_check_launch("k_cellsort_gather");
}

template <class PV>
int wm_launch_walls_x(const WmGeom &g, const WmConst &k, PV v, const int *np2, int max_row_count, int inject, double u0,
                      cudaStream_t st)
{
    const WallsX w = walls_x_params(g, k.delx, k.delt, k.c, inject, u0);
    k_walls_x<PV><<<row_grid(g, max_row_count, 256), 256, 0, st>>>(g, w, v, np2);
    return wm_check_launch("k_walls_x");
}

#define WM_INST(PV)                                                                                                   \
    template int wm_launch_walls_x<PV>(const WmGeom &, const WmConst &, PV, const int *, int, int, double, cudaStream_t); \
    template int wm_launch_wrap_classify<PV>(const WmGeom &, double, PV, const int *, int, int, const WmRebinScratch &, \
                                             cudaStream_t);                                                            \
    template int wm_launch_place<PV>(const WmGeom &, PV, const int *, int, const WmRebinScratch &, int *, cudaStream_t); \
    template int wm_launch_scatter_by_P<PV>(const WmGeom &, PV, PV, const int *, int, const WmRebinScratch &, const int *, \
                                            int, cudaStream_t);                                                        \
    template int wm_launch_slot_as_P<PV>(const WmGeom &, PV, const int *, int, const WmRebinScratch &, cudaStream_t);    \
    template int wm_launch_sort_move<PV>(const WmGeom &, PV, PV, const int *, int, const int *, const WmRebinScratch &,  \
                                         cudaStream_t);                                                                \
    template int wm_launch_place_sort<PV>(const WmGeom &, PV, PV, const int *, int, const int *, const WmRebinScratch &, \
                                          cudaStream_t);
WM_INST(SoAView)
WM_INST(AoSView)
WM_INST(MixedView)
#undef WM_INST
