// wm_mixed.cu -- the mixed-precision particle kernels (FP32 push and deposit) for sm_103a.
//
// Particles carry their position as (cell, FP32 offset in [0,1)) -- the cell is implicit in the
// cell-sorted rows -- and FP32 momenta.  k_mixed_fields turns the FP64 Yee fields into the
// cell-centred fields of particle.f90:68-81 once per step, as FP32.  k_mixed_push_deposit then
// does, for one (species, row, 32-cell tile): the Buneman-Boris push of particle.f90:96-161 in
// FP32, the Esirkepov deposit of field.f90:224-298 in FP32, the periodic wrap of
// boundary_periodic.f90:61-96 and :143-165 as integer cell arithmetic, and the destination cell key
// and row direction the rebin needs.  The tile's cell-centred fields arrive as one TMA box; four
// lanes share a cell, so the cell's (dx, dy, ux, uy) records move as two full 32-byte sectors per
// particle round; each step of the loop pushes two particles per lane (the cell's field
// coefficients read once for both) while the lane's next two (the 16-byte record and uz) are
// copied into shared memory (cp.async).  The TSC-weighted 3x3 gather of
// each field is a biquadratic in the particle's offsets, so the kernel stages its nine
// coefficients per cell and field and evaluates it by Horner's rule, two fields per packed
// fma.rn.f32x2.  Each lane keeps the cell's 5x5x3 partial currents in registers (the cell's
// particles all deposit on the same 5x5 nodes); the cell's lanes add theirs with shuffles, and the
// tile's node currents are summed from the per-cell partials in a fixed order.  Tile currents go
// to a per-tile buffer; k_mixed_jfold adds them into the FP64 global J node by node in a fixed
// order, so the result is deterministic and no atomics touch the currents.  The rebin either
// records the new cell order as a slot permutation that the next push reads through
// (k_mixed_perm; the push then writes its particles out in cell order) or moves the particles into
// it (k_mixed_move); both give the same state.
#include <algorithm>

#include "wm_launch.cuh"

namespace {

#ifndef WM_MX_THREADS
#define WM_MX_THREADS 128  // threads per push CTA (a build-time choice, 128 or 256; 128 measured 2.6 % faster)
#endif
constexpr int MX_THREADS = WM_MX_THREADS;
#ifndef WM_MX_LPC
#define WM_MX_LPC 4  // lanes per cell (4: the cell's four 16-byte records fill two sectors per step; 8 measured 14 % slower)
#endif
constexpr int MX_LPC = WM_MX_LPC;           // lanes per cell
constexpr int MX_TW = MX_THREADS / MX_LPC;  // cells per tile (one row, one species)
constexpr int MX_JW = MX_TW + 4;            // node columns a tile deposits on
constexpr int MX_FS = 60;                   // floats per cell of staged stencil: 9 x 6 used; 60 keeps 128-bit reads conflict-free
constexpr int MX_PW = MX_TW + 8;            // per-cell partial rows: 4 zero cells on each side
constexpr int MX_FTW = MX_TW + 4;           // columns of the staged field tile: the 34 a tile uses, rounded to 16 bytes
constexpr int MX_CB = 6;                    // bits of the tile cell in a move code: rank << 10 | cell << 4 | direction
static_assert(MX_TW <= (1 << MX_CB), "a tile's cells fit the move code");
constexpr unsigned FULL = 0xffffffffu;
#ifndef WM_MX_XQ
#define WM_MX_XQ 16
#endif
constexpr int MX_XQ = WM_MX_XQ;  // per-cell queue of particles that changed cell, deposited after the loop

struct MxConst {
    float fac1[WM_MAX_SP], txxx[WM_MAX_SP], fac2[WM_MAX_SP], mqdd[WM_MAX_SP], q[WM_MAX_SP];
    float dt_dx, inv_c2, c2;
    // walls in x (WM_BC_RECONNECTION, WM_BC_SHOCK); the shock's injection boundary
    // xend - nxgs*delx = xe_cell + xe_off (in cells) and its four-velocity u0
    int bc, xe_cell;
    float xe_off, u0;
};

// A particle at interior cell cn + offset off (cell units) mirrored about the wall at interior
// position w: cn' + off' = 2w - (cn + off).
__device__ __forceinline__ void mirror(int w2, int &cn, float &off)
{
    if (off == 0.f) {
        cn = w2 - cn;
    } else {
        cn = w2 - cn - 1;
        off = 1.f - off;
    }
}

// The TSC weights at centred offset h: 0.5 (0.5 + h)^2 = h (h/2 + 1/2) + 1/8 and
// 0.5 (0.5 - h)^2 = that - h, 3/4 - h^2: four instructions.
__device__ __forceinline__ void shape3(float h, float &a0, float &a1, float &a2)
{
    a2 = fmaf(h, fmaf(0.5f, h, 0.5f), 0.125f);
    a0 = a2 - h;
    a1 = fmaf(-h, h, 0.75f);
}

// Two FP32 values in one 64-bit register pair, and the packed FMA of sm_100+ on such pairs.
__device__ __forceinline__ unsigned long long pack2(float lo, float hi)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(unsigned long long r, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Asynchronous copy of one float into shared memory; nbytes = 0 writes a zero and reads nothing.
__device__ __forceinline__ void cp_async4(float *dst, const float *src, unsigned nbytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src), "r"(nbytes)
                 : "memory");
}
// The same for one 16-byte record (both addresses 16-byte aligned; nbytes 0 or 16).
__device__ __forceinline__ void cp_async16(float4 *dst, const float4 *src, unsigned nbytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src), "r"(nbytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// The pushed particle (one 16-byte record, uz) and its move code, stored only by lanes that
// hold a particle (one predicate for the three stores: the loop body has no branches).
__device__ __forceinline__ void store_particle(const MixedView &b, long long p, float x, float y, float ux, float uy, float uz,
                                               unsigned *code, unsigned cv, bool pred)
{
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %0, 0;\n\t"
                 "@q st.global.v4.f32 [%1], {%2, %3, %4, %5};\n\t@q st.global.f32 [%6], %7;\n\t@q st.global.u32 [%8], %9;\n\t}"
                 ::"r"((unsigned)pred), "l"(b.xyuv + p), "f"(x), "f"(y), "f"(ux), "f"(uy), "l"(b.uz + p), "f"(uz), "l"(code + p), "r"(cv)
                 : "memory");
}

// Cell-centred fields (i+1/2, j+1/2) of particle.f90:68-81 for cells -1..nx and rows -1..ny,
// averaged in FP64 and rounded once to FP32: fcc[m][(jy+1)*pitch + ix+1], the row pitch a
// multiple of 4 floats (16 bytes, for the push's TMA loads); the pad columns are never read.
__global__ void k_mixed_fields(WmGeom g, FView<6, false> uf, float *__restrict__ fcc, int pitch)
{
    const int W = g.nx + 2;
    const long long n = (long long)W * (g.ny + 2), plane = (long long)pitch * (g.ny + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(e % W) + 1, iy = (int)(e / W) + 1;  // ghosted index of cell ix-2, row iy-2
        const long long o = (long long)(iy - 1) * pitch + ix - 1;
        fcc[o] = (float)(0.5 * (uf(0, ix, iy) + uf(0, ix, iy + 1)));
        fcc[plane + o] = (float)(0.5 * (uf(1, ix, iy) + uf(1, ix + 1, iy)));
        fcc[2 * plane + o] = (float)(0.25 * (uf(2, ix, iy) + uf(2, ix + 1, iy) + uf(2, ix, iy + 1) + uf(2, ix + 1, iy + 1)));
        fcc[3 * plane + o] = (float)(0.5 * (uf(3, ix, iy) + uf(3, ix + 1, iy)));
        fcc[4 * plane + o] = (float)(0.5 * (uf(4, ix, iy) + uf(4, ix, iy + 1)));
        fcc[5 * plane + o] = (float)uf(5, ix, iy);
    }
}

// bounded mbarrier wait (parity), as the TMA load of the push's field tile needs
__device__ __forceinline__ bool mx_bar_wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t i = 0; i < (1u << 22); ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

// One CTA per (tile of MX_TW cells, row, species); MX_LPC lanes per cell.  The loop body has no branches:
// a lane past the end of its cell runs on a zero particle with zero deposit weights and its stores
// switched off.  A step of the loop pushes the lane's particles k and k+1 (rounds k and k+1 of the
// cell: the order of every sum, rank and queue entry is that of one particle per step) while
// particles k+2 and k+3 are copied into shared memory (cp.async).
#ifndef WM_MX_MINB
#define WM_MX_MINB (512 / MX_THREADS)  // resident CTAs per SM the register budget is sized for
#endif
// GATHER: the particle of cell-sorted slot p is at slot perm[p] of set a (the previous step's push
// output, see k_mixed_perm); otherwise it is at slot p.  The push does not touch the ids.
// fmap: TMA descriptor of the cell-centred fields (columns, rows, planes), boxes of MX_FTW x 3 x 6.
// SPLIT: particles that change cell go through the per-cell queue (a tile whose queue overflows is
// appended to ovf = {count, tiles...} and recomputed by k_mixed_push_redo); otherwise (the redo)
// every particle is deposited in the loop with the full form.  parity: the phase of the CTA's
// field-tile mbarrier for this tile (the CTA's tiles alternate it).
constexpr int MX_PJ_BYTES = 65 * MX_PW * 4;
constexpr int MX_XQ_BYTES = MX_TW * MX_XQ * 24;
template <int BC, bool GATHER, bool SPLIT>
__device__ __forceinline__ void mx_push_tile(const WmGeom &g, const MxConst &kc, const MixedView &a, const MixedView &b,
                                             const unsigned *__restrict__ perm, const CUtensorMap &fmap, const int *__restrict__ cumcnt,
                                             unsigned *__restrict__ code, int *__restrict__ cnt9, float *__restrict__ jtile, unsigned *status,
                                             unsigned *ovf, int tile, int jr, int isp, uint32_t parity)
{
    __shared__ int dcnt[MX_TW][9];  // per cell: particles so far that move in direction d
    __shared__ __align__(16) float fcell[MX_TW][MX_FS];  // [lane group][(b*3 + a)*6 + m]
    // per-cell partials after the loop (the first rows hold the node sums); during the loop (SPLIT)
    // the same bytes hold the per-cell queue of particles that changed cell
    __shared__ __align__(16) unsigned char qpj[SPLIT && MX_XQ_BYTES > MX_PJ_BYTES ? MX_XQ_BYTES : MX_PJ_BYTES];
    float(*cellpj)[MX_PW] = reinterpret_cast<float(*)[MX_PW]>(qpj);
    float4(*xq4)[MX_XQ] = reinterpret_cast<float4(*)[MX_XQ]>(qpj);                           // old dx, dy; new dx, dy
    float2(*xq2)[MX_XQ] = reinterpret_cast<float2(*)[MX_XQ]>(qpj + MX_TW * MX_XQ * 16);      // q vz; increments + 1 (2-bit fields)
    __shared__ int cc[MX_TW + 1];
    __shared__ unsigned char cord[MX_TW], crank[MX_TW];  // the tile's cells by particle count, most first: group g takes cell cord[g]
    __shared__ float spc[5];
    __shared__ float4 pbuf4[4][MX_THREADS];   // each lane's particles k .. k+3 (slot k & 3): (dx, dy, ux, uy)
    __shared__ float pbufz[4][MX_THREADS];    // and uz
    __shared__ unsigned permring[GATHER ? 8 : 1][MX_THREADS];  // perm entries, slot k & 7
    __shared__ __align__(128) float tmp[6][3][MX_FTW];  // the tile's cell-centred fields (one TMA box)
    __shared__ __align__(8) uint64_t fbar;
    const int row = isp * g.ny + jr;
    const int c0 = tile * MX_TW;
    const int ncell = min(MX_TW, g.nx - c0);
    const int tid = threadIdx.x;

    // cell-centred fields of cells c0-1 .. c0+MX_FTW-2, rows jr-1 .. jr+1: one TMA box (columns past
    // the grid read as zero), completing on an mbarrier that every thread waits on below
    const uint32_t fbar_a = (uint32_t)__cvta_generic_to_shared(&fbar);
    if (tid == 0) {
        if (parity == 0) {  // the CTA's first tile
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(fbar_a) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fbar_a), "r"((uint32_t)sizeof(tmp)) : "memory");
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&tmp[0][0][0])),
                     "l"(reinterpret_cast<uint64_t>(&fmap)), "r"(c0), "r"(jr), "r"(0), "r"(fbar_a)
                     : "memory");
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
    // A warp runs as many iterations as its fullest cell needs, so the cells are dealt to the lane
    // groups in order of their particle counts: each warp gets cells of similar counts and fewer
    // lanes run past the end of theirs.  (Only the warp a cell lands in changes: its lanes, their
    // particles and every sum stay the same.)  A group's field coefficients sit in the slot of the
    // group, not of the cell, so a warp's eight 16-byte reads still fall on 32 different banks.
    if (tid < MX_TW) {
        const int nme = tid < ncell ? cc[tid + 1] - cc[tid] : -1;
        int rank = 0;
        for (int o = 0; o < MX_TW; ++o) {
            const int no = o < ncell ? cc[o + 1] - cc[o] : -1;
            rank += (no > nme) || (no == nme && o < tid);
        }
        cord[rank] = (unsigned char)tid;
        crank[tid] = (unsigned char)rank;
    }
    // Every thread waits (bounded) for the field tile.  If any gave up, the CTA records the timeout
    // (the step then fails), waits once more (bounded) so that the copy is not left writing into
    // this CTA's shared memory after it exits, and pushes with zero fields rather than from a
    // partly written tile: the move codes, counts and tile currents stay well formed, so the
    // kernels after it stay in bounds.
    if (__syncthreads_or(!mx_bar_wait(fbar_a, parity))) {
        if (tid == 0) atomicOr(status, (unsigned)WMDEV_TIMEOUT);
        mx_bar_wait(fbar_a, parity);
        for (int e = tid; e < 6 * 3 * MX_FTW; e += MX_THREADS) (&tmp[0][0][0])[e] = 0.f;
        __syncthreads();
    }
    // Each cell's six fields as biquadratics in the centred offsets hx, hy of particle.f90:96-129:
    // sum_ab T(a,b) sx_a(hx) sy_b(hy) = sum_pq C(q,p) hx^p hy^q, with the TSC weights
    // sx = (1/8 - hx/2 + hx^2/2, 3/4 - hx^2, 1/8 + hx/2 + hx^2/2).  Stored [(q*3 + p)*6 + m].
    for (int e = tid; e < MX_TW * 6; e += MX_THREADS) {
        const int c = e / 6, m = e % 6;
        float P[3][3];  // row b: coefficients of hx^0, hx^1, hx^2
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float t0 = c < ncell ? tmp[m][b][c] : 0.f, t1 = c < ncell ? tmp[m][b][c + 1] : 0.f,
                        t2 = c < ncell ? tmp[m][b][c + 2] : 0.f;
            P[b][0] = 0.125f * t0 + 0.75f * t1 + 0.125f * t2;
            P[b][1] = 0.5f * (t2 - t0);
            P[b][2] = 0.5f * t0 - t1 + 0.5f * t2;
        }
        const int slot = crank[c];
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            fcell[slot][(0 * 3 + p) * 6 + m] = 0.125f * P[0][p] + 0.75f * P[1][p] + 0.125f * P[2][p];
            fcell[slot][(1 * 3 + p) * 6 + m] = 0.5f * (P[2][p] - P[0][p]);
            fcell[slot][(2 * 3 + p) * 6 + m] = 0.5f * P[0][p] - P[1][p] + 0.5f * P[2][p];
        }
    }
    for (int e = tid; e < MX_TW * 9; e += MX_THREADS) (&dcnt[0][0])[e] = 0;
    __syncthreads();

    const float fac1 = spc[0], txxx = spc[1], fac2 = spc[2], mqdd = spc[3], qs = spc[4];
    const int grp = tid / MX_LPC;  // lane group: cell cord[grp], field coefficients in slot grp
    const int c = cord[grp], sub = tid % MX_LPC, lane = tid & 31;
    const bool has_cell = c < ncell;
    const int s_beg = has_cell ? cc[c] : 0, s_end = has_cell ? cc[c + 1] : 0;
    const int nmine = (s_end - s_beg > sub) ? (s_end - s_beg - sub + MX_LPC - 1) / MX_LPC : 0;
    int nwarp = nmine;  // trip count of the warp: the largest over its lanes
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nwarp = max(nwarp, __shfl_xor_sync(FULL, nwarp, o));
    const long long rbase = a.rowbase[row];
    const ulonglong2 *stencil = reinterpret_cast<const ulonglong2 *>(&fcell[grp][0]);
    const int cg = c0 + c;

    float ax[5][4], ay[4][5], az[5][5];
#pragma unroll
    for (int jp = 0; jp < 5; ++jp)
#pragma unroll
        for (int ip = 0; ip < 5; ++ip) {
            if (ip < 4) ax[jp][ip] = 0.f;
            if (jp < 4) ay[jp][ip] = 0.f;
            az[jp][ip] = 0.f;
        }
    // Esirkepov's full 5x5 form (field.f90:224-298) for one particle: old offsets (dxo, dyo) in its
    // cell, new offsets (nxn, nyn) in the cell inc = (ix, iy) away, weights mq = -q dx/dt and
    // qg = q vz (zero for no deposit), added to this lane's accumulators.
    auto deposit_full = [&](float dxo, float dyo, float nxn, float nyn, int ix, int iy, float mq, float qg) {
        float sx0, sx1, sx2, sy0, sy1, sy2;
        shape3(dxo - 0.5f, sx0, sx1, sx2);
        shape3(dyo - 0.5f, sy0, sy1, sy2);
        // old shape on nodes 1..3 about the old cell, new shape on 1+inc..3+inc
        float dsx[5], dsy[5];
        {
            float b0, b1, b2;
            shape3(nxn - 0.5f, b0, b1, b2);
            const bool lo = ix < 0, mid = ix == 0, hi = ix > 0;
            dsx[0] = lo ? b0 : 0.f;
            dsx[1] = (lo ? b1 : mid ? b0 : 0.f) - sx0;
            dsx[2] = (lo ? b2 : mid ? b1 : b0) - sx1;
            dsx[3] = (hi ? b1 : mid ? b2 : 0.f) - sx2;
            dsx[4] = hi ? b2 : 0.f;
            shape3(nyn - 0.5f, b0, b1, b2);
            const bool ylo = iy < 0, ymid = iy == 0, yhi = iy > 0;
            dsy[0] = ylo ? b0 : 0.f;
            dsy[1] = (ylo ? b1 : ymid ? b0 : 0.f) - sy0;
            dsy[2] = (ylo ? b2 : ymid ? b1 : b0) - sy1;
            dsy[3] = (yhi ? b1 : ymid ? b2 : 0.f) - sy2;
            dsy[4] = yhi ? b2 : 0.f;
        }
        const float s0x[5] = {0.f, sx0, sx1, sx2, 0.f}, s0y[5] = {0.f, sy0, sy1, sy2, 0.f};
        float cx[4], cy[4];
        cx[0] = dsx[0];
        cy[0] = dsy[0];
    #pragma unroll
        for (int m = 1; m < 4; ++m) {
            cx[m] = cx[m - 1] + dsx[m];
            cy[m] = cy[m - 1] + dsy[m];
        }
        // the species factor folded into the cumulative weights, qg/2 and qg/3 formed once
    #pragma unroll
        for (int m = 0; m < 4; ++m) {
            cx[m] *= mq;
            cy[m] *= mq;
        }
        const float qh = 0.5f * qg, q3 = (1.f / 3.f) * qg;
        float wy[5], z1[5], z2[5];
    #pragma unroll
        for (int jp = 0; jp < 5; ++jp) {
            const bool inner = jp >= 1 && jp <= 3;
            wy[jp] = inner ? s0y[jp] + 0.5f * dsy[jp] : 0.5f * dsy[jp];
            z1[jp] = qg * wy[jp];
            z2[jp] = inner ? fmaf(qh, s0y[jp], q3 * dsy[jp]) : q3 * dsy[jp];
        }
        // the accumulators in pairs, one packed FMA per pair (each element's FMAs in the same order)
        auto acc2 = [](float &lo, float &hi, unsigned long long m1, unsigned long long m2) {
            unpack2(fma2(m1, m2, pack2(lo, hi)), lo, hi);
            };
            const unsigned long long cx01 = pack2(cx[0], cx[1]), cx23 = pack2(cx[2], cx[3]);
            const unsigned long long cy01 = pack2(cy[0], cy[1]), cy23 = pack2(cy[2], cy[3]);
    #pragma unroll
            for (int jp = 0; jp < 5; ++jp) {
                const unsigned long long w2 = pack2(wy[jp], wy[jp]);
                acc2(ax[jp][0], ax[jp][1], w2, cx01);
                acc2(ax[jp][2], ax[jp][3], w2, cx23);
            }
    #pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                const float fx = (ip >= 1 && ip <= 3) ? s0x[ip] + 0.5f * dsx[ip] : 0.5f * dsx[ip];
                const unsigned long long f2 = pack2(fx, fx);
                acc2(ay[0][ip], ay[1][ip], f2, cy01);
                acc2(ay[2][ip], ay[3][ip], f2, cy23);
            }
            const unsigned long long z2a = pack2(z2[0], z2[1]), z2b = pack2(z2[2], z2[3]);
            const unsigned long long z1a = pack2(z1[0], z1[1]), z1b = pack2(z1[2], z1[3]);
    #pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                const unsigned long long d2 = pack2(dsx[ip], dsx[ip]);
                acc2(az[0][ip], az[1][ip], d2, z2a);
                acc2(az[2][ip], az[3][ip], d2, z2b);
                az[4][ip] = fmaf(dsx[ip], z2[4], az[4][ip]);
                if (ip >= 1 && ip <= 3) {
                    const unsigned long long s2 = pack2(s0x[ip], s0x[ip]);
                    acc2(az[0][ip], az[1][ip], s2, z1a);
                    acc2(az[2][ip], az[3][ip], s2, z1b);
                    az[4][ip] = fmaf(s0x[ip], z1[4], az[4][ip]);
                }
            }
    };
    const unsigned cellmask = ((1u << MX_LPC) - 1u) << (lane & ~(MX_LPC - 1));  // this cell's lanes in the warp
    int xn = 0;  // particles of this cell that changed cell so far (the same in all its lanes)
    unsigned bad = 0;
    // lane's particle k (at slot q of set a) -> pbuf[k & 3]; a lane past its cell copies zeros.
    // GATHER: the perm entry of particle k + 4 travels in particle k's copy group (into
    // permring[(k + 4) & 7]), so it is in shared memory when particle k + 4 is fetched.
    auto canon = [&](int it) { return rbase + s_beg + sub + (long long)it * MX_LPC; };
    auto prefetch = [&](int k, long long q) {
        const bool v = k < nmine;
        cp_async16(&pbuf4[k & 3][tid], a.xyuv + q, v ? 16u : 0u);
        cp_async4(&pbufz[k & 3][tid], a.uz + q, v ? 4u : 0u);
        if constexpr (GATHER) {
            const int jp = k + 4;
            const bool vp = jp < nmine;
            cp_async4(reinterpret_cast<float *>(&permring[jp & 7][tid]), reinterpret_cast<const float *>(perm + (vp ? canon(jp) : 0)), vp ? 4u : 0u);
        }
        cp_async_commit();
    };
    auto source = [&](int k) -> long long {
        if constexpr (GATHER) return k < nmine ? (long long)permring[k & 7][tid] : 0LL;
        else return k < nmine ? canon(k) : 0LL;
    };
    auto direct = [&](int j) -> long long {
        if constexpr (GATHER) return j < nmine ? (long long)__ldg(perm + canon(j)) : 0LL;
        else return j < nmine ? canon(j) : 0LL;
    };
    if constexpr (GATHER) {
        permring[2][tid] = (unsigned)direct(2);
        permring[3][tid] = (unsigned)direct(3);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        if (i < nwarp) prefetch(i, direct(i));
        else cp_async_commit();
    }
    // the six fields at a particle's offsets: Horner in hx then hy, two fields per packed FMA
    auto gather = [&](const unsigned long long (&cw)[28], float dx, float dy, float (&f)[6]) {
        const unsigned long long hx2 = pack2(dx - 0.5f, dx - 0.5f), hy2 = pack2(dy - 0.5f, dy - 0.5f);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            unsigned long long r[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) r[q] = fma2(hx2, fma2(hx2, cw[(q * 3 + 2) * 3 + j], cw[(q * 3 + 1) * 3 + j]), cw[(q * 3) * 3 + j]);
            unpack2(fma2(hy2, fma2(hy2, r[2], r[1]), r[0]), f[2 * j], f[2 * j + 1]);
        }
    };
    // the rest of one particle's step: lane particle it, record pin and uz, fields f
    auto process = [&](int it, const float4 &pin, float u3, const float (&f)[6]) {
        const bool valid = it < nmine;
        const long long p = canon(it);
        const float dx = pin.x, dy = pin.y;
        float u1 = pin.z, u2 = pin.w;
        float sx0, sx1, sx2, sy0, sy1, sy2;
        shape3(dx - 0.5f, sx0, sx1, sx2);
        shape3(dy - 0.5f, sy0, sy1, sy2);
        // Buneman-Boris
        float v1 = u1 + fac1 * f[3], v2 = u2 + fac1 * f[4], v3 = u3 + fac1 * f[5];
        const float g2 = kc.c2 + v1 * v1 + v2 * v2 + v3 * v3;
        const float igam = rsqrtf(g2);
        const float gam = g2 * igam;
        const float fac1r = fac1 * igam;
        const float fac2r = __fdividef(fac2, gam + txxx * (f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) * igam);
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
        const bool ox = nx1 >= 1.f, oy = ny1 >= 1.f;
        nx1 = ox ? nx1 - 1.f : nx1;
        ny1 = oy ? ny1 - 1.f : ny1;
        incx += ox;
        incy += oy;
        bad |= valid & (incx < -1 || incx > 1 || incy < -1 || incy > 1);
        float ig_dep = ig;
        if constexpr (BC == WM_BC_SHOCK) {  // the injection boundary acts before the deposit (proj/shock/app.f90:112-117)
            int cn = cg + incx;
            if (cn < 1) {  // wall at nxs+1 (boundary_shock.f90:272-276)
                mirror(2, cn, nx1);
                u1 = -u1;
                u2 = -u2;
                u3 = -u3;
            } else if (cn > kc.xe_cell || (cn == kc.xe_cell && nx1 > kc.xe_off)) {  // beyond xend (:277-281)
                const float v = 2.f * kc.xe_off - nx1;
                const float fl = floorf(v);
                cn = 2 * kc.xe_cell - cn + (int)fl;
                nx1 = v - fl;
                u1 = 2.f * kc.u0 - u1;
                u2 = -u2;
                u3 = -u3;
                ig_dep = rsqrtf(1.f + (u1 * u1 + u2 * u2 + u3 * u3) * kc.inv_c2);
            }
            incx = cn - cg;
            bad |= valid & (incx < -1 || incx > 1);
        }
        // Esirkepov (field.f90:224-298).  A particle that stays in its cell (inc = 0 in x and y: most
        // of them) has its old and new shapes on the 3x3 nodes about the cell, so it adds only Jx on
        // columns 1-2, Jy on rows 1-2 and Jz on the 3x3 block: the terms the full form gives there,
        // each node's FMAs in the same order.  (The full form's other terms are zero for it, but for
        // the rounding residue of the cumulative sums cx(3) and cy(3), which the continuity equation
        // sets to zero and which are dropped.)  A particle that changes cell is queued in shared
        // memory and deposited with the full form by its cell's lanes after the loop; a tile whose
        // queue overflows is recomputed by k_mixed_push_redo.
        const float mq = valid ? mqdd : 0.f;  // zero weights for a lane past its cell
        const float qg = valid ? qs * u3 * ig_dep : 0.f;
        const bool stay = !SPLIT || (incx == 0 && incy == 0);
        const bool cross = SPLIT && valid && !stay;
        const unsigned xm = __ballot_sync(FULL, cross) & cellmask;
        const int xslot = xn + __popc(xm & lanemask_lt());
        xn += __popc(xm);
        if (cross && xslot < MX_XQ) {
            xq4[c][xslot] = make_float4(dx, dy, nx1, ny1);
            xq2[c][xslot] = make_float2(qg, __int_as_float(((incx > 0) - (incx < 0) + 1) | (((incy > 0) - (incy < 0) + 1) << 2)));
        }
        if constexpr (!SPLIT) {
            deposit_full(dx, dy, nx1, ny1, incx, incy, mq, qg);
        } else {
            float b0, b1, b2, c0, c1, c2;
            shape3(nx1 - 0.5f, b0, b1, b2);
            shape3(ny1 - 0.5f, c0, c1, c2);
            const float ms = stay ? mq : 0.f, qz = stay ? qg : 0.f;
            const float ex[3] = {b0 - sx0, b1 - sx1, b2 - sx2}, ey[3] = {c0 - sy0, c1 - sy1, c2 - sy2};  // dsx, dsy on nodes 1..3
            const float sxa[3] = {sx0, sx1, sx2}, sya[3] = {sy0, sy1, sy2};
            const float cx1 = ex[0] * ms, cx2 = (ex[0] + ex[1]) * ms;
            const float cy1 = ey[0] * ms, cy2 = (ey[0] + ey[1]) * ms;
            const float qh = 0.5f * qz, q3 = (1.f / 3.f) * qz;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float wy = sya[j] + 0.5f * ey[j];
                ax[j + 1][1] = fmaf(wy, cx1, ax[j + 1][1]);
                ax[j + 1][2] = fmaf(wy, cx2, ax[j + 1][2]);
                const float fx = sxa[j] + 0.5f * ex[j];
                ay[1][j + 1] = fmaf(fx, cy1, ay[1][j + 1]);
                ay[2][j + 1] = fmaf(fx, cy2, ay[2][j + 1]);
            }
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float wy = sya[j] + 0.5f * ey[j];
                const float z1 = qz * wy, z2 = fmaf(qh, sya[j], q3 * ey[j]);
#pragma unroll
                for (int i = 0; i < 3; ++i) az[j + 1][i + 1] = fmaf(sxa[i], z1, fmaf(ex[i], z2, az[j + 1][i + 1]));
            }
        }
        if constexpr (BC == WM_BC_RECONNECTION) {  // particle_x after the field solve (boundary_reconnection.f90:80-91)
            int cn = cg + incx;
            if (cn < 1 || cn >= g.nx - 2) {
                mirror(cn < 1 ? 2 : 2 * (g.nx - 2), cn, nx1);
                u1 = -u1;
                u2 = -u2;
                u3 = -u3;
            }
            incx = cn - cg;
        }
        // direction d = (dy+1)*3 + dx+1 and the rank among this cell's particles moving that way,
        // in particle order: the cell's lanes before this one with the same d this round (three
        // shuffles within the cell's lane group; a lane past its cell matches none), plus earlier
        // rounds; the cell's last lane with that d advances the count.  (A step of more than one
        // cell is flagged above; the clamp keeps the move in bounds.)
        const int d = (min(max(incy, -1), 1) + 1) * 3 + (min(max(incx, -1), 1) + 1);
        const int dv = valid ? d : -1 - sub;
        int below = 0, above = 0;
#pragma unroll
        for (int k = 1; k < MX_LPC; ++k) {
            const int ou = __shfl_up_sync(FULL, dv, k, MX_LPC), od = __shfl_down_sync(FULL, dv, k, MX_LPC);
            below += (sub >= k) && (ou == dv);
            above += (sub + k < MX_LPC) && (od == dv);
        }
        const int rank = (valid ? dcnt[c][d] : 0) + below;
        __syncwarp();
        if (valid && above == 0) dcnt[c][d] = rank + 1;
        __syncwarp();
        bad |= valid & (rank >= (1 << (28 - MX_CB)));
        store_particle(b, p, nx1, ny1, u1, u2, u3, code, ((unsigned)rank << (4 + MX_CB)) | ((unsigned)c << 4) | (unsigned)d, valid);
    };
    // two particles per step of the loop: the cell's field coefficients are read once for both
    for (int it = 0; it < nwarp; it += 2) {
        const bool has_b = it + 1 < nwarp;  // (uniform over the warp)
        if (it + 2 < nwarp) prefetch(it + 2, source(it + 2));
        else cp_async_commit();
        if (it + 3 < nwarp) prefetch(it + 3, source(it + 3));
        else cp_async_commit();
        cp_async_wait<2>();  // one copy group per particle: those of it and it+1 have landed, it+2 and it+3 fly
        // (without a particle it+1, slot (it+1) & 3 holds an older record: gathered, never used)
        const float4 pa = pbuf4[it & 3][tid], pb = pbuf4[(it + 1) & 3][tid];
        const float za = pbufz[it & 3][tid], zb = pbufz[(it + 1) & 3][tid];
        float fa[6], fb[6];
        {
            unsigned long long cw[28];
#pragma unroll
            for (int q4 = 0; q4 < 14; ++q4) {
                const ulonglong2 t = stencil[q4];
                cw[2 * q4] = t.x;
                cw[2 * q4 + 1] = t.y;
            }
            gather(cw, pa.x, pa.y, fa);
            gather(cw, pb.x, pb.y, fb);
        }
        process(it, pa, za, fa);
        if (has_b) process(it + 1, pb, zb, fb);
    }
    // the queued particles of each cell that changed cell, deposited by the cell's lanes with the full form
    if constexpr (SPLIT) {
        const int nq = min(xn, MX_XQ);
        int nit = nq > sub ? (nq - sub + MX_LPC - 1) / MX_LPC : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nit = max(nit, __shfl_xor_sync(FULL, nit, o));
        __syncwarp();
        for (int j = 0; j < nit; ++j) {
            const int k = sub + j * MX_LPC;
            const bool v = k < nq;
            const float4 r = v ? xq4[c][k] : make_float4(0.5f, 0.5f, 0.5f, 0.5f);
            const float2 r2 = v ? xq2[c][k] : make_float2(0.f, __int_as_float(5));
            const int ic = __float_as_int(r2.y);
            deposit_full(r.x, r.y, r.z, r.w, (ic & 3) - 1, (ic >> 2) - 1, v ? mqdd : 0.f, v ? r2.x : 0.f);
        }
    }
    if (bad) atomicOr(status, (unsigned)WMDEV_CELL);
    if constexpr (SPLIT) {  // a queue that overflowed: the whole tile is recomputed by k_mixed_push_redo
        if (__syncthreads_or(xn > MX_XQ) && tid == 0) {
            const unsigned k = atomicAdd(ovf, 1u);
            ovf[1 + k] = (unsigned)(((isp * g.ny + jr) * ((g.nx + MX_TW - 1) / MX_TW)) + tile);
        }
    }
    // this tile's per-cell direction counts (the cells of a warp are its own)
    if (has_cell)
        for (int dd = sub; dd < 9; dd += MX_LPC) cnt9[((long long)row * g.nx + cg) * 9 + dd] = dcnt[c][dd];

    // the MX_LPC lanes of a cell add their partial currents; lane 0 of the cell keeps the sum
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
    // (the queue is consumed by every warp: the barrier of the overflow test is behind)
    for (int e = tid; e < 65 * 8; e += MX_THREADS) {  // zero pad columns of the partials
        const int r = e >> 3, q = e & 7;
        cellpj[r][q < 4 ? q : MX_TW + q] = 0.f;
    }
    if (sub == 0) {
        const int col = c + 4;
#pragma unroll
        for (int jp = 0; jp < 5; ++jp)
#pragma unroll
            for (int ip = 0; ip < 5; ++ip) {
                if (ip < 4) cellpj[jp * 4 + ip][col] = has_cell ? ax[jp][ip] : 0.f;
                if (jp < 4) cellpj[20 + jp * 5 + ip][col] = has_cell ? ay[jp][ip] : 0.f;
                cellpj[40 + jp * 5 + ip][col] = has_cell ? az[jp][ip] : 0.f;
            }
    }
    __syncthreads();
    // node currents of the tile footprint (5 rows x (64+4) columns): node lx takes cell lx-ip's
    // entry ip, cells ascending; pad cells are zero.  Per-tile buffer [isp][jr][tile][3][5][MX_JW].
    float *out = jtile + ((((long long)isp * g.ny + jr) * ((g.nx + MX_TW - 1) / MX_TW) + tile) * 3) * 5 * MX_JW;
    for (int e = tid; e < 5 * MX_JW; e += MX_THREADS) {
        const int ly = e / MX_JW, lx = e % MX_JW;
        float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int ip = 4; ip >= 0; --ip) {
            const int col = lx - ip + 4;
            if (ip >= 1) sx += cellpj[ly * 4 + ip - 1][col];
            sz += cellpj[40 + ly * 5 + ip][col];
        }
        if (ly >= 1) {
#pragma unroll
            for (int ip = 4; ip >= 0; --ip) sy += cellpj[20 + (ly - 1) * 5 + ip][lx - ip + 4];
        }
        out[e] = sx;
        out[5 * MX_JW + e] = sy;
        out[10 * MX_JW + e] = sz;
    }
}

template <int BC, bool GATHER>  // BC = WM_BC_*: the walls' code is compiled only where it runs
__global__ void __launch_bounds__(MX_THREADS, WM_MX_MINB)
    k_mixed_push_deposit(WmGeom g, MxConst kc, MixedView a, MixedView b, const unsigned *__restrict__ perm,
                         const __grid_constant__ CUtensorMap fmap, const int *__restrict__ cumcnt, unsigned *__restrict__ code,
                         int *__restrict__ cnt9, float *__restrict__ jtile, unsigned *status, unsigned *ovf)
{
    mx_push_tile<BC, GATHER, true>(g, kc, a, b, perm, fmap, cumcnt, code, cnt9, jtile, status, ovf, blockIdx.x, blockIdx.y, blockIdx.z, 0u);
}

// The tiles whose queue of cell-changing particles overflowed, recomputed from the same inputs
// with every particle deposited in the loop (the same pushed particles, codes and counts, and the
// tile's currents in full); a persistent grid over the list ovf = {count, tiles...}, which
// finishes at once when the list is empty.
template <int BC, bool GATHER>
__global__ void __launch_bounds__(MX_THREADS, WM_MX_MINB)
    k_mixed_push_redo(WmGeom g, MxConst kc, MixedView a, MixedView b, const unsigned *__restrict__ perm,
                      const __grid_constant__ CUtensorMap fmap, const int *__restrict__ cumcnt, unsigned *__restrict__ code,
                      int *__restrict__ cnt9, float *__restrict__ jtile, unsigned *status, const unsigned *__restrict__ ovf)
{
    const unsigned n = ovf[0];
    const int ntiles = (g.nx + MX_TW - 1) / MX_TW;
    uint32_t parity = 0;
    for (unsigned k = blockIdx.x; k < n; k += gridDim.x) {
        const int t = (int)ovf[1 + k];
        const int tile = t % ntiles, rw = t / ntiles;
        mx_push_tile<BC, GATHER, false>(g, kc, a, b, perm, fmap, cumcnt, code, cnt9, jtile, status, nullptr, tile, rw % g.ny, rw / g.ny, parity);
        parity ^= 1u;
        __syncthreads();
    }
}


// Rebin of the mixed path (the wrap of boundary_periodic.f90:61-96 and :143-165 and the per-cell
// order of sort.f90:36-82): a particle of source cell s that moved in direction d (code = rank << 4
// | d) goes to cell s + d.  The particles of a destination cell are ordered by source, in the fixed
// order k = (sy+1)*3 + sx+1 of the source's offset (sy, sx) from the destination (d = 8 - k),
// then by rank, which is the particle order within the source cell: a deterministic cell-sorted
// order.  (The FP64 path keeps the reference's particle_y slot order instead.)
// off9[dest][k] = particles coming from the sources before k; cellcnt[dest] = all of them.
__global__ void k_mixed_incoming(WmGeom g, const int *__restrict__ cnt9, int *__restrict__ off9, int *__restrict__ cellcnt)
{
    const long long n = (long long)g.nrows * g.nx;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(e % g.nx), row = (int)(e / g.nx);
        const int isp = row / g.ny, jr = row % g.ny;
        int run = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            int sr = jr + k / 3 - 1, sc = ci + k % 3 - 1;
            sr += sr < 0 ? g.ny : (sr >= g.ny ? -g.ny : 0);
            sc += sc < 0 ? g.nx : (sc >= g.nx ? -g.nx : 0);
            off9[e * 9 + k] = run;
            run += cnt9[((long long)(isp * g.ny + sr) * g.nx + sc) * 9 + (8 - k)];
        }
        cellcnt[e] = run;
    }
}

// Move every pushed particle (src: the push output in the old order) to its slot in the new
// cell-sorted order (dst), ids included.  One CTA per (tile, row, species) of source cells.  The
// slot of the first particle each tile cell sends in each direction is set up once per tile; a
// particle's code (rank << 10 | tile cell << 4 | direction) then gives its slot directly.
__global__ void __launch_bounds__(MX_THREADS) k_mixed_move(WmGeom g, MixedView src, MixedView dst, const int *__restrict__ cumcnt_old,
                                                           const int *__restrict__ cumcnt_new, const int *__restrict__ off9,
                                                           const unsigned *__restrict__ code)
{
    __shared__ long long base9[MX_TW][9];
    __shared__ int span[2];
    const int tile = blockIdx.x, jr = blockIdx.y, isp = blockIdx.z;
    const int row = isp * g.ny + jr;
    const int c0 = tile * MX_TW;
    const int ncell = min(MX_TW, g.nx - c0);
    const int *ccrow = cumcnt_old + (long long)(g.nx + 1) * row;
    for (int e = threadIdx.x; e < ncell * 9; e += MX_THREADS) {
        const int c = e / 9, d = e % 9;
        int dr = jr + d / 3 - 1, dc = c0 + c + d % 3 - 1;
        dr += dr < 0 ? g.ny : (dr >= g.ny ? -g.ny : 0);
        dc += dc < 0 ? g.nx : (dc >= g.nx ? -g.nx : 0);
        const int drow = isp * g.ny + dr;
        base9[c][d] = dst.rowbase[drow] + cumcnt_new[(long long)(g.nx + 1) * drow + dc] + off9[((long long)drow * g.nx + dc) * 9 + (8 - d)];
    }
    if (threadIdx.x == 0) {
        span[0] = ccrow[c0];
        span[1] = ccrow[c0 + ncell];
    }
    __syncthreads();
    const long long rb = src.rowbase[row];
    for (int s = span[0] + threadIdx.x; s < span[1]; s += MX_THREADS) {
        const long long p = rb + s;
        const unsigned cv = code[p];
        const long long q = base9[(cv >> 4) & ((1u << MX_CB) - 1)][cv & 15u] + (cv >> (4 + MX_CB));
        copy_particle(dst, q, src, p);
    }
}

// The rebin as a permutation: instead of moving the pushed particles (k_mixed_move), record for
// every slot q of the new cell-sorted order the slot p of the push output that holds its particle,
// perm[q] = p (same slots as k_mixed_move computes).  The next push reads its particles through
// perm, which moves them into cell order as a side effect of the step's own reads and writes.
// The ids are not moved at all: idperm maps a cell-sorted slot to the slot of the id array that
// holds its particle's id, idperm_new[q] = idperm_old[p] (idperm_old = null: the identity).
__global__ void __launch_bounds__(MX_THREADS) k_mixed_perm(WmGeom g, const long long *__restrict__ rowbase_src,
                                                           const long long *__restrict__ rowbase_dst, const int *__restrict__ cumcnt_old,
                                                           const int *__restrict__ cumcnt_new, const int *__restrict__ off9,
                                                           const unsigned *__restrict__ code, unsigned *__restrict__ perm,
                                                           const unsigned *__restrict__ idperm_old, unsigned *__restrict__ idperm_new)
{
    __shared__ long long base9[MX_TW][9];
    __shared__ int span[2];
    const int tile = blockIdx.x, jr = blockIdx.y, isp = blockIdx.z;
    const int row = isp * g.ny + jr;
    const int c0 = tile * MX_TW;
    const int ncell = min(MX_TW, g.nx - c0);
    const int *ccrow = cumcnt_old + (long long)(g.nx + 1) * row;
    for (int e = threadIdx.x; e < ncell * 9; e += MX_THREADS) {
        const int c = e / 9, d = e % 9;
        int dr = jr + d / 3 - 1, dc = c0 + c + d % 3 - 1;
        dr += dr < 0 ? g.ny : (dr >= g.ny ? -g.ny : 0);
        dc += dc < 0 ? g.nx : (dc >= g.nx ? -g.nx : 0);
        const int drow = isp * g.ny + dr;
        base9[c][d] = rowbase_dst[drow] + cumcnt_new[(long long)(g.nx + 1) * drow + dc] + off9[((long long)drow * g.nx + dc) * 9 + (8 - d)];
    }
    if (threadIdx.x == 0) {
        span[0] = ccrow[c0];
        span[1] = ccrow[c0 + ncell];
    }
    __syncthreads();
    const long long rb = rowbase_src[row];
    for (int s = span[0] + threadIdx.x; s < span[1]; s += MX_THREADS) {
        const long long p = rb + s;
        const unsigned cv = code[p];
        const long long q = base9[(cv >> 4) & ((1u << MX_CB) - 1)][cv & 15u] + (cv >> (4 + MX_CB));
        perm[q] = (unsigned)p;
        idperm_new[q] = idperm_old ? idperm_old[p] : (unsigned)p;
    }
}

// dst slot p = src slot perm[p] for the np2[row] slots of every row, the id from slot idperm[p]
// of src's id array: the cell-sorted state that the other kernels and the host copies read.
__global__ void k_mixed_gather(WmGeom g, MixedView src, MixedView dst, const unsigned *__restrict__ perm, const unsigned *__restrict__ idperm,
                               const int *__restrict__ np2)
{
    const int row = blockIdx.y;
    const int n = np2[row];
    const long long rb = dst.rowbase[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const long long p = rb + s, q = perm[p];
        dst.XYUV(p) = src.XYUV(q);
        dst.UZ(p) = src.UZ(q);
        dst.setpid(p, src.getpid((long long)idperm[p]));
    }
}

// FP32 -> FP64 by moving the exponent and mantissa bits (integer instructions; GB300's FP64 pipe
// runs about 2 operations per clock per SM, and the conversion instruction would be one of them).
// Exact, as the conversion is: zeros keep their sign, denormals, infinities and NaNs take the
// conversion instruction.
__device__ __forceinline__ double f2d_exact(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)sign);
    if (ex == 0u || ex == 0xffu) return (double)f;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// A compensated FP32 sum (Knuth's TwoSum: hi + lo carries the sum to about 2^-48 of the sum of
// magnitudes, near FP64's rounding) with no FP64 instruction until the end: GB300's FP64 pipe
// runs about 2 operations per clock per SM, its FP32 pipes 128.
struct Sum2f {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float s = hi + x, bb = s - hi;
        lo += (hi - (s - bb)) + (x - bb);
        hi = s;
    }
    __device__ __forceinline__ double value() const { return f2d_exact(hi) + f2d_exact(lo); }
};

// uj(k, ix, iy) over the ghosted grid = sum of the tile currents that cover the node, in the
// order (species, cell row, tile), accumulated as a compensated FP32 sum and rounded once to FP64.
// A node is covered by the tiles of at most 5 cell rows (iy-4 .. iy) and, in the first 4 columns
// of every tile but the first, by 2 tiles (ix/32 - 1 and ix/32).  The threads take those two-tile
// columns first and the one-tile columns after, so a warp's lanes agree on the number of tiles;
// all of a node's loads are issued before its sums.
template <bool PAIR>
__device__ __forceinline__ void jfold_node(const WmGeom &g, int ntiles, const float *__restrict__ jtile, FView<3, false> &uj, int ix, int iy)
{
    const long long tstride = 3LL * 5 * MX_JW;  // floats per tile
    const int th = min(ntiles - 1, ix / MX_TW);
    const int lx1 = ix - th * MX_TW, lx0 = lx1 + MX_TW;  // column in tile th and (PAIR) in tile th-1
    Sum2f s[3];
    for (int isp = 0; isp < g.nsp; ++isp) {
        float v[5][2][3];
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            const int cj = iy - 4 + r, ly = 4 - r;
            const bool rok = cj >= 0 && cj < g.ny;
            const float *row = jtile + (((long long)isp * g.ny + (rok ? cj : 0)) * ntiles + th) * tstride + ly * MX_JW;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if constexpr (PAIR) v[r][0][k] = rok ? __ldg(row - tstride + k * 5 * MX_JW + lx0) : 0.f;
                v[r][1][k] = rok ? __ldg(row + k * 5 * MX_JW + lx1) : 0.f;
            }
        }
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            const int cj = iy - 4 + r;
            if (cj < 0 || cj >= g.ny) continue;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if constexpr (PAIR) s[k].add(v[r][0][k]);
                s[k].add(v[r][1][k]);
            }
        }
    }
    uj(0, ix, iy) = s[0].value();
    uj(1, ix, iy) = s[1].value();
    uj(2, ix, iy) = s[2].value();
}

__global__ void k_mixed_jfold(WmGeom g, int ntiles, const float *__restrict__ jtile, FView<3, false> uj)
{
    const int npc = 4 * max(0, min(ntiles - 1, (g.nxw - MX_TW) / MX_TW + 1));  // two-tile columns 32t .. 32t+3, t = 1 .. ntiles-1
    const int nsc = g.nxw - npc;                                                // the other columns
    const long long npair = (long long)npc * g.nyw, n = (long long)g.nxw * g.nyw;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        if (e < npair) {
            const int iy = (int)(e / npc), j = (int)(e % npc);
            jfold_node<true>(g, ntiles, jtile, uj, MX_TW * (1 + j / 4) + j % 4, iy);
        } else {
            const long long m = e - npair;
            const int iy = (int)(m / nsc), j = (int)(m % nsc);
            int ix;
            if (j < MX_TW) {
                ix = j;  // tile 0
            } else {
                const int j2 = j - MX_TW, blk = j2 / (MX_TW - 4);
                ix = blk < ntiles - 1 ? MX_TW * (1 + blk) + 4 + j2 % (MX_TW - 4) : MX_TW * ntiles + (j2 - (MX_TW - 4) * (ntiles - 1));
            }
            jfold_node<false>(g, ntiles, jtile, uj, ix, iy);
        }
    }
}

// FP64 reference-layout staging (pitch slots per row) -> mixed set; key = row * nx + cell for the
// load-time sort.  Offsets are taken against the particle's own cell int(x) and its row.
__global__ void k_mixed_unpack(WmGeom g, const double *__restrict__ stage, int pitch, const int *__restrict__ np2, MixedView dst,
                               int *__restrict__ key, int *__restrict__ cellcnt, unsigned *status, int row0)
{
    const int row = row0 + blockIdx.y;
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
        dst.XYUV(p) = make_float4(ox, oy, (float)a[2], (float)a[3]);
        dst.UZ(p) = (float)a[4];
        dst.setpid(p, __double_as_longlong(a[5]));
        const int k = row * g.nx + ci;
        key[p] = k;
        atomicAdd(&cellcnt[k], 1);
    }
    if (bad) atomicOr(status, (unsigned)WMDEV_CELL);
}

// mixed set -> FP64 reference-layout staging; the cell of each particle comes from cumcnt.
constexpr int PACK_TW = 64;       // cells per pack CTA
constexpr int PACK_THREADS = 256;

// One CTA per (64-cell tile, row) writes the tile's particles, in slot order, as reference-layout
// records (x, y, ux, uy, uz, id as 6 doubles) -- the cell comes from cumcnt, searched in shared
// memory -- through a shared-memory buffer, so the stage is written in 16-byte vectors; the CTA
// past the last tile zeroes the row's slots from np2 to the pitch.  Rows are rstride slots apart
// (rstride >= pitch: the stage may be the caller's mapped host array, whose rows hold np slots).
// With perm, slot p's particle is read from slot perm[p] of src and its id from slot idperm[p]:
// the permuted state packed without first gathering it into cell order.
__global__ void __launch_bounds__(PACK_THREADS) k_mixed_pack(WmGeom g, MixedView src, const int *__restrict__ np2,
                                                             const int *__restrict__ cumcnt, int pitch, long long rstride,
                                                             double *__restrict__ stage, int row0, const unsigned *__restrict__ perm,
                                                             const unsigned *__restrict__ idperm)
{
    __shared__ int cc[PACK_TW + 1];
    __shared__ __align__(16) double buf[PACK_THREADS * 6];
    const int row = row0 + blockIdx.y;
    const int jr = row % g.ny;
    const long long rs = (long long)row * rstride;  // the row's first slot in the stage
    const int ntile = (g.nx + PACK_TW - 1) / PACK_TW;
    if ((int)blockIdx.x == ntile) {  // zero tail
        const int n = np2[row];
        uint4 *z = reinterpret_cast<uint4 *>(stage + 6 * (rs + n));
        const long long nv = 3LL * (pitch - n);
        for (long long e = threadIdx.x; e < nv; e += PACK_THREADS) z[e] = make_uint4(0u, 0u, 0u, 0u);
        return;
    }
    const int c0 = blockIdx.x * PACK_TW, ncell = min(PACK_TW, g.nx - c0);
    const int *ccrow = cumcnt + (long long)(g.nx + 1) * row;
    for (int e = threadIdx.x; e <= ncell; e += PACK_THREADS) cc[e] = ccrow[c0 + e];
    __syncthreads();
    const int beg = cc[0], end = cc[ncell];
    const long long rb = src.rowbase[row];
    for (int s0 = beg; s0 < end; s0 += PACK_THREADS) {
        const int s = s0 + threadIdx.x;
        if (s < end) {
            int lo = 0, hi = ncell - 1;  // the last cell whose start is <= s
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (cc[mid] <= s) lo = mid;
                else hi = mid - 1;
            }
            const long long p = rb + s, q = perm ? (long long)perm[p] : p;  // (perm: as k_mixed_gather reads it)
            double *a = buf + 6 * threadIdx.x;
            const float4 r = src.XYUV(q);
            a[0] = (double)(g.nxgs + c0 + lo) + (double)r.x;
            a[1] = (double)(g.nys + jr) + (double)r.y;
            a[2] = r.z;
            a[3] = r.w;
            a[4] = src.UZ(q);
            a[5] = __longlong_as_double(src.getpid(idperm ? (long long)idperm[p] : p));
        }
        __syncthreads();
        const int nv = 3 * min(PACK_THREADS, end - s0);  // 16-byte words of this chunk
        const uint4 *b = reinterpret_cast<const uint4 *>(buf);
        uint4 *d = reinterpret_cast<uint4 *>(stage + 6 * (rs + s0));
        for (int e = threadIdx.x; e < nv; e += PACK_THREADS) d[e] = b[e];
        __syncthreads();
    }
}

}  // namespace

int wm_mixed_ntiles(const WmGeom &g) { return (g.nx + MX_TW - 1) / MX_TW; }
size_t wm_mixed_jtile_floats(const WmGeom &g) { return (size_t)g.nsp * g.ny * wm_mixed_ntiles(g) * 3 * 5 * MX_JW; }
static int fcc_pitch(const WmGeom &g) { return (g.nx + 2 + 3) & ~3; }
size_t wm_mixed_fcc_floats(const WmGeom &g) { return (size_t)6 * fcc_pitch(g) * (g.ny + 2); }

int wm_launch_mixed_fields(const WmGeom &g, FView<6, false> uf, float *fcc, cudaStream_t st)
{
    const long long n = (long long)(g.nx + 2) * (g.ny + 2);
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_mixed_fields<<<blocks, 256, 0, st>>>(g, uf, fcc, fcc_pitch(g));
    return wm_check_launch("k_mixed_fields");
}

size_t wm_mixed_ovf_words(const WmGeom &g) { return 1 + (size_t)wm_mixed_ntiles(g) * g.nrows; }

int wm_launch_mixed_push_deposit(const WmGeom &g, const WmConst &k, MixedView a, MixedView b, const unsigned *perm, const float *fcc,
                                 const int *cumcnt, const WmRebinScratch &sc, int *cnt9, float *jtile, unsigned *ovf, cudaStream_t st)
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
    kc.bc = g.bc;
    {  // xend of boundary_shock.f90:266 in interior cells, at the active nxe
        const double xend = (g.nxgs + g.nxa - 1) * k.delx + k.u0 / sqrt(1 + (k.u0 * k.u0) / (k.c * k.c)) * k.delt;
        const double xe = xend / k.delx - g.nxgs;
        kc.xe_cell = (int)floor(xe);
        kc.xe_off = (float)(xe - kc.xe_cell);
        kc.u0 = (float)k.u0;
    }
    dim3 grid(wm_mixed_ntiles(g), g.ny, g.nsp);
    unsigned *code = reinterpret_cast<unsigned *>(sc.key);
    CUtensorMap fmap;
    {
        const unsigned long long p = (unsigned long long)fcc_pitch(g);
        const unsigned long long dims[3] = {(unsigned long long)g.nx + 2, (unsigned long long)g.ny + 2, 6};
        const unsigned long long strides[2] = {4 * p, 4 * p * (g.ny + 2)};
        const unsigned box[3] = {MX_FTW, 3, 6};
        WM_TRY(wm_tensor_map(&fmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, fcc, dims, strides, box));
    }
    static int redo_blocks = 0;  // a persistent grid of one wave for the recomputed tiles
    if (redo_blocks == 0) {
        int dev = 0, nsm = 0;
        WM_CUDA(cudaGetDevice(&dev));
        WM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        redo_blocks = std::max(1, nsm * WM_MX_MINB);
    }
    WM_CUDA(cudaMemsetAsync(ovf, 0, sizeof(unsigned), st));
#define WM_MX_PUSH(BCV, GV)                                                                                                      \
    do {                                                                                                                          \
        k_mixed_push_deposit<BCV, GV><<<grid, MX_THREADS, 0, st>>>(g, kc, a, b, perm, fmap, cumcnt, code, cnt9, jtile, sc.status, ovf); \
        WM_TRY(wm_check_launch("k_mixed_push_deposit"));                                                                       \
        k_mixed_push_redo<BCV, GV><<<redo_blocks, MX_THREADS, 0, st>>>(g, kc, a, b, perm, fmap, cumcnt, code, cnt9, jtile, sc.status, ovf); \
    } while (0)
    if (g.bc == WM_BC_RECONNECTION) {
        if (perm) WM_MX_PUSH(WM_BC_RECONNECTION, true);
        else WM_MX_PUSH(WM_BC_RECONNECTION, false);
    } else if (g.bc == WM_BC_SHOCK) {
        if (perm) WM_MX_PUSH(WM_BC_SHOCK, true);
        else WM_MX_PUSH(WM_BC_SHOCK, false);
    } else {
        if (perm) WM_MX_PUSH(WM_BC_PERIODIC, true);
        else WM_MX_PUSH(WM_BC_PERIODIC, false);
    }
#undef WM_MX_PUSH
    return wm_check_launch("k_mixed_push_redo");
}

int wm_launch_mixed_incoming(const WmGeom &g, const int *cnt9, int *off9, const WmRebinScratch &sc, cudaStream_t st)
{
    const long long n = (long long)g.nrows * g.nx;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_mixed_incoming<<<blocks, 256, 0, st>>>(g, cnt9, off9, sc.cellcnt);
    return wm_check_launch("k_mixed_incoming");
}

int wm_launch_mixed_move(const WmGeom &g, MixedView src, MixedView dst, const int *cumcnt_old, const int *cumcnt_new, const int *off9,
                         const WmRebinScratch &sc, cudaStream_t st)
{
    dim3 grid(wm_mixed_ntiles(g), g.ny, g.nsp);
    k_mixed_move<<<grid, MX_THREADS, 0, st>>>(g, src, dst, cumcnt_old, cumcnt_new, off9, reinterpret_cast<const unsigned *>(sc.key));
    return wm_check_launch("k_mixed_move");
}

int wm_launch_mixed_perm(const WmGeom &g, const long long *rowbase_src, const long long *rowbase_dst, const int *cumcnt_old,
                         const int *cumcnt_new, const int *off9, const WmRebinScratch &sc, unsigned *perm, const unsigned *idperm_old,
                         unsigned *idperm_new, cudaStream_t st)
{
    dim3 grid(wm_mixed_ntiles(g), g.ny, g.nsp);
    k_mixed_perm<<<grid, MX_THREADS, 0, st>>>(g, rowbase_src, rowbase_dst, cumcnt_old, cumcnt_new, off9, reinterpret_cast<const unsigned *>(sc.key),
                                              perm, idperm_old, idperm_new);
    return wm_check_launch("k_mixed_perm");
}

int wm_launch_mixed_gather(const WmGeom &g, MixedView src, MixedView dst, const unsigned *perm, const unsigned *idperm, const int *np2, int max_row,
                           cudaStream_t st)
{
    dim3 grid(std::min(wm_div_up(std::max(max_row, 1), 256), 64u), g.nrows);
    k_mixed_gather<<<grid, 256, 0, st>>>(g, src, dst, perm, idperm, np2);
    return wm_check_launch("k_mixed_gather");
}

int wm_launch_mixed_jfold(const WmGeom &g, const float *jtile, FView<3, false> uj, cudaStream_t st)
{
    const long long n = (long long)g.nxw * g.nyw;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_mixed_jfold<<<blocks, 256, 0, st>>>(g, wm_mixed_ntiles(g), jtile, uj);
    return wm_check_launch("k_mixed_jfold");
}

int wm_launch_mixed_unpack(const WmGeom &g, const double *stage, int pitch, const int *np2, MixedView dst, const WmRebinScratch &sc,
                           cudaStream_t st, int row0, int nrows)
{
    if (nrows < 0) nrows = g.nrows - row0;
    if (row0 == 0) WM_CUDA(cudaMemsetAsync(sc.cellcnt, 0, sizeof(int) * (size_t)g.nrows * g.nx, st));
    dim3 grid(std::min(wm_div_up(std::max(pitch, 1), 256), 64u), nrows);
    k_mixed_unpack<<<grid, 256, 0, st>>>(g, stage, pitch, np2, dst, sc.key, sc.cellcnt, sc.status, row0);
    return wm_check_launch("k_mixed_unpack");
}

int wm_launch_mixed_pack(const WmGeom &g, MixedView src, const int *np2, const int *cumcnt, int pitch, double *stage, cudaStream_t st,
                         int row0, int nrows, long long rstride, const unsigned *perm, const unsigned *idperm)
{
    if (nrows < 0) nrows = g.nrows - row0;
    if (rstride < 0) rstride = pitch;
    dim3 grid((g.nx + PACK_TW - 1) / PACK_TW + 1, nrows);
    k_mixed_pack<<<grid, PACK_THREADS, 0, st>>>(g, src, np2, cumcnt, pitch, rstride, stage, row0, perm, idperm);
    return wm_check_launch("k_mixed_pack");
}
