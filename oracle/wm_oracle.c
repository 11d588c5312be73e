/*
 * wm_oracle.c -- CPU restatement of the WumingPIC2D FP64 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke() entry of
 * __graft_entry__.py and the cpu_baseline leg of bench.py call it to produce the expected
 * answer.  Nothing in the product (the CUDA library under wumingpic2d_gb300/) links, loads or
 * calls it, and the product has no CPU fallback through it.
 *
 * Each routine restates one reference Fortran routine (path:line in WumingPIC2D) and keeps its
 * operation order: left-to-right evaluation of sums and products, int() truncation, default-real
 * literals (0.5, 0.75, 0.25, 1., 4. -- all exact in binary), downward rounding inside the
 * particle boundary routines, and the lagged CG stop test.  Build with -ffp-contract=off and
 * -frounding-math so that the compiler neither fuses multiply-adds nor folds the round-down
 * additions.  With OMP_NUM_THREADS=1 the results follow the reference's single-thread semantics;
 * with more threads the OpenMP reductions mirror the reference's own OMP directives.
 *
 * Arrays use the reference's column-major layout and lower bounds (single MPI rank, so
 * nys = nygs and nye = nyge):
 *   up(ndim, np, nys:nye, nsp)                 particles, slots 1..np per row
 *   uf(6, nxgs-2:nxge+2, nys-2:nye+2)          fields (Bx,By,Bz,Ex,Ey,Ez)
 *   uj(3, nxgs-2:nxge+2, nys-2:nye+2)          current
 *   cumcnt(nxgs:nxge+1, nys:nye, nsp)          cell start offsets per row
 *   np2(nys:nye, nsp)                          particles per row
 *   mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp)    moments
 *
 * Parity: the reference is Fortran and no Fortran compiler exists on either machine this
 * project runs on.  This restatement is pinned to the reference's own code through a statement-
 * by-statement C translation of the Fortran modules (f90c.py, ref_glue.c): at one thread the two
 * agree bit for bit on every routine and on whole runs (tests/test_reference_pin.py, golden
 * vectors in tests/golden/), and by the known-answer and invariant tests in tests/test_oracle.py.
 */
#include <fenv.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#pragma STDC FENV_ACCESS ON

enum { WMO_OK = 0, WMO_ERR_CG_MAXITER = 1, WMO_ERR_OVERFLOW = 2, WMO_ERR_BAD_ARG = 3, WMO_ERR_CELL = 4 };

/* Boundary module of the application: common/boundary_periodic.f90 (Weibel),
 * proj/reconnection/boundary_reconnection.f90 (walls in x, periodic in y) or
 * proj/shock/boundary_shock.f90 (reflecting wall at nxs, injection boundary at nxe). */
enum { WMO_BC_PERIODIC = 0, WMO_BC_RECONNECTION = 1, WMO_BC_SHOCK = 2 };

typedef struct wmo_par {
    int ndim, np, nsp;
    int nxgs, nxge, nygs, nyge, nys, nye;
    double delx, delt, c, gfac;
    double q[8], r[8];
    double cg_err;  /* field.f90:339  err = 1d-6 */
    int cg_itemax;  /* field.f90:337  ite_max = 100 */
    int bc;         /* WMO_BC_* */
    double u0;      /* shock: upstream four-velocity of the injection boundary (proj/shock/app.f90) */
} wmo_par;

/* ---------------------------------------------------------------- indexing helpers */
#define NYL (P->nye - P->nys + 1)
#define NXW (P->nxge - P->nxgs + 5)
static inline size_t o_up(const wmo_par *P, int k, int ii, int j, int isp)
{
    return (size_t)(k - 1) + (size_t)P->ndim * ((size_t)(ii - 1) + (size_t)P->np * ((size_t)(j - P->nys) + (size_t)NYL * (size_t)(isp - 1)));
}
static inline size_t o_f(const wmo_par *P, int nc, int k, int i, int j)
{
    return (size_t)(k - 1) + (size_t)nc * ((size_t)(i - (P->nxgs - 2)) + (size_t)NXW * (size_t)(j - (P->nys - 2)));
}
static inline size_t o_cc(const wmo_par *P, int i, int j, int isp)
{
    return (size_t)(i - P->nxgs) + (size_t)(P->nxge - P->nxgs + 2) * ((size_t)(j - P->nys) + (size_t)NYL * (size_t)(isp - 1));
}
static inline size_t o_np2(const wmo_par *P, int j, int isp) { return (size_t)(j - P->nys) + (size_t)NYL * (size_t)(isp - 1); }
static inline size_t o_mom(const wmo_par *P, int k, int i, int j, int isp)
{
    return (size_t)(k - 1) + 7 * ((size_t)(i - (P->nxgs - 1)) + (size_t)(P->nxge - P->nxgs + 3) * ((size_t)(j - (P->nys - 1)) + (size_t)(NYL + 2) * (size_t)(isp - 1)));
}
#define UP(k, ii, j, isp) up[o_up(P, k, ii, j, isp)]
#define GP(k, ii, j, isp) gp[o_up(P, k, ii, j, isp)]
#define UF(k, i, j) uf[o_f(P, 6, k, i, j)]
#define DF(k, i, j) df[o_f(P, 6, k, i, j)]
#define DBL(k, i, j) db[o_f(P, 6, k, i, j)]
#define UJ(k, i, j) uj[o_f(P, 3, k, i, j)]
#define CUMCNT(i, j, isp) cumcnt[o_cc(P, i, j, isp)]
#define NP2(j, isp) np2[o_np2(P, j, isp)]
#define MOM(k, i, j, isp) mom[o_mom(P, k, i, j, isp)]

static const double PI = 3.14159265358979311599796346854418516; /* 4*atan(1) in binary64 */

/* -------------------------------------------------------------- particle push
 * particle.f90:48-177 (particle__solv), and mom_calc.f90:48-164 (mom_calc__accl) when
 * half_step != 0: there delt is delt_in*0.5 (mom_calc.f90:34), positions are copied and the
 * pid column is left alone.                                                             */
static void push_core(const wmo_par *P, double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe,
                      int half_step)
{
    const int nys = P->nys, nye = P->nye;
    const double d_delx = 1. / P->delx;
    const double delt = half_step ? P->delt * 0.5 : P->delt;
    const double c = P->c;
    const int tnx = nxe - nxs + 3, tny = nye - nys + 3;
    double *tmp = (double *)malloc(sizeof(double) * 6 * (size_t)tnx * (size_t)tny);
#define TMP(k, i, j) tmp[(size_t)((k) - 1) + 6 * ((size_t)((i) - (nxs - 1)) + (size_t)tnx * (size_t)((j) - (nys - 1)))]

    /* fields at (i+1/2, j+1/2): particle.f90:68-81 */
#pragma omp parallel for
    for (int j = nys - 1; j <= nye + 1; ++j) {
        for (int i = nxs - 1; i <= nxe + 1; ++i) {
            TMP(1, i, j) = 0.5 * (+UF(1, i, j) + UF(1, i, j + 1));
            TMP(2, i, j) = 0.5 * (+UF(2, i, j) + UF(2, i + 1, j));
            TMP(3, i, j) = 0.25 * (+UF(3, i, j) + UF(3, i + 1, j) + UF(3, i, j + 1) + UF(3, i + 1, j + 1));
            TMP(4, i, j) = 0.5 * (+UF(4, i, j) + UF(4, i + 1, j));
            TMP(5, i, j) = 0.5 * (+UF(5, i, j) + UF(5, i, j + 1));
            TMP(6, i, j) = UF(6, i, j);
        }
    }

    /* particle loop: particle.f90:83-169 */
#pragma omp parallel for
    for (int j = nys; j <= nye; ++j) {
        for (int i = nxs; i <= nxe; ++i) {
            for (int isp = 1; isp <= P->nsp; ++isp) {
                const double qs = P->q[isp - 1], rs = P->r[isp - 1];
                const double fac1 = qs / rs * 0.5 * delt;
                const double txxx = fac1 * fac1;
                const double fac2 = qs * delt / rs;
                for (int ii = CUMCNT(i, j, isp) + 1; ii <= CUMCNT(i + 1, j, isp); ++ii) {
                    double sh[3][2], dh;
                    dh = UP(1, ii, j, isp) * d_delx - 0.5 - i;
                    sh[0][0] = 0.5 * (0.5 - dh) * (0.5 - dh);
                    sh[1][0] = 0.75 - dh * dh;
                    sh[2][0] = 0.5 * (0.5 + dh) * (0.5 + dh);
                    dh = UP(2, ii, j, isp) * d_delx - 0.5 - j;
                    sh[0][1] = 0.5 * (0.5 - dh) * (0.5 - dh);
                    sh[1][1] = 0.75 - dh * dh;
                    sh[2][1] = 0.5 * (0.5 + dh) * (0.5 + dh);
#define GATHER(k)                                                                                                   \
    (+(+TMP(k, i - 1, j - 1) * sh[0][0] + TMP(k, i, j - 1) * sh[1][0] + TMP(k, i + 1, j - 1) * sh[2][0]) * sh[0][1] \
     + (+TMP(k, i - 1, j) * sh[0][0] + TMP(k, i, j) * sh[1][0] + TMP(k, i + 1, j) * sh[2][0]) * sh[1][1]           \
     + (+TMP(k, i - 1, j + 1) * sh[0][0] + TMP(k, i, j + 1) * sh[1][0] + TMP(k, i + 1, j + 1) * sh[2][0]) * sh[2][1])
                    const double bpx = GATHER(1), bpy = GATHER(2), bpz = GATHER(3);
                    const double epx = GATHER(4), epy = GATHER(5), epz = GATHER(6);
#undef GATHER
                    double uvm1 = UP(3, ii, j, isp) + fac1 * epx;
                    double uvm2 = UP(4, ii, j, isp) + fac1 * epy;
                    double uvm3 = UP(5, ii, j, isp) + fac1 * epz;
                    double gam = sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
                    const double igam = 1. / gam;
                    const double fac1r = fac1 * igam;
                    const double fac2r = fac2 / (gam + txxx * (bpx * bpx + bpy * bpy + bpz * bpz) * igam);
                    const double uvm4 = uvm1 + fac1r * (+uvm2 * bpz - uvm3 * bpy);
                    const double uvm5 = uvm2 + fac1r * (+uvm3 * bpx - uvm1 * bpz);
                    const double uvm6 = uvm3 + fac1r * (+uvm1 * bpy - uvm2 * bpx);
                    uvm1 = uvm1 + fac2r * (+uvm5 * bpz - uvm6 * bpy);
                    uvm2 = uvm2 + fac2r * (+uvm6 * bpx - uvm4 * bpz);
                    uvm3 = uvm3 + fac2r * (+uvm4 * bpy - uvm5 * bpx);
                    if (half_step) {
                        /* mom_calc.f90:151-155 */
                        GP(1, ii, j, isp) = UP(1, ii, j, isp);
                        GP(2, ii, j, isp) = UP(2, ii, j, isp);
                        GP(3, ii, j, isp) = uvm1 + fac1 * epx;
                        GP(4, ii, j, isp) = uvm2 + fac1 * epy;
                        GP(5, ii, j, isp) = uvm3 + fac1 * epz;
                    } else {
                        GP(3, ii, j, isp) = uvm1 + fac1 * epx;
                        GP(4, ii, j, isp) = uvm2 + fac1 * epy;
                        GP(5, ii, j, isp) = uvm3 + fac1 * epz;
                        gam = 1. / sqrt(1.0 + (+GP(3, ii, j, isp) * GP(3, ii, j, isp) + GP(4, ii, j, isp) * GP(4, ii, j, isp)
                                               + GP(5, ii, j, isp) * GP(5, ii, j, isp))
                                                  / (c * c));
                        GP(1, ii, j, isp) = UP(1, ii, j, isp) + GP(3, ii, j, isp) * delt * gam;
                        GP(2, ii, j, isp) = UP(2, ii, j, isp) + GP(4, ii, j, isp) * delt * gam;
                    }
                }
            }
        }
    }
#undef TMP
    free(tmp);

    /* pid copy over every slot: particle.f90:171-175 */
    if (!half_step && P->ndim == 6) {
        const size_t nslot = (size_t)P->np * (size_t)NYL * (size_t)P->nsp;
#pragma omp parallel for
        for (size_t s = 0; s < nslot; ++s) gp[5 + 6 * s] = up[5 + 6 * s];
    }
}

void wmo_particle_solv(const wmo_par *P, double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe)
{
    push_core(P, gp, up, uf, cumcnt, nxs, nxe, 0);
}

void wmo_mom_accl(const wmo_par *P, double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe)
{
    push_core(P, gp, up, uf, cumcnt, nxs, nxe, 1);
}

/* -------------------------------------------------------- Esirkepov deposit
 * field.f90:189-316 (ele_cur).  Zeroes uj over (nxs-2:nxe+2, nys-2:nye+2) first.          */
void wmo_ele_cur(const wmo_par *P, double *uj, const double *up, const double *gp, const int *cumcnt, int nxs, int nxe)
{
    const int nys = P->nys, nye = P->nye;
    const double d_delx = 1. / P->delx, d_delt = 1. / P->delt, delx = P->delx, c = P->c;
    const double fac = 1.0 / 3.0;
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int i = nxs - 2; i <= nxe + 2; ++i)
            for (int k = 1; k <= 3; ++k) UJ(k, i, j) = 0.0;
    const size_t ujlen = (size_t)3 * (size_t)NXW * (size_t)(NYL + 4);

#pragma omp parallel for reduction(+ : uj[0 : ujlen])
    for (int j = nys; j <= nye; ++j) {
        for (int i = nxs; i <= nxe; ++i) {
            /* pj?(ip,jp) stored as [jp+2][ip+2] */
            double pjx[5][5], pjy[5][5], pjz[5][5], pjtmp[5][5];
            memset(pjx, 0, sizeof pjx);
            memset(pjy, 0, sizeof pjy);
            memset(pjz, 0, sizeof pjz);
            for (int isp = 1; isp <= P->nsp; ++isp) {
                const double qs = P->q[isp - 1];
                for (int ii = CUMCNT(i, j, isp) + 1; ii <= CUMCNT(i + 1, j, isp); ++ii) {
                    double s0[5][2], ds[5][2], dh, s1_1, s1_2, s1_3, smo_1, smo_2, smo_3;
                    int i2, inc;
                    dh = UP(1, ii, j, isp) * d_delx - 0.5 - i;
                    s0[0][0] = 0.0;
                    s0[1][0] = 0.5 * (0.5 - dh) * (0.5 - dh);
                    s0[2][0] = 0.75 - dh * dh;
                    s0[3][0] = 0.5 * (0.5 + dh) * (0.5 + dh);
                    s0[4][0] = 0.0;
                    dh = UP(2, ii, j, isp) * d_delx - 0.5 - j;
                    s0[0][1] = 0.0;
                    s0[1][1] = 0.5 * (0.5 - dh) * (0.5 - dh);
                    s0[2][1] = 0.75 - dh * dh;
                    s0[3][1] = 0.5 * (0.5 + dh) * (0.5 + dh);
                    s0[4][1] = 0.0;

                    i2 = (int)(GP(1, ii, j, isp) * d_delx);
                    dh = GP(1, ii, j, isp) * d_delx - 0.5 - i2;
                    inc = i2 - i;
                    s1_1 = 0.5 * (0.5 - dh) * (0.5 - dh);
                    s1_2 = 0.75 - dh * dh;
                    s1_3 = 0.5 * (0.5 + dh) * (0.5 + dh);
                    smo_1 = -(inc - abs(inc)) * 0.5 + 0;
                    smo_2 = -abs(inc) + 1;
                    smo_3 = (inc + abs(inc)) * 0.5 + 0;
                    ds[0][0] = s1_1 * smo_1;
                    ds[1][0] = s1_1 * smo_2 + s1_2 * smo_1;
                    ds[2][0] = s1_2 * smo_2 + s1_3 * smo_1 + s1_1 * smo_3;
                    ds[3][0] = s1_3 * smo_2 + s1_2 * smo_3;
                    ds[4][0] = s1_3 * smo_3;

                    i2 = (int)(GP(2, ii, j, isp) * d_delx);
                    dh = GP(2, ii, j, isp) * d_delx - 0.5 - i2;
                    inc = i2 - j;
                    s1_1 = 0.5 * (0.5 - dh) * (0.5 - dh);
                    s1_2 = 0.75 - dh * dh;
                    s1_3 = 0.5 * (0.5 + dh) * (0.5 + dh);
                    smo_1 = -(inc - abs(inc)) * 0.5 + 0;
                    smo_2 = -abs(inc) + 1;
                    smo_3 = (inc + abs(inc)) * 0.5 + 0;
                    ds[0][1] = s1_1 * smo_1;
                    ds[1][1] = s1_1 * smo_2 + s1_2 * smo_1;
                    ds[2][1] = s1_2 * smo_2 + s1_3 * smo_1 + s1_1 * smo_3;
                    ds[3][1] = s1_3 * smo_2 + s1_2 * smo_3;
                    ds[4][1] = s1_3 * smo_3;

                    for (int a = 0; a < 5; ++a) {
                        ds[a][0] = ds[a][0] - s0[a][0];
                        ds[a][1] = ds[a][1] - s0[a][1];
                    }

                    const double g3 = GP(3, ii, j, isp), g4 = GP(4, ii, j, isp), g5 = GP(5, ii, j, isp);
                    const double gvz = g5 / sqrt(1. + (+g3 * g3 + g4 * g4 + g5 * g5) / (c * c));

                    memset(pjtmp, 0, sizeof pjtmp);
                    for (int jp = -2; jp <= 2; ++jp)
                        for (int ip = -2; ip <= 1; ++ip)
                            pjtmp[jp + 2][ip + 3] = pjtmp[jp + 2][ip + 2] - qs * delx * d_delt * ds[ip + 2][0] * (s0[jp + 2][1] + 0.5 * ds[jp + 2][1]);
                    for (int a = 0; a < 5; ++a)
                        for (int b = 0; b < 5; ++b) pjx[a][b] = pjx[a][b] + pjtmp[a][b];

                    memset(pjtmp, 0, sizeof pjtmp);
                    for (int jp = -2; jp <= 1; ++jp)
                        for (int ip = -2; ip <= 2; ++ip)
                            pjtmp[jp + 3][ip + 2] = pjtmp[jp + 2][ip + 2] - qs * delx * d_delt * ds[jp + 2][1] * (s0[ip + 2][0] + 0.5 * ds[ip + 2][0]);
                    for (int a = 0; a < 5; ++a)
                        for (int b = 0; b < 5; ++b) pjy[a][b] = pjy[a][b] + pjtmp[a][b];

                    for (int jp = -2; jp <= 2; ++jp)
                        for (int ip = -2; ip <= 2; ++ip)
                            pjz[jp + 2][ip + 2] = pjz[jp + 2][ip + 2]
                                                  + qs * gvz
                                                        * (+s0[ip + 2][0] * s0[jp + 2][1] + 0.5 * ds[ip + 2][0] * s0[jp + 2][1]
                                                           + 0.5 * s0[ip + 2][0] * ds[jp + 2][1] + fac * ds[ip + 2][0] * ds[jp + 2][1]);
                }
            }
            for (int jp = -2; jp <= 2; ++jp)
                for (int ip = -2; ip <= 2; ++ip) {
                    UJ(1, i + ip, j + jp) = UJ(1, i + ip, j + jp) + pjx[jp + 2][ip + 2];
                    UJ(2, i + ip, j + jp) = UJ(2, i + ip, j + jp) + pjy[jp + 2][ip + 2];
                    UJ(3, i + ip, j + jp) = UJ(3, i + ip, j + jp) + pjz[jp + 2][ip + 2];
                }
        }
    }
}

/* ------------------------------------------------- periodic boundaries, one rank
 * With one rank nup = ndown = the rank itself (mpi_set.f90:44-47), so every MPI_SENDRECV
 * in boundary_periodic.f90 is a copy from the packed rows to the receiving rows.           */

/* boundary_periodic.f90:357-508 */
void wmo_bc_curre(const wmo_par *P, double *uj, int nxs, int nxe)
{
    const int nys = P->nys, nye = P->nye;
    /* rows nys-2,nys-1 -> added into nye-1,nye (:369-398) */
    for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int k = 1; k <= 3; ++k) {
            const double a = UJ(k, i, nys - 2), b = UJ(k, i, nys - 1);
            UJ(k, i, nye - 1) = UJ(k, i, nye - 1) + a;
            UJ(k, i, nye) = UJ(k, i, nye) + b;
        }
    /* rows nye+1,nye+2 -> added into nys,nys+1 (:400-429) */
    for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int k = 1; k <= 3; ++k) {
            const double a = UJ(k, i, nye + 1), b = UJ(k, i, nye + 2);
            UJ(k, i, nys) = UJ(k, i, nys) + a;
            UJ(k, i, nys + 1) = UJ(k, i, nys + 1) + b;
        }
    /* refill ghost rows (:433-493) */
    for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int k = 1; k <= 3; ++k) {
            UJ(k, i, nye + 1) = UJ(k, i, nys);
            UJ(k, i, nye + 2) = UJ(k, i, nys + 1);
        }
    for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int k = 1; k <= 3; ++k) {
            UJ(k, i, nys - 2) = UJ(k, i, nye - 1);
            UJ(k, i, nys - 1) = UJ(k, i, nye);
        }
    /* walls in x (boundary_reconnection.f90:364-502, boundary_shock.f90:410-548): y only */
    if (P->bc != WMO_BC_PERIODIC) return;
    /* x fold, then x refill (:495-506); each line is a whole-column statement */
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int k = 1; k <= 3; ++k) UJ(k, nxe - 1, j) = UJ(k, nxe - 1, j) + UJ(k, nxs - 2, j);
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int k = 1; k <= 3; ++k) UJ(k, nxe, j) = UJ(k, nxe, j) + UJ(k, nxs - 1, j);
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int k = 1; k <= 3; ++k) UJ(k, nxs, j) = UJ(k, nxs, j) + UJ(k, nxe + 1, j);
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int k = 1; k <= 3; ++k) UJ(k, nxs + 1, j) = UJ(k, nxs + 1, j) + UJ(k, nxe + 2, j);
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int k = 1; k <= 3; ++k) {
            UJ(k, nxs - 2, j) = UJ(k, nxe - 1, j);
            UJ(k, nxs - 1, j) = UJ(k, nxe, j);
            UJ(k, nxe + 1, j) = UJ(k, nxs, j);
            UJ(k, nxe + 2, j) = UJ(k, nxs + 1, j);
        }
}

/* boundary_periodic.f90:251-354 (6 components, 2 ghost cells) */
void wmo_bc_dfield(const wmo_par *P, double *df, int nxs, int nxe)
{
    const int nys = P->nys, nye = P->nye;
    for (int i = nxs; i <= nxe; ++i)
        for (int k = 1; k <= 6; ++k) {
            DF(k, i, nye + 1) = DF(k, i, nys);
            DF(k, i, nye + 2) = DF(k, i, nys + 1);
        }
    for (int i = nxs; i <= nxe; ++i)
        for (int k = 1; k <= 6; ++k) {
            DF(k, i, nys - 2) = DF(k, i, nye - 1);
            DF(k, i, nys - 1) = DF(k, i, nye);
        }
    if (P->bc == WMO_BC_PERIODIC) {
        for (int j = nys - 2; j <= nye + 2; ++j)
            for (int k = 1; k <= 6; ++k) {
                DF(k, nxs - 2, j) = DF(k, nxe - 1, j);
                DF(k, nxs - 1, j) = DF(k, nxe, j);
                DF(k, nxe + 1, j) = DF(k, nxs, j);
                DF(k, nxe + 2, j) = DF(k, nxs + 1, j);
            }
        return;
    }
    /* conducting wall at nxs (boundary_reconnection.f90:351-360, boundary_shock.f90:397-406) */
    for (int j = nys - 2; j <= nye + 2; ++j) {
        DF(1, nxs - 1, j) = -DF(1, nxs, j);
        for (int k = 2; k <= 4; ++k) DF(k, nxs - 1, j) = DF(k, nxs + 1, j);
        for (int k = 5; k <= 6; ++k) DF(k, nxs - 1, j) = -DF(k, nxs, j);
        if (P->bc == WMO_BC_RECONNECTION) {  /* conducting wall at nxe */
            DF(1, nxe, j) = -DF(1, nxe - 1, j);
            for (int k = 2; k <= 4; ++k) DF(k, nxe + 1, j) = DF(k, nxe - 1, j);
            for (int k = 5; k <= 6; ++k) DF(k, nxe, j) = -DF(k, nxe - 1, j);
        } else {  /* shock: zero beyond the injection boundary */
            for (int k = 1; k <= 6; ++k) DF(k, nxe + 1, j) = 0.0;
        }
    }
}

/* boundary_periodic.f90:511-568; phi(nxs-1:nxe+1, nys-1:nye+1).  Walls in x
 * (boundary_reconnection.f90:557-577, boundary_shock.f90:603-623): component l = 1 (Bx) odd
 * about nxs - 1/2, l = 2, 3 even about nxs; zero at nxe + 1. */
static void bc_phi(const wmo_par *P, double *phi, int nxs, int nxe, int l)
{
    const int nys = P->nys, nye = P->nye, pw = nxe - nxs + 3;
#define PHI(i, j) phi[(size_t)((i) - (nxs - 1)) + (size_t)pw * (size_t)((j) - (nys - 1))]
    for (int i = nxs; i <= nxe; ++i) PHI(i, nye + 1) = PHI(i, nys);
    for (int i = nxs; i <= nxe; ++i) PHI(i, nys - 1) = PHI(i, nye);
    if (P->bc == WMO_BC_PERIODIC) {
        for (int j = nys - 1; j <= nye + 1; ++j) PHI(nxs - 1, j) = PHI(nxe, j);
        for (int j = nys - 1; j <= nye + 1; ++j) PHI(nxe + 1, j) = PHI(nxs, j);
    } else {
        for (int j = nys - 1; j <= nye + 1; ++j) {
            PHI(nxs - 1, j) = (l == 1) ? -PHI(nxs, j) : PHI(nxs + 1, j);
            PHI(nxe + 1, j) = 0.0;
        }
    }
#undef PHI
}
void wmo_bc_phi(const wmo_par *P, double *phi, int nxs, int nxe, int l) { bc_phi(P, phi, nxs, nxe, l); }

/* ---------------------------------------------------------- conjugate gradient
 * field.f90:319-461 (cgm).  db has the df layout; gkl(3, nxgs:nxge, nys:nye).  iters[l-1]
 * receives the iteration count of component l.  Where the reference stops the program at
 * ite_max (field.f90:427-430) this returns WMO_ERR_CG_MAXITER.                              */
int wmo_cgm(const wmo_par *P, double *db, const double *gkl, int nxs, int nxe, int *iters)
{
    const int nys = P->nys, nye = P->nye;
    const double c = P->c, delt = P->delt, delx = P->delx, gfac = P->gfac;
    const double f4 = 4.0 + (delx / (c * delt * gfac)) * (delx / (c * delt * gfac));
    const double f5 = (delx / (c * delt * gfac)) * (delx / (c * delt * gfac));
    const double err = P->cg_err;
    const int ite_max = P->cg_itemax;
    const int pw = nxe - nxs + 3, ph = nye - nys + 3, iw = nxe - nxs + 1, ih = nye - nys + 1;
    const int gw = P->nxge - P->nxgs + 1;
    double *phi = (double *)calloc((size_t)pw * ph, sizeof(double));
    double *p = (double *)calloc((size_t)pw * ph, sizeof(double));
    double *r = (double *)calloc((size_t)iw * ih, sizeof(double));
    double *b = (double *)calloc((size_t)iw * ih, sizeof(double));
    double *ap = (double *)calloc((size_t)iw * ih, sizeof(double));
#define PHI(i, j) phi[(size_t)((i) - (nxs - 1)) + (size_t)pw * (size_t)((j) - (nys - 1))]
#define PP(i, j) p[(size_t)((i) - (nxs - 1)) + (size_t)pw * (size_t)((j) - (nys - 1))]
#define RR(i, j) r[(size_t)((i) - nxs) + (size_t)iw * (size_t)((j) - nys)]
#define BB(i, j) b[(size_t)((i) - nxs) + (size_t)iw * (size_t)((j) - nys)]
#define AP(i, j) ap[(size_t)((i) - nxs) + (size_t)iw * (size_t)((j) - nys)]
#define GKL(l, i, j) gkl[(size_t)((l) - 1) + 3 * ((size_t)((i) - P->nxgs) + (size_t)gw * (size_t)((j) - nys))]
    int status = WMO_OK;
    for (int l = 1; l <= 3 && status == WMO_OK; ++l) {
        int ite = 0;
        double sum = 0.0, sumr, sum1, sum2, av, bv, sum_g, sumr_g, eps;
#pragma omp parallel for reduction(+ : sum)
        for (int j = nys; j <= nye; ++j)
            for (int i = nxs; i <= nxe; ++i) {
                PHI(i, j) = DBL(l, i, j);
                BB(i, j) = f5 * GKL(l, i, j);
                sum = sum + BB(i, j) * BB(i, j);
            }
        sum_g = sum;
        eps = sqrt(sum_g) * err;
        bc_phi(P, phi, nxs, nxe, l);
        sumr = 0.0;
#pragma omp parallel for reduction(+ : sumr)
        for (int j = nys; j <= nye; ++j)
            for (int i = nxs; i <= nxe; ++i) {
                RR(i, j) = BB(i, j) + PHI(i, j - 1) + PHI(i - 1, j) - f4 * PHI(i, j) + PHI(i + 1, j) + PHI(i, j + 1);
                PP(i, j) = RR(i, j);
                sumr = sumr + RR(i, j) * RR(i, j);
            }
        sumr_g = sumr;
        if (sqrt(sumr_g) > eps) {
            while (sum_g > eps) {
                ite = ite + 1;
                bc_phi(P, p, nxs, nxe, l);
                sumr = 0.0;
                sum2 = 0.0;
#pragma omp parallel for reduction(+ : sumr, sum2)
                for (int j = nys; j <= nye; ++j)
                    for (int i = nxs; i <= nxe; ++i) {
                        AP(i, j) = -PP(i, j - 1) - PP(i - 1, j) + f4 * PP(i, j) - PP(i + 1, j) - PP(i, j + 1);
                        sumr = sumr + RR(i, j) * RR(i, j);
                        sum2 = sum2 + PP(i, j) * AP(i, j);
                    }
                sumr_g = sumr;
                av = sumr_g / sum2;
#pragma omp parallel for
                for (int j = nys; j <= nye; ++j)
                    for (int i = nxs; i <= nxe; ++i) {
                        PHI(i, j) = PHI(i, j) + av * PP(i, j);
                        RR(i, j) = RR(i, j) - av * AP(i, j);
                    }
                sum_g = sqrt(sumr_g);
                if (ite >= ite_max) {
                    status = WMO_ERR_CG_MAXITER;
                    break;
                }
                sum1 = 0.0;
#pragma omp parallel for reduction(+ : sum1)
                for (int j = nys; j <= nye; ++j)
                    for (int i = nxs; i <= nxe; ++i) sum1 = sum1 + RR(i, j) * RR(i, j);
                bv = sum1 / sumr_g;
#pragma omp parallel for
                for (int j = nys; j <= nye; ++j)
                    for (int i = nxs; i <= nxe; ++i) PP(i, j) = RR(i, j) + bv * PP(i, j);
            }
        }
        if (status == WMO_OK)
            for (int j = nys; j <= nye; ++j)
                for (int i = nxs; i <= nxe; ++i) DBL(l, i, j) = PHI(i, j);
        if (iters) iters[l - 1] = ite;
    }
#undef PHI
#undef PP
#undef RR
#undef BB
#undef AP
#undef GKL
    free(phi);
    free(p);
    free(r);
    free(b);
    free(ap);
    return status;
}

/* ------------------------------------------------------------- field update
 * field.f90:66-186 (field__fdtd_i) with the periodic boundary routines as its procedure
 * arguments.  df, gkl and uj are the routine's SAVE'd work arrays (field.f90:98): df(1:3)
 * carries the previous step's delta-B as the CG initial guess, so the caller keeps them.     */
int wmo_field_fdtd_i(const wmo_par *P, double *uf, const double *up, const double *gp, const int *cumcnt, int nxs, int nxe,
                     double *df, double *gkl, double *uj, int *iters)
{
    const int nys = P->nys, nye = P->nye;
    const double c = P->c, delt = P->delt, delx = P->delx, gfac = P->gfac;
    const double f1 = c * delt / delx;
    const double f2 = gfac * f1 * f1;
    const double f3 = 4.0 * PI * delx / c;
    const int gw = P->nxge - P->nxgs + 1;
#define GKL(l, i, j) gkl[(size_t)((l) - 1) + 3 * ((size_t)((i) - P->nxgs) + (size_t)gw * (size_t)((j) - nys))]

    wmo_ele_cur(P, uj, up, gp, cumcnt, nxs, nxe);
    wmo_bc_curre(P, uj, nxs, nxe);

#pragma omp parallel for
    for (int j = nys; j <= nye; ++j)
        for (int i = nxs; i <= nxe; ++i) {
            GKL(1, i, j) = +f2 * (+UF(1, i, j - 1) + UF(1, i - 1, j) - 4. * UF(1, i, j) + UF(1, i + 1, j) + UF(1, i, j + 1)
                                  + f3 * (-UJ(3, i, j - 1) + UJ(3, i, j)))
                           - f1 * (-UF(6, i, j - 1) + UF(6, i, j));
            GKL(2, i, j) = +f2 * (+UF(2, i, j - 1) + UF(2, i - 1, j) - 4. * UF(2, i, j) + UF(2, i + 1, j) + UF(2, i, j + 1)
                                  - f3 * (-UJ(3, i - 1, j) + UJ(3, i, j)))
                           + f1 * (-UF(6, i - 1, j) + UF(6, i, j));
            GKL(3, i, j) = +f2 * (+UF(3, i, j - 1) + UF(3, i - 1, j) - 4. * UF(3, i, j) + UF(3, i + 1, j) + UF(3, i, j + 1)
                                  + f3 * (-UJ(2, i - 1, j) + UJ(2, i, j) + UJ(1, i, j - 1) - UJ(1, i, j)))
                           - f1 * (-UF(5, i - 1, j) + UF(5, i, j) + UF(4, i, j - 1) - UF(4, i, j));
        }
#undef GKL

    const int st = wmo_cgm(P, df, gkl, nxs, nxe, iters);
    if (st != WMO_OK) return st;

    wmo_bc_dfield(P, df, nxs, nxe);

#pragma omp parallel for
    for (int j = nys; j <= nye; ++j)
        for (int i = nxs; i <= nxe; ++i) {
            DF(4, i, j) = +f1 * (+gfac * (-DF(3, i, j) + DF(3, i, j + 1)) + (-UF(3, i, j) + UF(3, i, j + 1))) - 4. * PI * delt * UJ(1, i, j);
            DF(5, i, j) = -f1 * (+gfac * (-DF(3, i, j) + DF(3, i + 1, j)) + (-UF(3, i, j) + UF(3, i + 1, j))) - 4. * PI * delt * UJ(2, i, j);
            DF(6, i, j) = +f1 * (+gfac * (-DF(2, i, j) + DF(2, i + 1, j) + DF(1, i, j) - DF(1, i, j + 1))
                                 + (-UF(2, i, j) + UF(2, i + 1, j) + UF(1, i, j) - UF(1, i, j + 1)))
                          - 4. * PI * delt * UJ(3, i, j);
        }

    wmo_bc_dfield(P, df, nxs, nxe);

#pragma omp parallel for
    for (int j = nys - 2; j <= nye + 2; ++j)
        for (int i = nxs - 2; i <= nxe + 2; ++i)
            for (int ieq = 1; ieq <= 6; ++ieq) UF(ieq, i, j) = UF(ieq, i, j) + DF(ieq, i, j);
    return WMO_OK;
}

/* ------------------------------------------------------ particle boundaries
 * boundary_periodic.f90:61-96.  The reference sets the rounding mode to downward on entry;
 * the Fortran IEEE rules restore the caller's mode on return, which fesetround mirrors here. */
void wmo_bc_particle_x(const wmo_par *P, double *up, const int *np2)
{
    const double delx = P->delx;
    for (int isp = 1; isp <= P->nsp; ++isp) {
        /* The rounding mode is per thread: every OpenMP thread switches to downward rounding,
         * which gives the single-thread semantics of the reference at any thread count. */
#pragma omp parallel
        {
            const int save = fegetround();
            fesetround(FE_DOWNWARD);
#pragma omp for
            for (int j = P->nys; j <= P->nye; ++j)
                for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                    volatile double x = UP(1, ii, j, isp);
                    const int ipos = (int)(x / delx);
                    if (ipos < P->nxgs)
                        UP(1, ii, j, isp) = x + (P->nxge - P->nxgs + 1) * delx;
                    else if (ipos >= P->nxge + 1)
                        UP(1, ii, j, isp) = x - (P->nxge - P->nxgs + 1) * delx;
                }
            fesetround(save);
        }
    }
}

/* Reflecting walls, boundary_reconnection.f90:61-99 (= boundary_shock.f90:62-100): a particle
 * in cell ipos < nxs+1 is mirrored about x = nxs+1, one in ipos >= nxe-1 about nxe-1, and its
 * momentum reversed.  `2.*(nxs+1)` is a default-real (FP32) product, exact here. */
void wmo_bc_particle_x_walls(const wmo_par *P, double *up, const int *np2, int nxs, int nxe)
{
    const double delx = P->delx;
    const double xl = (double)(2.0f * (float)(nxs + 1)) * delx, xr = (double)(2.0f * (float)(nxe - 1)) * delx;
    for (int isp = 1; isp <= P->nsp; ++isp)
#pragma omp parallel for
        for (int j = P->nys; j <= P->nye; ++j)
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                const int ipos = (int)(UP(1, ii, j, isp) / delx);
                if (ipos < nxs + 1 || ipos >= nxe - 1) {
                    UP(1, ii, j, isp) = (ipos < nxs + 1 ? xl : xr) - UP(1, ii, j, isp);
                    for (int k = 3; k <= 5; ++k) UP(k, ii, j, isp) = -UP(k, ii, j, isp);
                }
            }
}

/* boundary_shock.f90:255-297: reflecting wall at nxs+1 and the injection boundary
 * xend = nxe*delx + u0/sqrt(1+u0^2/c^2)*delt, where particles are mirrored into the inflow
 * (u_x -> 2 u0 - u_x). */
void wmo_bc_injection(const wmo_par *P, double *up, const int *np2, int nxs, int nxe, double u0)
{
    const double delx = P->delx, c = P->c;
    const double xend = nxe * delx + u0 / sqrt(1 + (u0 * u0) / (c * c)) * P->delt;
    const double xl = (double)(2.0f * (float)(nxs + 1)) * delx;
    for (int isp = 1; isp <= P->nsp; ++isp)
#pragma omp parallel for
        for (int j = P->nys; j <= P->nye; ++j)
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                const int ipos = (int)(UP(1, ii, j, isp) / delx);
                if (ipos < nxs + 1) {
                    UP(1, ii, j, isp) = xl - UP(1, ii, j, isp);
                    for (int k = 3; k <= 5; ++k) UP(k, ii, j, isp) = -UP(k, ii, j, isp);
                } else if (UP(1, ii, j, isp) > xend) {
                    UP(1, ii, j, isp) = 2.0 * xend - UP(1, ii, j, isp);
                    UP(3, ii, j, isp) = 2.0 * u0 - UP(3, ii, j, isp);
                    UP(4, ii, j, isp) = -UP(4, ii, j, isp);
                    UP(5, ii, j, isp) = -UP(5, ii, j, isp);
                }
            }
}

/* boundary_periodic.f90:99-248, single-thread semantics.  The reference sizes its exchange
 * buffers bff_ptcl(ndim*np, nys-1:nye+1); here each destination buffer is sized by a counting
 * pre-pass, which changes only the allocation, not the order in which particles are appended,
 * exchanged or used to fill holes.  Returns WMO_ERR_OVERFLOW where the reference stops on
 * np2 > np (:231-234).                                                                      */
int wmo_bc_particle_y(const wmo_par *P, double *up, int *np2)
{
    const int save = fegetround();
    fesetround(FE_DOWNWARD);
    const int nys = P->nys, nye = P->nye, ndim = P->ndim, nyl = NYL;
    const double delx = P->delx;
    int status = WMO_OK;
    /* rows nys-1..nye+1 -> index 0..nyl+1 */
    size_t *cap = (size_t *)calloc((size_t)nyl + 2, sizeof(size_t));
    size_t *boff = (size_t *)calloc((size_t)nyl + 3, sizeof(size_t));
    int *cnt = (int *)calloc((size_t)nyl + 2, sizeof(int));
    int *cnt2 = (int *)calloc((size_t)nyl, sizeof(int));
    size_t *foff = (size_t *)calloc((size_t)nyl + 1, sizeof(size_t));
    for (int isp = 1; isp <= P->nsp && status == WMO_OK; ++isp) {
        /* counting pre-pass (allocation only) */
        memset(cap, 0, sizeof(size_t) * (nyl + 2));
        for (int j = nys; j <= nye; ++j) {
            foff[j - nys + 1] = foff[j - nys];
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                volatile double y = UP(2, ii, j, isp);
                const int jpos = (int)(y / delx);
                if (jpos != j) {
                    cap[jpos - (nys - 1)]++;
                    foff[j - nys + 1]++;
                }
            }
        }
        {
            size_t cn = cap[nye - (nys - 1)], cs = cap[0], ce = cap[nyl + 1];
            cap[nye - (nys - 1)] = cn + cs;
            cap[nys - (nys - 1)] += ce;
        }
        boff[0] = 0;
        for (int k = 0; k < nyl + 2; ++k) boff[k + 1] = boff[k] + cap[k];
        double *bff = (double *)malloc(sizeof(double) * (size_t)ndim * (boff[nyl + 2] + 1));
        int *flag = (int *)malloc(sizeof(int) * (foff[nyl] + 1));
#define BFF(idx, k) bff[(size_t)(idx) + (size_t)ndim * boff[(k) - (nys - 1)]]   /* idx is 0-based element */
#define FLAG(n, j) flag[(size_t)((n) - 1) + foff[(j) - nys]]

        memset(cnt, 0, sizeof(int) * (nyl + 2));
        memset(cnt2, 0, sizeof(int) * nyl);
        /* scan (:143-168) */
        for (int j = nys; j <= nye; ++j)
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                volatile double y = UP(2, ii, j, isp);
                const int jpos = (int)(y / delx);
                if (jpos != j) {
                    if (jpos <= P->nygs - 1)
                        UP(2, ii, j, isp) = y + (P->nyge - P->nygs + 1) * delx;
                    else if (jpos >= P->nyge + 1)
                        UP(2, ii, j, isp) = y - (P->nyge - P->nygs + 1) * delx;
                    for (int idim = 1; idim <= ndim; ++idim) BFF(idim - 1 + ndim * cnt[jpos - (nys - 1)], jpos) = UP(idim, ii, j, isp);
                    cnt[jpos - (nys - 1)]++;
                    cnt2[j - nys]++;
                    FLAG(cnt2[j - nys], j) = ii;
                }
            }
        /* exchange with the rank itself (:173-189) */
        {
            int cnt_tmp = cnt[0];
            for (int e = 0; e < ndim * cnt_tmp; ++e) BFF(ndim * cnt[nye - (nys - 1)] + e, nye) = BFF(e, nys - 1);
            cnt[nye - (nys - 1)] += cnt_tmp;
            cnt_tmp = cnt[nyl + 1];
            for (int e = 0; e < ndim * cnt_tmp; ++e) BFF(ndim * cnt[nys - (nys - 1)] + e, nys) = BFF(e, nye + 1);
            cnt[nys - (nys - 1)] += cnt_tmp;
        }
        /* fill holes (:193-225) */
        for (int j = nys; j <= nye; ++j) {
            int iii = 0, cnt_tmp = cnt2[j - nys];
            int *cj = &cnt[j - (nys - 1)];
            int *npj = &NP2(j, isp);
            for (int ii = 1; ii <= cnt2[j - nys]; ++ii) {
                if (*cj == 0) {
                    if (*npj < FLAG(ii, j)) goto exit_loop1;
                    while (*npj == FLAG(cnt_tmp, j)) {
                        *npj = *npj - 1;
                        if (*npj < FLAG(ii, j)) goto exit_loop1;
                        cnt_tmp = cnt_tmp - 1;
                    }
                    for (int idim = 1; idim <= ndim; ++idim) UP(idim, FLAG(ii, j), j, isp) = UP(idim, *npj, j, isp);
                    *npj = *npj - 1;
                } else {
                    for (int idim = 1; idim <= ndim; ++idim) UP(idim, FLAG(ii, j), j, isp) = BFF(idim - 1 + ndim * iii, j);
                    iii = iii + 1;
                    *cj = *cj - 1;
                }
            }
        exit_loop1:
            if (*cj > 0) {
                if (*npj + *cj > P->np) {
                    status = WMO_ERR_OVERFLOW;
                    break;
                }
                for (int ii = 1; ii <= *cj; ++ii)
                    for (int idim = 1; idim <= ndim; ++idim) UP(idim, *npj + ii, j, isp) = BFF(ndim * iii + idim - 1 + ndim * (ii - 1), j);
            }
        }
        if (status == WMO_OK)
            for (int j = nys; j <= nye; ++j) {
                NP2(j, isp) = NP2(j, isp) + cnt[j - (nys - 1)];
                if (NP2(j, isp) > P->np) status = WMO_ERR_OVERFLOW;
            }
#undef BFF
#undef FLAG
        free(bff);
        free(flag);
    }
    free(cap);
    free(boff);
    free(cnt);
    free(cnt2);
    free(foff);
    fesetround(save);
    return status;
}

/* ------------------------------------------------------------ counting sort
 * sort.f90:36-82 (sort__bucket(gp, up, ...): gp is the output).  The cell of a particle is
 * int(x) with no division by delx (:60,72).  Returns WMO_ERR_CELL for a particle outside
 * nxs..nxe, where the reference would index out of bounds.                                 */
int wmo_sort_bucket(const wmo_par *P, double *gp, const double *up, int *cumcnt, const int *np2, int nxs, int nxe)
{
    int status = WMO_OK;
    const int ndim = P->ndim;
    for (int isp = 1; isp <= P->nsp; ++isp) {
#pragma omp parallel for
        for (int j = P->nys; j <= P->nye; ++j) {
            int *cnt = (int *)calloc((size_t)(nxe - nxs + 1), sizeof(int));
            int *sum_cnt = (int *)calloc((size_t)(nxe - nxs + 2), sizeof(int));
            int bad = 0;
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                const int i = (int)UP(1, ii, j, isp);
                if (i < nxs || i > nxe) {
                    bad = 1;
                    break;
                }
                cnt[i - nxs] = cnt[i - nxs] + 1;
            }
            if (!bad) {
                sum_cnt[0] = 0;
                CUMCNT(nxs, j, isp) = 0;
                for (int i = nxs + 1; i <= nxe + 1; ++i) {
                    sum_cnt[i - nxs] = sum_cnt[i - 1 - nxs] + cnt[i - 1 - nxs];
                    CUMCNT(i, j, isp) = sum_cnt[i - nxs];
                }
                for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                    const int i = (int)UP(1, ii, j, isp);
                    for (int k = 1; k <= ndim; ++k) GP(k, sum_cnt[i - nxs] + 1, j, isp) = UP(k, ii, j, isp);
                    sum_cnt[i - nxs] = sum_cnt[i - nxs] + 1;
                }
            } else {
#pragma omp atomic write
                status = WMO_ERR_CELL;
            }
            free(cnt);
            free(sum_cnt);
        }
    }
    return status;
}

/* ------------------------------------------------------------------- moments
 * mom_calc.f90:167-249 (mom_calc__nvt): CIC deposit of N, V(3), T-diagonal(3).            */
void wmo_mom_nvt(const wmo_par *P, double *mom, const double *up, const int *np2)
{
    const double d_delx = 1. / P->delx, c = P->c;
    const size_t momlen = (size_t)7 * (size_t)(P->nxge - P->nxgs + 3) * (size_t)(NYL + 2) * (size_t)P->nsp;
    memset(mom, 0, sizeof(double) * momlen);
    for (int isp = 1; isp <= P->nsp; ++isp) {
#pragma omp parallel for reduction(+ : mom[0 : momlen])
        for (int j = P->nys; j <= P->nye; ++j)
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                const double u3 = UP(3, ii, j, isp), u4 = UP(4, ii, j, isp), u5 = UP(5, ii, j, isp);
                const int ih = (int)(UP(1, ii, j, isp) * d_delx - 0.5);
                const int jh = (int)(UP(2, ii, j, isp) * d_delx - 0.5);
                const double dx = UP(1, ii, j, isp) * d_delx - 0.5 - ih;
                const double dxm = 1. - dx;
                const double dy = UP(2, ii, j, isp) * d_delx - 0.5 - jh;
                const double dym = 1. - dy;
                const double gam = 1. / sqrt(1.0 + (+u3 * u3 + u4 * u4 + u5 * u5) / (c * c));
                MOM(1, ih, jh, isp) = MOM(1, ih, jh, isp) + dxm * dym;
                MOM(1, ih + 1, jh, isp) = MOM(1, ih + 1, jh, isp) + dx * dym;
                MOM(1, ih, jh + 1, isp) = MOM(1, ih, jh + 1, isp) + dxm * dy;
                MOM(1, ih + 1, jh + 1, isp) = MOM(1, ih + 1, jh + 1, isp) + dx * dy;
#define MV(k, v)                                                                         \
    MOM(k, ih, jh, isp) = MOM(k, ih, jh, isp) + (v) * gam * dxm * dym;                   \
    MOM(k, ih + 1, jh, isp) = MOM(k, ih + 1, jh, isp) + (v) * gam * dx * dym;            \
    MOM(k, ih, jh + 1, isp) = MOM(k, ih, jh + 1, isp) + (v) * gam * dxm * dy;            \
    MOM(k, ih + 1, jh + 1, isp) = MOM(k, ih + 1, jh + 1, isp) + (v) * gam * dx * dy;
                MV(2, u3)
                MV(3, u4)
                MV(4, u5)
                MV(5, u3 * u3)
                MV(6, u4 * u4)
                MV(7, u5 * u5)
#undef MV
            }
    }
}

/* boundary_periodic.f90:571-636 (ghost fold of the moments, one rank) */
void wmo_bc_mom(const wmo_par *P, double *mom)
{
    const int nxgs = P->nxgs, nxge = P->nxge, nys = P->nys, nye = P->nye;
    const int walls = P->bc != WMO_BC_PERIODIC;  /* boundary_reconnection.f90:590-593: fold onto the own edge */
    for (int isp = 1; isp <= P->nsp; ++isp)
        for (int j = nys - 1; j <= nye + 1; ++j)
            for (int k = 1; k <= 7; ++k) {
                MOM(k, nxgs, j, isp) = MOM(k, nxgs, j, isp) + MOM(k, walls ? nxgs - 1 : nxge + 1, j, isp);
                MOM(k, nxge, j, isp) = MOM(k, nxge, j, isp) + MOM(k, walls ? nxge + 1 : nxgs - 1, j, isp);
            }
    for (int isp = 1; isp <= P->nsp; ++isp) {
        for (int i = nxgs - 1; i <= nxge + 1; ++i)
            for (int k = 1; k <= 7; ++k) MOM(k, i, nye, isp) = MOM(k, i, nye, isp) + MOM(k, i, nys - 1, isp);
        for (int i = nxgs - 1; i <= nxge + 1; ++i)
            for (int k = 1; k <= 7; ++k) MOM(k, i, nys, isp) = MOM(k, i, nys, isp) + MOM(k, i, nye + 1, isp);
    }
}

/* proj/weibel/app.f90:479-545 (energy_history, one rank): out = {KE_1..KE_nsp, E/8pi, B/8pi} */
void wmo_energy(const wmo_par *P, double *out, const double *up, const double *uf, const int *np2)
{
    const double c = P->c;
    double efield = 0, bfield = 0;
    for (int isp = 1; isp <= P->nsp; ++isp) {
        double vene = 0;
#pragma omp parallel for reduction(+ : vene)
        for (int j = P->nys; j <= P->nye; ++j)
            for (int ii = 1; ii <= NP2(j, isp); ++ii) {
                const double u2 = UP(3, ii, j, isp) * UP(3, ii, j, isp) + UP(4, ii, j, isp) * UP(4, ii, j, isp) + UP(5, ii, j, isp) * UP(5, ii, j, isp);
                const double gam = sqrt(1 + u2 / (c * c));
                vene = vene + P->r[isp - 1] * (gam - 1);
            }
        out[isp - 1] = vene;
    }
#pragma omp parallel for reduction(+ : bfield, efield)
    for (int j = P->nys; j <= P->nye; ++j)
        for (int i = P->nxgs; i <= P->nxge; ++i) {
            bfield = bfield + UF(1, i, j) * UF(1, i, j) + UF(2, i, j) * UF(2, i, j) + UF(3, i, j) * UF(3, i, j);
            efield = efield + UF(4, i, j) * UF(4, i, j) + UF(5, i, j) * UF(5, i, j) + UF(6, i, j) * UF(6, i, j);
        }
    out[P->nsp] = efield / (8 * PI);
    out[P->nsp + 1] = bfield / (8 * PI);
}

/* One pass of the main loop body, proj/weibel/app.f90:102-107. */
int wmo_step(const wmo_par *P, double *up, double *gp, double *uf, int *cumcnt, int *np2, int nxs, int nxe, double *df, double *gkl,
             double *uj, int *iters)
{
    int st;
    wmo_particle_solv(P, gp, up, uf, cumcnt, nxs, nxe);
    if (P->bc == WMO_BC_SHOCK)  /* proj/shock/app.f90:112-117: injection boundary before the field solve */
        wmo_bc_injection(P, gp, np2, nxs, nxe, P->u0);
    if ((st = wmo_field_fdtd_i(P, uf, up, gp, cumcnt, nxs, nxe, df, gkl, uj, iters)) != WMO_OK) return st;
    if (P->bc == WMO_BC_PERIODIC)
        wmo_bc_particle_x(P, gp, np2);
    else if (P->bc == WMO_BC_RECONNECTION)  /* proj/reconnection/app.f90:101-106 */
        wmo_bc_particle_x_walls(P, gp, np2, nxs, nxe);
    if ((st = wmo_bc_particle_y(P, gp, np2)) != WMO_OK) return st;
    return wmo_sort_bucket(P, up, gp, cumcnt, np2, nxs, nxe);
}

int wmo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void wmo_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
