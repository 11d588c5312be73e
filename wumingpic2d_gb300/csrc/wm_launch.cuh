// wm_launch.cuh -- host launchers exported by the kernel translation units.
#pragma once
#include <cuda.h>  // CUtensorMap (TMA descriptors)

#include "wm_internal.cuh"

// wm_particles.cu
template <class PV, class FV>
int wm_launch_push(const WmGeom &g, const WmConst &k, PV up, PV gp, FV uf, const int *cumcnt, int half_step, int copy_pid,
                   cudaStream_t st);
int wm_launch_pid_copy_aos(double *gp, const double *up, long long nslots, cudaStream_t st);
template <class PV>
int wm_launch_deposit_cells(const WmGeom &g, const WmConst &k, PV up, PV gp, const int *cumcnt, double *pjcell,
                            unsigned *status, cudaStream_t st);
template <class FV3>
int wm_launch_deposit_fold(const WmGeom &g, FV3 uj, const double *pjcell, cudaStream_t st);
template <class PV>
int wm_launch_mom_nvt(const WmGeom &g, const WmConst &k, PV up, const int *np2, double *mom, int max_row_count,
                      cudaStream_t st);
template <class PV>
int wm_launch_energy_particles(const WmGeom &g, const WmConst &k, PV up, const int *np2, double *partial, int nblocks,
                               cudaStream_t st);

// wm_rebin.cu
// particle_x of the walls (inject = 0) or the shock's injection boundary (inject = 1) over the
// first np2[row] particles of every row; x range nxgs..nxge.
template <class PV>
int wm_launch_walls_x(const WmGeom &g, const WmConst &k, PV v, const int *np2, int max_row_count, int inject, double u0,
                      cudaStream_t st);
template <class PV>
int wm_launch_wrap_classify(const WmGeom &g, double delx, PV v, const int *np2, int max_row_count, int mode,
                            const WmRebinScratch &sc, cudaStream_t st);
template <class PV>
int wm_launch_place(const WmGeom &g, PV v, const int *np2, int max_row_count, const WmRebinScratch &sc, int *drow,
                    cudaStream_t st);
int wm_launch_np2_after_y(const WmGeom &g, const int *np2, const WmRebinScratch &sc, int *np2_new, int np_limit,
                          cudaStream_t st);
template <class PV>
int wm_launch_scatter_by_P(const WmGeom &g, PV src, PV dst, const int *np2, int max_row_count, const WmRebinScratch &sc,
                           const int *drow, int np_limit, cudaStream_t st);
template <class PV>
int wm_launch_slot_as_P(const WmGeom &g, PV v, const int *np2, int max_row_count, const WmRebinScratch &sc, cudaStream_t st);
int wm_launch_scan_cells(const WmGeom &g, const WmRebinScratch &sc, int *cumcnt, int *np2_out, cudaStream_t st);
int wm_launch_rowbase(int nrows, const int *np2, long long *rowbase, cudaStream_t st);
template <class PV>
int wm_launch_place_sort(const WmGeom &g, PV src, PV dst, const int *np2, int max_row_count, const int *cumcnt,
                         const WmRebinScratch &sc, cudaStream_t st);
template <class PV>
int wm_launch_sort_move(const WmGeom &g, PV src, PV dst, const int *src_np2, int max_row_count, const int *cumcnt,
                        const WmRebinScratch &sc, cudaStream_t st);

// wm_field.cu
struct CgScal;
struct WmFieldWork {
    double *b, *r, *p, *ap;
    double *partial;
    unsigned *ticket;
    CgScal *scal;
    CgScal *scal_host;
};
typedef void (*wm_mark_fn)(void *ctx, const char *name);
int wm_field_cg_blocks();
size_t wm_field_scal_bytes();
template <class FV>
int wm_launch_curre_bc(const WmGeom &g, FV uj, cudaStream_t st);
template <class FV>
int wm_launch_dfield_bc(const WmGeom &g, FV df, cudaStream_t st);
int wm_launch_phi_bc(int nx, int ny, double *phi, int bc, int l, cudaStream_t st);
int wm_launch_mom_bc(const WmGeom &g, double *mom, cudaStream_t st);
int wm_launch_aos_to_soa(int nc, long long npts, const double *a, double *s, cudaStream_t st);
int wm_launch_soa_to_aos(int nc, long long npts, const double *s, double *a, cudaStream_t st);
// Optional initial guess for the CG: run() writes cand ([3][nx*ny], x fastest) from uf and the
// folded uj; the solve then starts each component from whichever of cand and the previous dB has
// the smaller residual.  stats (device, 12 doubles): |b - A cand|^2 [3], |b - A dB_prev|^2 [3],
// 1.0 where cand was taken [3], |b|^2 [3].
struct WmGuess {
    int (*run)(void *ctx, cudaStream_t st);
    void *ctx;
    double *cand;
    double *stats;
};
int wm_field_solve(const WmGeom &g, const WmConst &k, FView<6, false> uf, FView<3, false> uj, FView<6, false> df, WmFieldWork &w,
                   int *iters, int cg_batch, cudaStream_t st, wm_mark_fn mark, void *mctx, long long *launches,
                   const WmGuess *guess = nullptr);
int wm_launch_energy_fields(const WmGeom &g, FView<6, false> uf, double *partial, int nblocks, cudaStream_t st);
int wm_launch_sum_partials(const double *partial, int nparts, int nsets, double *out, cudaStream_t st);

// wm_mixed.cu
int wm_mixed_ntiles(const WmGeom &g);
size_t wm_mixed_jtile_floats(const WmGeom &g);
size_t wm_mixed_fcc_floats(const WmGeom &g);
int wm_launch_mixed_fields(const WmGeom &g, FView<6, false> uf, float *fcc, cudaStream_t st);
// sc.key receives each particle's move code (rank << 10 | tile cell << 4 | direction), cnt9
// [cells][9] the per-cell direction counts; k_mixed_incoming turns them into destination counts
// (sc.cellcnt) and offsets off9 [cells][9]; k_mixed_move writes the new cell-sorted order, or
// k_mixed_perm records it as a slot permutation that the next push reads through (perm != null:
// the particle of slot p is at slot perm[p] of a; the push leaves the ids alone, and k_mixed_perm
// composes the permutation of the id array, idperm, instead).
// ovf: 1 + (tiles of the grid) u32 of scratch for the list of tiles whose queue of cell-changing
// particles overflowed (wm_mixed_ovf_words); those tiles are recomputed by a second launch.
int wm_launch_mixed_push_deposit(const WmGeom &g, const WmConst &k, MixedView a, MixedView b, const unsigned *perm, const float *fcc,
                                 const int *cumcnt, const WmRebinScratch &sc, int *cnt9, float *jtile, unsigned *ovf, cudaStream_t st);
size_t wm_mixed_ovf_words(const WmGeom &g);
int wm_launch_mixed_incoming(const WmGeom &g, const int *cnt9, int *off9, const WmRebinScratch &sc, cudaStream_t st);
int wm_launch_mixed_move(const WmGeom &g, MixedView src, MixedView dst, const int *cumcnt_old, const int *cumcnt_new, const int *off9,
                         const WmRebinScratch &sc, cudaStream_t st);
// perm[q] = p and idperm_new[q] = idperm_old[p] (idperm_old = null: p) for the push output slot p
// that lands on slot q of the new order
int wm_launch_mixed_perm(const WmGeom &g, const long long *rowbase_src, const long long *rowbase_dst, const int *cumcnt_old,
                         const int *cumcnt_new, const int *off9, const WmRebinScratch &sc, unsigned *perm, const unsigned *idperm_old,
                         unsigned *idperm_new, cudaStream_t st);
// dst slot p <- src slot perm[p] over the np2 slots of every row, the id from src slot idperm[p]
int wm_launch_mixed_gather(const WmGeom &g, MixedView src, MixedView dst, const unsigned *perm, const unsigned *idperm, const int *np2, int max_row,
                           cudaStream_t st);
int wm_launch_mixed_jfold(const WmGeom &g, const float *jtile, FView<3, false> uj, cudaStream_t st);
// rows row0 .. row0+nrows-1 of the stage (nrows < 0: to the last row)
int wm_launch_mixed_unpack(const WmGeom &g, const double *stage, int pitch, const int *np2, MixedView dst, const WmRebinScratch &sc,
                           cudaStream_t st, int row0 = 0, int nrows = -1);
// mixed set -> reference-layout rows: pitch slots written per row (slots past np2 zero), rows
// rstride slots apart (rstride < 0: pitch); with perm/idperm, the permuted state read through them
int wm_launch_mixed_pack(const WmGeom &g, MixedView src, const int *np2, const int *cumcnt, int pitch, double *stage, cudaStream_t st,
                         int row0 = 0, int nrows = -1, long long rstride = -1, const unsigned *perm = nullptr,
                         const unsigned *idperm = nullptr);

// wm_cnn.cu: the learned-guess network inside the solve (layer shapes are padded channel counts)
constexpr int WM_CNN_LAYERS = 6;
constexpr int wm_cnn_cin[WM_CNN_LAYERS] = {16, 48, 48, 48, 48, 48};
constexpr int wm_cnn_cout[WM_CNN_LAYERS] = {48, 48, 48, 48, 48, 8};
constexpr int WM_CNN_RED_BLOCKS = 1024;
struct WmCnnNet {
    float *params;  // FP32, per layer w[9][cout][cin] then b[cout]
    void *wf[WM_CNN_LAYERS];
    const float *bias[WM_CNN_LAYERS];
};
struct WmCnnWork {
    void *x, *a0, *a1;  // BF16 [ny][nx][16], [ny][nx][48] x 2
    float *pred;        // FP32 [ny][nx][8]
    double *partial;    // 3 * WM_CNN_RED_BLOCKS
    double *scale;      // 6
};
size_t wm_cnn_param_count();
int wm_cnn_net_prepare(WmCnnNet &net, cudaStream_t st);
int wm_cnn_infer_guess(const WmGeom &g, const WmCnnNet &net, FView<6, false> uf, FView<3, false> uj, const WmCnnWork &w, double *cand,
                       cudaStream_t st,
                       unsigned *status);
// A tiled TMA descriptor (no interleave, no swizzle, zero fill out of bounds): dims and box
// innermost first, strides in bytes of dims 1 .. rank-1.
int wm_tensor_map(CUtensorMap *map, CUtensorMapDataType type, int rank, const void *base, const unsigned long long *dims,
                  const unsigned long long *strides, const unsigned *box);
// wm_cnn_tc.cu: the convolutions on tcgen05 (h a multiple of 16, w of 8): (cin, cout) = (16, 48) or
// (48, 48) with mode WM_CNN_FWD_TRAIN / _INFER / _BWD (zprev), (48, 8) with WM_CNN_FWD_LINEAR; a
// timed-out wait sets WMDEV_TIMEOUT in *status
bool wm_cnn_tc_shape_ok(int nimg, int H, int W);
int wm_cnn_conv3x3_tc(const void *in, const void *w, const float *bias, int cin, int cout, int mode, int nimg, int h, int wd, void *out,
                      void *zout, const void *zprev, unsigned *status, cudaStream_t st);
// the weight gradient on tcgen05, (cin, coutp) = (16, 48), (48, 48), (48, 16): per-CTA partials
// [cta][9][coutp][cin] + [coutp] into part (*nparts CTAs, at most the SM count), summed by the caller
int wm_cnn_wgrad_tc(const void *x, const void *dz, int cin, int coutp, bool grouped, int nimg, int h, int wd, float *part, long long part_floats,
                    int *nparts, unsigned *status, cudaStream_t st);

// wm_paraio.cu: the resident state in the order of the paraio files
int wm_launch_mom_file(const WmGeom &g, const double *mom, FView<6, false> uf, double *out, cudaStream_t st);
int wm_launch_uf_interior(const WmGeom &g, FView<6, false> uf, double *out, cudaStream_t st);
int wm_launch_row_count(int nrows, const double *stage, int pitch, const int *np2, int mode, long long *cnt, cudaStream_t st);
int wm_launch_row_compact(int nrows, const double *stage, int pitch, const int *np2, int mode, const long long *off, double *out,
                          cudaStream_t st);

// wm_init.cu: seeded initial conditions on the GPU (generator tags in wm_rng.cuh)
#define WM_PI 3.14159265358979311599796346854418516
struct WmInitArgs {
    unsigned tag;           // WM_RNG_WEIBEL, _HARRIS or _SHOCK
    int n_row;              // particles per row and species
    unsigned long long seed;
    double delx, c;
    double vth_e, vth_i;
    double ud;              // weibel: beam four-velocity
    int ibg;                // harris: background particles per row
    double lcs, x0, y0, tanh_edge, b0, e1, ncs, nbg, f1, f2;   // harris
    double v0, l_damp_ini, nxgs_delx, xrs, xre, bx, by, bz;   // shock
};
int wm_launch_init_particles(const WmGeom &g, const WmInitArgs &a, double *stage, cudaStream_t st);
int wm_launch_init_fields(const WmGeom &g, const WmInitArgs &a, FView<6, false> uf, cudaStream_t st);

// wm_init.cu: particle injection of the shock application (proj/shock/app.f90:695-850)
struct WmInjectArgs {
    unsigned long long seed;
    int it;                    // step number (the draws' counter)
    double pflux;              // n0 |v0| dt dx ny: particles per step and species
    double x0;                 // |v0| dt
    double xe;                 // nxe dx
    double v0, delt, c, delx, vth_e, vth_i, l_damp_ini, nxgs_delx;
    int cell;                  // interior cell the new particles are counted in (nxe-1)
    long long cap;             // particle capacity of the sets
    double by0, bz0;           // upstream field
    int n_expand;              // particles per row and species the box's expansion adds this step (0: none)
};
constexpr int WM_INJECT_MAX_ROWS = 12288;
// counts per row (inj[ny]), their exclusive prefix (ninc[ny]) and the species totals before the
// injection (nptot[2]); reads the new row counts np2
int wm_launch_inject_counts(const WmGeom &g, const WmInjectArgs &a, const int *np2, int *inj, long long *ninc, long long *nptot,
                            unsigned *status, cudaStream_t st);
// tmp[row] = np2[row] + inj[row % ny] + a.n_expand: row counts with room for the new particles
int wm_launch_inject_reserve(const WmGeom &g, const WmInjectArgs &a, const int *np2, const int *inj, int *tmp, cudaStream_t st);
// write the new particles behind each row's sorted ones, then np2 += inj, cumcnt(nxe), total += inj;
// with perm (a permuted mixed state): the particles go to fresh slots from *phys0 on and perm /
// idperm of their cell-sorted slots point there
template <class PV>
int wm_launch_inject_particles(const WmGeom &g, const WmInjectArgs &a, PV dst, int *np2, int *cumcnt, const int *inj,
                               const long long *ninc, const long long *nptot, cudaStream_t st, unsigned *perm = nullptr,
                               unsigned *idperm = nullptr, const long long *phys0 = nullptr);
int wm_launch_inject_fields(const WmGeom &g, const WmInjectArgs &a, FView<6, false> uf, cudaStream_t st);
// the box's expansion (relocate): a.n_expand particles per row and species in the cell after
// a.cell, behind the rows' particles (after the injection's), np2 and cumcnt advanced; the caller
// then moves nxe on (g.nxa, a.cell, a.xe) and sets the boundary columns (wm_launch_inject_fields)
template <class PV>
int wm_launch_expand_particles(const WmGeom &g, const WmInjectArgs &a, PV dst, int *np2, int *cumcnt, const int *inj, const long long *ninc,
                               const long long *nptot, cudaStream_t st, unsigned *perm = nullptr, unsigned *idperm = nullptr,
                               const long long *phys0 = nullptr);
