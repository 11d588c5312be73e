/*
 * wumingpic2d.h -- C ABI of the GB300 implementation of the WumingPIC2D time step.
 *
 * Two layers:
 *
 * 1. Module-procedure mirror.  One entry point per public procedure of the reference's
 *    common/ modules, with the same arguments in the same order.  Arrays are host pointers in the
 *    reference's Fortran layout (column-major, first element of each custom-bounded array):
 *        up, gp  (ndim, np, nys:nye, nsp)     uf, df (6, nxgs-2:nxge+2, nys-2:nye+2)
 *        uj      (3, nxgs-2:nxge+2, nys-2:nye+2)
 *        cumcnt  (nxgs:nxge+1, nys:nye, nsp)  np2 (nys:nye, nsp)   [int32]
 *        mom     (7, nxgs-1:nxge+1, nys-1:nye+1, nsp)
 *        phi     (nxs-1:nxe+1, nys-1:nye+1)
 *    Like the Fortran modules, each *_init stores its arguments as module state; the SAVE'd work
 *    arrays of field__fdtd_i (df, uj, gkl) live on the GPU between calls.  Each call copies its
 *    array arguments to the GPU, runs the hand-written sm_103a kernels and copies the results
 *    back; elements the reference routine does not write keep their values.  MPI arguments
 *    (mnpi, mnpr, ncomw, opsum, nerr, nstat, nup, ndown) are accepted and ignored: one process
 *    owns the whole periodic domain (nys = nygs, nye = nyge).  The x range arguments take
 *    nxs = nxgs and nxe = nxge, or, under the shock's boundary module, a smaller nxe (its growing
 *    box, proj/shock/app.f90:277 and relocate :613-690): the procedures then work over nxs..nxe as
 *    the Fortran does (cells, cumcnt(nxs:nxe+1), the field solve and ghosts at nxe+1, phi sized by
 *    nxe) and leave the rest of the arrays as they are.  A Fortran application binds these
 *    through ISO_C_BINDING; where the reference calls `stop`, these return a nonzero status.
 *
 * 2. Resident simulation (wm_sim_*).  Particles and fields stay on the GPU across steps in a
 *    compact structure-of-arrays layout sorted by (species, row, cell); host arrays in the
 *    reference layout are read at load and written at store.  wm_sim_step runs the main-loop
 *    body of proj/weibel/app.f90:102-107 (particle__solv, field__fdtd_i, bc__particle_x,
 *    bc__particle_y, sort__bucket), or the reconnection / shock applications' bodies (their wall
 *    modules; the shock's injection and expanding box).
 *
 * Every function returns WM_OK (0) or one of the WM_ERR_* codes; wm_status_string names them.
 */
#ifndef WUMINGPIC2D_H
#define WUMINGPIC2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    WM_OK = 0,
    WM_ERR_CG_MAXITER = 1,   /* CG reached ite_max (field.f90:427-430 stops the program there)   */
    WM_ERR_OVERFLOW = 2,     /* a row needs more than np slots (boundary_periodic.f90:231-234)     */
    WM_ERR_BAD_ARG = 3,      /* unsupported or inconsistent argument                               */
    WM_ERR_CELL = 4,         /* a particle outside nxs..nxe, or moved more than one row in a step  */
    WM_ERR_CUDA = 5,         /* a CUDA runtime call failed                                         */
    WM_ERR_NOT_INIT = 6,     /* *_init was not called first (the reference stops there)           */
    WM_ERR_UNSUPPORTED = 7,  /* option outside the supported single-GPU path                       */
    WM_ERR_IO = 8            /* a snapshot/output file could not be opened, written or read, or its
                                contents do not match the module parameters (paraio.f90 stops)   */
};

enum { WM_PREC_FP64 = 0, WM_PREC_MIXED = 1 };
/* Boundary module of the application (x direction; y is periodic in all three):
 * common/boundary_periodic.f90 (Weibel), proj/reconnection/boundary_reconnection.f90 (conducting,
 * reflecting walls at both x ends), proj/shock/boundary_shock.f90 (reflecting wall at nxs,
 * injection boundary at nxe). */
enum { WM_BC_PERIODIC = 0, WM_BC_RECONNECTION = 1, WM_BC_SHOCK = 2 };

/* ---------------------------------------------------------------- particle.f90 */
/* particle__init, common/particle.f90:18-45 */
int wm_particle_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, double delx,
                     double delt, double c, const double *q, const double *r);
/* particle__solv(gp, up, uf, cumcnt, nxs, nxe), common/particle.f90:48-177 */
int wm_particle_solv(double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe);

/* ------------------------------------------------------------------- field.f90 */
/* field__init, common/field.f90:22-63 */
int wm_field_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int mnpr, int ncomw,
                  int opsum, int nerr, double delx, double delt, double c, const double *q, const double *r, double gfac);
/* field__fdtd_i(uf, up, gp, cumcnt, nxs, nxe, bc_dfield, bc_curre, bc_phi), common/field.f90:66-186.
 * The three procedure arguments are the boundary routines of the module whose *_init ran last
 * (boundary_periodic here); the device applies that boundary kind. */
int wm_field_fdtd_i(double *uf, const double *up, const double *gp, const int *cumcnt, int nxs, int nxe);

/* -------------------------------------------------------------------- sort.f90 */
/* sort__init, common/sort.f90:16-33 */
int wm_sort_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye);
/* sort__bucket(gp, up, cumcnt, np2, nxs, nxe), common/sort.f90:36-82: gp is the output */
int wm_sort_bucket(double *gp, const double *up, int *cumcnt, const int *np2, int nxs, int nxe);

/* ---------------------------------------------------------------- mom_calc.f90 */
/* mom_calc__init, common/mom_calc.f90:18-45 */
int wm_mom_calc_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, double delx,
                     double delt, double c, const double *q, const double *r);
/* mom_calc__accl(gp, up, uf, cumcnt, nxs, nxe), common/mom_calc.f90:48-164 */
int wm_mom_calc_accl(double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe);
/* mom_calc__nvt(mom, up, np2), common/mom_calc.f90:167-249 */
int wm_mom_calc_nvt(double *mom, const double *up, const int *np2);

/* ------------------------------------------------------- boundary_periodic.f90 */
/* boundary_periodic__init, common/boundary_periodic.f90:26-58 */
int wm_bc_periodic_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nup,
                        int ndown, int mnpi, int mnpr, int ncomw, int nerr, const int *nstat, int nstat_len, double delx,
                        double delt, double c);
/* boundary_periodic__particle_x(up, np2), :61-96 */
int wm_bc_periodic_particle_x(double *up, const int *np2);
/* boundary_periodic__particle_y(up, np2), :99-248 */
int wm_bc_periodic_particle_y(double *up, int *np2);
/* boundary_periodic__dfield(df, nxs, nxe, nys, nye, nxgs, nxge), :251-354 */
int wm_bc_periodic_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge);
/* boundary_periodic__curre(uj, nxs, nxe, nys, nye, nxgs, nxge), :357-508 */
int wm_bc_periodic_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge);
/* boundary_periodic__phi(phi, nxs, nxe, nys, nye, l), :511-568 */
int wm_bc_periodic_phi(double *phi, int nxs, int nxe, int nys, int nye, int l);
/* boundary_periodic__mom(mom), :571-636 */
int wm_bc_periodic_mom(double *mom);

/* ------------------------------------------- proj/reconnection/boundary_reconnection.f90 */
/* boundary_reconnection__init, :26-58 (same arguments as boundary_periodic__init) */
int wm_bc_reconnection_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nup,
                            int ndown, int mnpi, int mnpr, int ncomw, int nerr, const int *nstat, int nstat_len, double delx,
                            double delt, double c);
/* boundary_reconnection__particle_x(up, np2, nxs, nxe), :61-99: reflecting walls */
int wm_bc_reconnection_particle_x(double *up, const int *np2, int nxs, int nxe);
/* boundary_reconnection__particle_y(up, np2), :102-251 */
int wm_bc_reconnection_particle_y(double *up, int *np2);
/* boundary_reconnection__dfield(df, nxs, nxe, nys, nye, nxgs, nxge), :254-361: conducting walls */
int wm_bc_reconnection_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge);
/* boundary_reconnection__curre(uj, nxs, nxe, nys, nye, nxgs, nxge), :364-502: y fold only */
int wm_bc_reconnection_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge);
/* boundary_reconnection__phi(phi, nxs, nxe, nys, nye, l), :505-579 */
int wm_bc_reconnection_phi(double *phi, int nxs, int nxe, int nys, int nye, int l);
/* boundary_reconnection__mom(mom), :582-647 */
int wm_bc_reconnection_mom(double *mom);

/* ------------------------------------------------------- proj/shock/boundary_shock.f90 */
/* boundary_shock__init, :27-59 */
int wm_bc_shock_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nup, int ndown,
                     int mnpi, int mnpr, int ncomw, int nerr, const int *nstat, int nstat_len, double delx, double delt, double c);
/* boundary_shock__particle_x(up, np2, nxs, nxe), :62-100 */
int wm_bc_shock_particle_x(double *up, const int *np2, int nxs, int nxe);
/* boundary_shock__particle_y(up, np2), :103-252 */
int wm_bc_shock_particle_y(double *up, int *np2);
/* boundary_shock__injection(up, np2, nxs, nxe, u0), :255-297 */
int wm_bc_shock_injection(double *up, const int *np2, int nxs, int nxe, double u0);
/* boundary_shock__dfield, :300-407; __curre, :410-548; __phi, :551-625; __mom, :628-693 */
int wm_bc_shock_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge);
int wm_bc_shock_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge);
int wm_bc_shock_phi(double *phi, int nxs, int nxe, int nys, int nye, int l);
int wm_bc_shock_mom(double *mom);
/* field__fdtd_i uses the boundary procedures of the module whose *_init ran last.  The walls'
 * procedures support the whole grid as the active range (nxs = nxgs, nxe = nxge). */

/* ------------------------------------------------------------- diagnostics */
/* Energy sums of energy_history, proj/weibel/app.f90:479-545:
 * out[0..nsp-1] = sum m_s (gamma-1), out[nsp] = sum E^2/8pi, out[nsp+1] = sum B^2/8pi.
 * Uses the dimensions of the last particle/field init. */
int wm_energy_sums(const double *up, const double *uf, const int *np2, double *out);
/* CG iterations per component (Bx, By, Bz) of the last field__fdtd_i call. */
int wm_field_cg_iters(int *iters3);
/* The SAVE'd work arrays of field__fdtd_i (field.f90:98): df (6,..) carries the previous step's
 * delta-B as the next CG initial guess, uj (3,..) is the last deposited current.  No
 * counterpart in the reference's public interface; used for restart and parity checks. */
int wm_field_get_work(double *df, double *uj);
int wm_field_set_work(const double *df);
/* Release every GPU buffer held by the module-procedure layer. */
int wm_finalize(void);

const char *wm_status_string(int status);
/* Library build string: architecture and precision paths compiled in. */
const char *wm_build_info(void);

/* -------------------------------------------------------- resident simulation */
typedef struct wm_sim wm_sim;

typedef struct wm_sim_config {
    int nx, ny, nsp;      /* interior cells; species (<= 4) */
    int np;               /* slots per row in the host reference layout used by load/store */
    double delx, delt, c, gfac;
    double q[4], r[4];    /* charge and mass per species */
    double cg_err;        /* relative CG tolerance (field.f90:339 uses 1e-6) */
    int cg_itemax;        /* CG iteration limit (field.f90:337 uses 100) */
    int precision;        /* WM_PREC_FP64 or WM_PREC_MIXED */
    int64_t capacity;     /* particle slots held on the GPU; 0 = the loaded count (enough unless
                             particles are injected: see wm_sim_set_injection) */
    int bc;               /* WM_BC_* (the step follows that application's main loop) */
    double u0;            /* WM_BC_SHOCK: upstream four-velocity at the injection boundary */
} wm_sim_config;

int wm_sim_create(const wm_sim_config *cfg, wm_sim **out);
int wm_sim_destroy(wm_sim *s);
/* Copy a host state (reference layout) to the GPU and cell-sort it (sort__bucket). */
int wm_sim_load(wm_sim *s, const double *up, const double *uf, const int *np2);
/* Copy the GPU state to host arrays in the reference layout: up slots 1..np2(j) of each row
 * (slots after that and up to the largest np2 are zeroed), uf, np2 and cumcnt. */
int wm_sim_store(wm_sim *s, double *up, double *uf, int *np2, int *cumcnt);
/* Advance nsteps steps on the GPU. */
int wm_sim_step(wm_sim *s, int nsteps);
/* The step with host buffers: load (up, uf, np2), nsteps steps, store (up, uf, np2, cumcnt).
 * up must be cell-sorted with a matching cumcnt on entry (the state the step loop keeps). */
int wm_sim_step_host(wm_sim *s, double *up, double *uf, int *np2, int *cumcnt, int nsteps);
int wm_sim_energy(wm_sim *s, double *out);
/* mom_calc__accl + mom_calc__nvt + boundary_periodic__mom on the resident state, into a host
 * array mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp). */
int wm_sim_moments(wm_sim *s, double *mom);
/* Snapshot and output files of the resident state, in the format of common/paraio.f90 for one
 * rank (a <name>.json description and a <name>.raw data file; `dir` is a prefix joined to the
 * file name as the Fortran does, so it ends in '/').  The data are put into file order on the GPU
 * (moments, cell-centred fields, ordered compaction of particles) and streamed to disk.
 *   write_snapshot   = paraio__output (paraio.f90:93-222) with nxs = nxgs, nxe = nxge; slots
 *                      beyond a row's count are written as zeros
 *   read_snapshot    = paraio__input (:227-417) followed by wm_sim_load; *it = the step
 *   write_moments    = mom_calc__accl/__nvt + boundary__mom, then paraio__mom (:555-713), file
 *                      <it:07d>_mom
 *   write_particles  = paraio__ptcl (tracers_only = 0, file <it:07d>_ptcl) or paraio__orb (1,
 *                      ids > 0, <it:07d>_orb), write_particle (:743-849).  In the mixed path the
 *                      particles of a cell follow that path's order (the FP64 path keeps the
 *                      reference's). */
int wm_sim_write_snapshot(wm_sim *s, const char *dir, const char *filename, int it);
int wm_sim_read_snapshot(wm_sim *s, const char *dir, const char *filename, int *it);
/* Seeded initial conditions generated on the GPU (two species: ions, electrons) and loaded as
 * wm_sim_load would, cell-sorted, with zero dB history.  Random numbers are Philox4x32-10 draws
 * keyed by `seed` and counted per particle, so a seed gives the same state on any GPU and launch
 * shape (the CPU restatement is oracle/init.py).
 *   weibel  ppc*nx particles per row and species at uniform random positions; ions Maxwellian
 *           (vth_i), electrons Maxwellian (vth_e) drifting along z at +/- v_drift (in c) by slot
 *           parity; ids 1..n per species; fields zero
 *   harris  proj/reconnection/app.f90:353-470 (bc = WM_BC_RECONNECTION): nbg background and ncs
 *           sheet particles per cell, half-thickness lcs (cells), field b0, perturbation e1,
 *           thermal speeds vte/vti, temperature ratio rtemp = Te/Ti (drifts split by it)
 *   shock   proj/shock/app.f90:408-525 (bc = WM_BC_SHOCK) over cells nxs+1 .. nxe-1 (nxe = nxge
 *           unless wm_sim_set_expansion set a smaller box): n0 per cell,
 *           upstream four-velocity u0 (< 0), field b0 at angles theta_bn/phi_bn, damping length
 *           l_damp_ini, tracer window [xrs, xre] (positive ids) */
int wm_sim_init_weibel(wm_sim *s, int ppc, double v_drift, double vth_e, double vth_i, uint64_t seed);
int wm_sim_init_harris(wm_sim *s, int nbg, int ncs, double lcs, double b0, double e1, double vte, double vti, double rtemp,
                       uint64_t seed);
int wm_sim_init_shock(wm_sim *s, int n0, double u0, double vth_e, double vth_i, double b0, double theta_bn, double phi_bn,
                      double l_damp_ini, double xrs, double xre, uint64_t seed);
/* Particle injection of the shock application (proj/shock/app.f90:695-850; bc = WM_BC_SHOCK,
 * at the active nxe): every step, after the sort, nginj = int(pflux) particles per species (one
 * more with probability frac(pflux)), pflux = n0 |v0| dt dx ny, v0 = u0/gamma0 from the
 * configuration's u0, enter behind the rows -- nginj/ny per row, one more in nginj mod ny rows
 * drawn at random -- at x = nxe dx + (k+1/2)/n_j |v0| dt moved by (v0 + u_x) dt, Maxwellian
 * (vth_e, vth_i) boosted by vprofile (l_damp_ini), ids negative after the species' count; np2 and
 * cumcnt(nxe) grow by the row's count (the row total with them), and the upstream field (b0,
 * theta_bn, phi_bn) is set in columns nxe-1 and nxe.  The draws are keyed by `seed` and counted by
 * the step number (wm_sim_set_step / wm_sim_get_step; generated states start at 0, a snapshot at
 * its own step).  on = 0 switches the injection off.  A step whose injection would exceed the
 * capacity injects nothing and returns WM_ERR_OVERFLOW. */
int wm_sim_set_injection(wm_sim *s, int on, int n0, double vth_e, double vth_i, double b0, double theta_bn, double phi_bn,
                         double l_damp_ini, uint64_t seed);
/* The shock application's expanding box (proj/shock/app.f90:277, :123-125, relocate :613-690;
 * bc = WM_BC_SHOCK): nxe = nxgs + n_x_ini (3 <= n_x_ini <= nx - 1) instead of nxge, set before
 * wm_sim_init_shock (whose plasma then fills nxs+1 .. nxe-1).  The particles, the injection
 * boundary at nxe and the field solve (nxs..nxe, field.f90:319-461; the fields past nxe + 1 keep
 * their values) follow nxe.  Every intvl_expand steps (0: never), after the injection, nxe grows by
 * one cell while nxe < nxge: n0 (the injection's) particles per row and species enter the new cell
 * nxe-1 at x = (nxe-1 + (k+1/2)/n0) dx, y = (j + U) dx, Maxwellian boosted by vprofile, ids
 * negative after the species' count; np2 and cumcnt(nxe) grow by n0; the upstream field is set in
 * columns nxe-1 and nxe.  The draws are Philox, keyed by the injection's seed and counted by the
 * step number.  A snapshot stores nxe and a read restores it. */
int wm_sim_set_expansion(wm_sim *s, int n_x_ini, int intvl_expand);
int wm_sim_get_nxe(wm_sim *s, int *nxe);
int wm_sim_set_step(wm_sim *s, int64_t it);
int wm_sim_get_step(wm_sim *s, int64_t *it);
int wm_sim_write_moments(wm_sim *s, const char *dir, int it);
int wm_sim_write_particles(wm_sim *s, const char *dir, int it, int tracers_only);
/* CG iterations per component of the last step. */
int wm_sim_cg_iters(wm_sim *s, int *iters3);
/* Per-kernel GPU time of the last wm_sim_step call, from CUDA events on the simulation's
 * stream: names[i] (static strings) and milliseconds ms[i]; *n in = capacity, out = count. */
int wm_sim_kernel_times(wm_sim *s, const char **names, double *ms, int *n);
/* Enable (1) or disable (0) the per-kernel event timing of wm_sim_step. */
int wm_sim_set_timing(wm_sim *s, int on);
/* Number of kernel launches of the last wm_sim_step call. */
int wm_sim_launches(wm_sim *s, int64_t *count);
/* Particle count and device bytes held. */
int wm_sim_info(wm_sim *s, int64_t *nparticles, int64_t *device_bytes);
/* Block until every launched step has finished. */
int wm_sim_sync(wm_sim *s);
/* Rebin of the mixed-precision step (no reference counterpart: the reference sorts its FP64
 * particles in place, sort.f90:36-82).  WM_REBIN_PERMUTE (the default) records the new cell order
 * as a slot permutation that the next push reads through, so the particles move once per step,
 * inside the push; the cell-sorted order is written out only when a call needs it (store, energy,
 * moments, files).  WM_REBIN_MOVE moves them into cell order after every step.  Both give the
 * same particles in the same order, bit for bit (injected particles included). */
enum { WM_REBIN_PERMUTE = 0, WM_REBIN_MOVE = 1 };
int wm_sim_set_rebin(wm_sim *s, int mode);
/* wm_sim_step bracketed by CUDA events on the simulation's stream: *ms = GPU time of the
 * nsteps steps (host synchronisations inside the step loop included). */
int wm_sim_step_timed(wm_sim *s, int nsteps, double *ms);
/* Learned initial guess for the CG (no reference counterpart; see wm_cnn_* below): params =
 * the network's FP32 parameters on the HOST, per layer w[9][cout][cin] then b[cout] for the
 * padded (cin, cout) = (16,48), (48,48) x 4, (48,8): 93560 values.  From the next step on, each
 * field component's CG starts from the network's dB or the previous step's dB, whichever has the
 * smaller residual, and runs to the usual tolerance.  params = NULL switches it off.  Needs nx a
 * multiple of 16 and ny a multiple of 8. */
int wm_sim_set_guess(wm_sim *s, const float *params, long long nparams);
/* For the last step with the guess on: stats[0..2] = |b - A dB_net|^2, stats[3..5] =
 * |b - A dB_prev|^2 per component, stats[6..8] = 1.0 where the network's guess was taken,
 * stats[9..11] = |b|^2 (12 values). */
int wm_sim_guess_stats(wm_sim *s, double *stats);
/* Select the CUDA device used by the calling host thread (one process per GPU). */
int wm_set_device(int device);

/* The SAVE'd field work arrays of the resident simulation (see wm_field_get_work). */
int wm_sim_get_work(wm_sim *s, double *df, double *uj);
int wm_sim_set_work(wm_sim *s, const double *df);

/* ------------------------------------------------- deposit without allocation
 * No counterpart in the reference: an extra entry point for callers that cannot call cudaMalloc,
 * such as an application that gives this library GPU memory from its own pool and allows no
 * allocation (and the device synchronisation that comes with it) after start-up.
 *
 * The current deposit of field__fdtd_i -- ele_cur (common/field.f90:189-316) followed by the
 * periodic current fold boundary_periodic__curre (common/boundary_periodic.f90:357-508) -- on
 * caller-owned device buffers in the reference layout: up, gp (6, np, ny, nsp), cumcnt
 * (nx+1, ny, nsp) in, uj (3, nx+4, ny+4) out; q (nsp values) is a host array.  Its scratch is a
 * fixed static device array inside this library, so it allocates nothing: at most 65536 interior
 * cells (nx*ny; more returns WM_ERR_BAD_ARG), 39.3 MB of device memory held by every GPU that
 * loads the library until exit.  All calls share that scratch, so calls that overlap on the GPU
 * race.  The first call on a device looks the scratch up (cudaGetSymbolAddress); under CUDA's
 * default lazy module loading that first call is also when the array is placed in device memory,
 * which is an allocation: make it at start-up, so that the memory is committed then and later
 * calls allocate nothing.  stream: a cudaStream_t, or NULL for the default stream.  The call is
 * synchronous: it reads a status word back and waits for the stream, so no call can be captured
 * into a CUDA graph.  Returns WM_OK, or WM_ERR_CELL if a particle moved more than one cell. */
int wm_deposit_current_noalloc(const double *up, const double *gp, const int *cumcnt, double *uj, int ndim, int np, int nsp,
                               int nxgs, int nxge, int nygs, int nyge, double delx, double delt, double c, const double *q,
                               void *stream);

/* No counterpart in the reference: the measured FP64 rate of this GPU (TFLOP/s), from CUDA events
 * around a kernel of independent FP64 fused multiply-add chains on whole waves of the SMs; the
 * denominator of the FP64 path's roofline.  ms (may be NULL) receives the kernel's time. */
int wm_fp64_fma_rate(double *tflops, double *ms);

/* Page-lock (pin) a host buffer so that copies from and to it run at full link speed. */
int wm_host_register(void *ptr, size_t bytes);
int wm_host_unregister(void *ptr);

/* Allocate / free page-locked host memory (cudaHostAlloc, portable across devices, mapped into the
 * device's address space).  The state arrays up and uf that wm_sim_step_host copies every call are
 * best placed here: the copies reach their full rate on such memory whatever the CPU did to it
 * before, while a buffer that was registered after the CPU first touched it can copy several times
 * slower on Grace hosts; the particle rows of such memory are read and (mixed path) written by the
 * library's kernels directly. */
int wm_host_alloc(void **ptr, size_t bytes);
int wm_host_free(void *ptr);

/* -------------------------------------------------------------- module paraio (host arrays)
 * common/paraio.f90, procedure for procedure, for one rank (nproc = 1; other values return
 * WM_ERR_UNSUPPORTED).  Host-side file I/O on the caller's arrays in the reference layout; the
 * file pair is <dir><name>.json + <dir><name>.raw.  Where the Fortran stops (uninitialised
 * module, parameter mismatch on input) these return WM_ERR_NOT_INIT / WM_ERR_IO.  The GPU-resident
 * state is written by the wm_sim_write_* functions above instead. */
int wm_paraio_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nproc, int nrank,
                   double delx, double delt, double c, const double *q, const double *r, const char *dir); /* :37-72 */
int wm_paraio_finalize(void);                                                                     /* :77-85 */
int wm_paraio_output(const double *up, const double *uf, const int *np2, int nxs, int nxe, int it,
                     const char *filename);                                                       /* :93-222 */
int wm_paraio_input(double *up, double *uf, int *np2, int *nxs, int *nxe, int *it, const char *filename); /* :227-417 */
int wm_paraio_param(int n0, double wpe, double wpi, double wge, double wgi, double vti, double vte,
                    const char *filename);                                                        /* :422-550 */
/* mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp) is intent(inout): velocity and temperature rows are
 * divided by the density in place, ghost cells included, as the Fortran does (:641-660). */
int wm_paraio_mom(double *mom, const double *uf, int it);                                         /* :555-713 */
int wm_paraio_ptcl(const double *up, const double *uf, const int *np2, int it);                   /* :718-726 */
int wm_paraio_orb(const double *up, const double *uf, const int *np2, int it);                    /* :731-738 */

/* ------------------------------------------------- learned initial guess for the implicit solve
 * No reference counterpart: the reference starts its CG (common/field.f90:319-461) from the
 * previous step's dB only.  A six-layer 3x3 convolutional network on the periodic cell grid maps
 * (E, B at time n; J at n+1/2) to dB.  All pointers below are DEVICE pointers; activations are
 * BF16 NHWC [nimg][h][w][c] (periodic in h and w, h a multiple of 8, w a multiple of 16), weights
 * BF16 [9][cout][cin] (tap = (dy+1)*3 + dx+1), biases FP32.  stream: a cudaStream_t or NULL.  The
 * calls are asynchronous on the stream. */
enum { WM_CNN_FWD_TRAIN = 0, WM_CNN_FWD_INFER = 1, WM_CNN_FWD_LINEAR = 2, WM_CNN_BWD = 3 };
/* OR-ed into the mode (or the wgrad flags) of a (48, 48) layer: the weights are block-diagonal
 * over three groups of 16 channels, as in the learned guess, and only the diagonal blocks are
 * computed (the other weights must be zero; their gradient is returned as zero). */
enum { WM_CNN_GROUPED = 16 };
/* The convolutions (all four modes) and the weight gradient run on the 5th-generation tensor
 * cores (tcgen05.mma, accumulators in tensor memory) when h is a multiple of 16 and w of 8;
 * OR-ing WM_CNN_MMA_SYNC into the mode (or the wgrad flags) selects the warp-level mma.sync
 * kernel instead (the one other shapes use). */
enum { WM_CNN_MMA_SYNC = 32 };

/* One 3x3 convolution, (cin, cout) in {(16, 48), (48, 48), (48, 8)}.  Modes:
 *   FWD_TRAIN  out = GELU(conv + bias) BF16 and zout = conv + bias BF16;
 *   FWD_INFER  out = GELU(conv + bias) BF16;
 *   FWD_LINEAR out = conv + bias FP32 [.][cout] (cin 48, cout 8 only);
 *   BWD        out = conv (no bias) * GELU'(zprev) BF16, zprev [.][cout]: with the flipped,
 *              transposed weights of the next layer this is the pre-activation gradient. */
int wm_cnn_conv3x3(const void *in, const void *w, const float *bias, int cin, int cout, int mode, int nimg, int h, int wd, void *out,
                   void *zout, const void *zprev, void *stream);
/* WM_ERR_CUDA if a tensor-core convolution of the calls above gave up waiting for its MMAs (a
 * bounded wait; the output of that call is not valid), else WM_OK; clear != 0 resets the flag.
 * Call it after the stream's work has finished. */
int wm_cnn_status(int clear);
/* Weight and bias gradients dw[9][cout][cin] (FP32), db[cout] from the layer input x [.][cin] and
 * the pre-activation gradient dz [.][coutp], (cin, coutp) in {(16, 48), (48, 48), (48, 16)},
 * cout <= coutp.  scratch: at least 9*coutp*cin + coutp floats per CTA used (up to 304 CTAs for
 * mma.sync, one per SM for tcgen05; fewer CTAs are used when scratch is smaller).  A timed-out
 * wait of the tcgen05 kernel is reported by wm_cnn_status. */
int wm_cnn_conv3x3_wgrad(const void *x, const void *dz, int cin, int coutp, int cout, int nimg, int h, int wd, int flags, float *dw,
                         float *db, float *scratch, long long scratch_floats, void *stream);
/* *loss = sum over pixels and the 3 outputs of 0.5 (pred - target)^2 / (3 npix); dz = its gradient
 * as BF16 [npix][16].  pred FP32 [npix][8], target FP32 [npix][3]; partial holds nblocks doubles. */
int wm_cnn_mse(const float *pred, const float *target, long long npix, void *dz, double *partial, int nblocks, double *loss, void *stream);
/* The same over the interior of nimg images of h x w pixels: pixels within `border` of an edge are
 * left out of the loss and get a zero gradient (training on crops of a larger field, where the
 * network's periodic padding does not see the field's true neighbours). */
int wm_cnn_mse_interior(const float *pred, const float *target, int nimg, int h, int wd, int border, void *dz, double *partial, int nblocks,
                        double *loss, void *stream);
/* One Adam step (step = 1, 2, ...) on n FP32 parameters; mask (optional, n values) multiplies the
 * gradient, so parameters with mask 0 keep their value. */
int wm_cnn_adam(float *p, const float *grad, const float *mask, float *m, float *v, long long n, float lr, float beta1, float beta2,
                float eps, int step, void *stream);
/* BF16 layer weights from FP32 w[9][cout][cin]: wf = the same layout; wt (optional) = the flipped
 * transpose [9][cin][coutb], wt(tap, ci, co) = w(8 - tap, co, ci) for co < cout, else 0. */
int wm_cnn_prep_weights(const float *w, int cin, int cout, int coutb, void *wf, void *wt, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* WUMINGPIC2D_H */
