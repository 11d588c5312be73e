/* ref_glue.c -- entry points into the C translation of the reference's hot-path modules.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/f90c.py translates the reference's common/ modules into
 * oracle/_ref/wuming_ref.c; this file calls those translated procedures the way
 * proj/weibel/app.f90 does on one MPI rank (nup = ndown = the rank itself, datatype handles =
 * element sizes for the single-rank MPI stubs) and turns a Fortran `stop` into status 1.
 * tests/test_reference_pin.py and tests/golden/make_golden.py use it through oracle/reference.py. */
#include <setjmp.h>
#include <string.h>

jmp_buf f90_stop_env;
int f90_stopped;

void ref_boundary_periodic__init(int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *,
                                 int *, int *, long, double *, double *, double *);
void ref_boundary_periodic__particle_x(double *, int *);
void ref_boundary_periodic__particle_y(double *, int *);
void ref_boundary_periodic__dfield(double *, int *, int *, int *, int *, int *, int *);
void ref_boundary_periodic__curre(double *, int *, int *, int *, int *, int *, int *);
void ref_boundary_periodic__phi(double *, int *, int *, int *, int *, int *);
void ref_boundary_periodic__mom(double *);
/* the applications' boundary modules: proj/reconnection/boundary_reconnection.f90 and
 * proj/shock/boundary_shock.f90 (same init arguments) */
#define WALL_DECLS(M)                                                                                                                \
    void ref_boundary_##M##__init(int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *,  \
                                  int *, int *, long, double *, double *, double *);                                                 \
    void ref_boundary_##M##__particle_x(double *, int *, int *, int *);                                                             \
    void ref_boundary_##M##__particle_y(double *, int *);                                                                           \
    void ref_boundary_##M##__dfield(double *, int *, int *, int *, int *, int *, int *);                                            \
    void ref_boundary_##M##__curre(double *, int *, int *, int *, int *, int *, int *);                                             \
    void ref_boundary_##M##__phi(double *, int *, int *, int *, int *, int *);                                                      \
    void ref_boundary_##M##__mom(double *);                                                                                         \
    extern int boundary_##M##__boundary_##M##__particle_y__lflag;
WALL_DECLS(reconnection)
WALL_DECLS(shock)
void ref_boundary_shock__injection(double *, int *, int *, int *, double *);
void ref_particle__init(int *, int *, int *, int *, int *, int *, int *, int *, int *, double *, double *, double *, double *,
                        double *);
void ref_particle__solv(double *, double *, double *, int *, int *, int *);
void ref_field__init(int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, int *, double *, double *,
                     double *, double *, double *, double *);
void ref_field__fdtd_i(double *, double *, double *, int *, int *, int *, void (*)(), void (*)(), void (*)());
void ref_sort__init(int *, int *, int *, int *, int *, int *, int *, int *, int *);
void ref_sort__bucket(double *, double *, int *, int *, int *, int *);
void ref_mom_calc__init(int *, int *, int *, int *, int *, int *, int *, int *, int *, double *, double *, double *, double *,
                        double *);
void ref_mom_calc__accl(double *, double *, double *, int *, int *, int *);
void ref_mom_calc__nvt(double *, double *, int *);

/* SAVE'd state of field__fdtd_i (field.f90:96-98) and boundary_periodic__particle_y (:106-111) */
extern int field__field__fdtd_i__lflag;
extern double *field__field__fdtd_i__df, *field__field__fdtd_i__uj, *field__field__fdtd_i__gkl;
extern int boundary_periodic__boundary_periodic__particle_y__lflag;

#define GUARD                          \
    f90_stopped = 0;                   \
    if (setjmp(f90_stop_env)) return 1;

static int g_nxw, g_nyw, g_nx, g_ny;

int wmr_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, double delx, double delt, double c, const double *q,
             const double *r, double gfac)
{
    GUARD
    int nys = nygs, nye = nyge, nup = 0, ndown = 0, mnpi = (int)sizeof(int), mnpr = (int)sizeof(double), ncomw = 0, nerr = 0,
        opsum = 0;
    int nstat[1] = {0};
    double qq[8], rr[8];
    memcpy(qq, q, sizeof(double) * nsp);
    memcpy(rr, r, sizeof(double) * nsp);
    /* a fresh process: the first calls allocate the SAVE'd work arrays for these dimensions */
    field__field__fdtd_i__lflag = 1;
    boundary_periodic__boundary_periodic__particle_y__lflag = 1;
    ref_boundary_periodic__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye, &nup, &ndown, &mnpi, &mnpr, &ncomw, &nerr,
                                nstat, 1, &delx, &delt, &c);
    boundary_reconnection__boundary_reconnection__particle_y__lflag = 1;
    boundary_shock__boundary_shock__particle_y__lflag = 1;
    ref_boundary_reconnection__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye, &nup, &ndown, &mnpi, &mnpr, &ncomw,
                                    &nerr, nstat, 1, &delx, &delt, &c);
    ref_boundary_shock__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye, &nup, &ndown, &mnpi, &mnpr, &ncomw, &nerr,
                             nstat, 1, &delx, &delt, &c);
    ref_particle__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye, &delx, &delt, &c, qq, rr);
    ref_field__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye, &mnpr, &ncomw, &opsum, &nerr, &delx, &delt, &c, qq, rr,
                    &gfac);
    ref_sort__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye);
    ref_mom_calc__init(&ndim, &np, &nsp, &nxgs, &nxge, &nygs, &nyge, &nys, &nye, &delx, &delt, &c, qq, rr);
    g_nx = nxge - nxgs + 1;
    g_ny = nyge - nygs + 1;
    g_nxw = g_nx + 4;
    g_nyw = g_ny + 4;
    return 0;
}

int wmr_particle_solv(double *gp, double *up, double *uf, int *cumcnt, int nxs, int nxe)
{
    GUARD
    ref_particle__solv(gp, up, uf, cumcnt, &nxs, &nxe);
    return 0;
}

int wmr_mom_accl(double *gp, double *up, double *uf, int *cumcnt, int nxs, int nxe)
{
    GUARD
    ref_mom_calc__accl(gp, up, uf, cumcnt, &nxs, &nxe);
    return 0;
}

int wmr_mom_nvt(double *mom, double *up, int *np2)
{
    GUARD
    ref_mom_calc__nvt(mom, up, np2);
    return 0;
}

/* boundary module the procedures below use: 0 periodic (Weibel), 1 reconnection, 2 shock */
static int g_bc;
int wmr_set_bc(int kind)
{
    g_bc = kind;
    return 0;
}
#define BC_PROC(name) (g_bc == 1 ? (void (*)())ref_boundary_reconnection__##name \
                                 : g_bc == 2 ? (void (*)())ref_boundary_shock__##name : (void (*)())ref_boundary_periodic__##name)

int wmr_field_fdtd_i(double *uf, double *up, double *gp, int *cumcnt, int nxs, int nxe)
{
    GUARD
    ref_field__fdtd_i(uf, up, gp, cumcnt, &nxs, &nxe, BC_PROC(dfield), BC_PROC(curre), BC_PROC(phi));
    return 0;
}

/* Copy the SAVE'd work arrays out (get != 0) or df in.  Valid after the first field__fdtd_i. */
int wmr_field_work(double *df, double *uj, double *gkl, int get)
{
    if (field__field__fdtd_i__lflag) return 2;
    const size_t nf = (size_t)g_nxw * g_nyw;
    if (get) {
        if (df) memcpy(df, field__field__fdtd_i__df, sizeof(double) * 6 * nf);
        if (uj) memcpy(uj, field__field__fdtd_i__uj, sizeof(double) * 3 * nf);
        if (gkl) memcpy(gkl, field__field__fdtd_i__gkl, sizeof(double) * 3 * (size_t)g_nx * g_ny);
    } else if (df) {
        memcpy(field__field__fdtd_i__df, df, sizeof(double) * 6 * nf);
    }
    return 0;
}

int wmr_bc_particle_x(double *up, int *np2)
{
    GUARD
    ref_boundary_periodic__particle_x(up, np2);
    return 0;
}

/* the walls' particle_x (reconnection app) and the shock's injection boundary */
int wmr_bc_particle_x_walls(double *up, int *np2, int nxs, int nxe)
{
    GUARD
    if (g_bc == 2) ref_boundary_shock__particle_x(up, np2, &nxs, &nxe);
    else ref_boundary_reconnection__particle_x(up, np2, &nxs, &nxe);
    return 0;
}

int wmr_bc_injection(double *up, int *np2, int nxs, int nxe, double u0)
{
    GUARD
    ref_boundary_shock__injection(up, np2, &nxs, &nxe, &u0);
    return 0;
}

int wmr_bc_particle_y(double *up, int *np2)
{
    GUARD
    ((void (*)(double *, int *))BC_PROC(particle_y))(up, np2);
    return 0;
}

int wmr_sort_bucket(double *gp, double *up, int *cumcnt, int *np2, int nxs, int nxe)
{
    GUARD
    ref_sort__bucket(gp, up, cumcnt, np2, &nxs, &nxe);
    return 0;
}

int wmr_bc_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    GUARD
    ((void (*)(double *, int *, int *, int *, int *, int *, int *))BC_PROC(dfield))(df, &nxs, &nxe, &nys, &nye, &nxgs, &nxge);
    return 0;
}

int wmr_bc_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    GUARD
    ((void (*)(double *, int *, int *, int *, int *, int *, int *))BC_PROC(curre))(uj, &nxs, &nxe, &nys, &nye, &nxgs, &nxge);
    return 0;
}

int wmr_bc_phi(double *phi, int nxs, int nxe, int nys, int nye, int l)
{
    GUARD
    ((void (*)(double *, int *, int *, int *, int *, int *))BC_PROC(phi))(phi, &nxs, &nxe, &nys, &nye, &l);
    return 0;
}

int wmr_bc_mom(double *mom)
{
    GUARD
    ((void (*)(double *))BC_PROC(mom))(mom);
    return 0;
}
