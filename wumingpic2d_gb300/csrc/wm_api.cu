// wm_api.cu -- the C ABI: module-procedure mirror of the reference's common/ modules and the
// resident simulation.  Host code only; every kernel lives in wm_particles.cu, wm_rebin.cu and
// wm_field.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "wm_launch.cuh"

// ============================================================== shared helpers
namespace {

constexpr int CG_BATCH = 4;
constexpr double PI_REF = 3.14159265358979311599796346854418516;

int make_geom(WmGeom &g, int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye)
{
    if (ndim != 6 || nsp < 1 || nsp > WM_MAX_SP || np < 1) return WM_ERR_BAD_ARG;
    if (nys != nygs || nye != nyge) return WM_ERR_UNSUPPORTED;  // one process owns every row
    g.ndim = ndim;
    g.np = np;
    g.nsp = nsp;
    g.nxgs = nxgs;
    g.nxge = nxge;
    g.nygs = nygs;
    g.nyge = nyge;
    g.nys = nys;
    g.nye = nye;
    g.nx = nxge - nxgs + 1;
    g.ny = nye - nys + 1;
    if (g.nx < 4 || g.ny < 4) return WM_ERR_BAD_ARG;
    g.nrows = nsp * g.ny;
    g.nxw = g.nx + 4;
    g.nyw = g.ny + 4;
    g.bc = WM_BC_PERIODIC;  // the boundary module's init sets its own kind
    g.nxa = g.nx;
    return WM_OK;
}

void make_const(WmConst &k, int nsp, double delx, double delt, double c, const double *q, const double *r, double gfac)
{
    k.delx = delx;
    k.delt = delt;
    k.c = c;
    k.gfac = gfac;
    for (int s = 0; s < WM_MAX_SP; ++s) {
        k.q[s] = (s < nsp && q) ? q[s] : 0.0;
        k.r[s] = (s < nsp && r) ? r[s] : 1.0;
    }
    k.cg_err = 1e-6;  // field.f90:339
    k.cg_itemax = 100;  // field.f90:337
}

size_t up_doubles(const WmGeom &g) { return (size_t)g.ndim * g.np * g.nrows; }
size_t f_points(const WmGeom &g) { return (size_t)g.nxw * g.nyw; }
size_t cc_ints(const WmGeom &g) { return (size_t)(g.nx + 1) * g.nrows; }
size_t mom_doubles(const WmGeom &g) { return (size_t)7 * (g.nx + 2) * (g.ny + 2) * g.nsp; }

int map_status(unsigned dev)
{
    if (dev & WMDEV_OVERFLOW) return WM_ERR_OVERFLOW;
    if (dev & (WMDEV_CELL | WMDEV_ROWJUMP)) return WM_ERR_CELL;
    return WM_OK;
}

// Rebin scratch sized for `cap` particle indices.
struct RebinBufs {
    DevBuf dir, ord, P, key, holes, nup, ndown, cellcnt, pairs, np2_new, rowbase_new, drow, status;
    int ensure(long long cap, const WmGeom &g)
    {
        WM_TRY(dir.ensure((size_t)cap));
        WM_TRY(ord.ensure(sizeof(int) * (size_t)cap));
        WM_TRY(P.ensure(sizeof(int) * (size_t)cap));
        WM_TRY(key.ensure(sizeof(int) * (size_t)cap));
        WM_TRY(holes.ensure(sizeof(int) * (size_t)cap));
        WM_TRY(drow.ensure(sizeof(int) * (size_t)cap));
        WM_TRY(pairs.ensure(sizeof(unsigned long long) * (size_t)cap));
        WM_TRY(nup.ensure(sizeof(int) * g.nrows));
        WM_TRY(ndown.ensure(sizeof(int) * g.nrows));
        WM_TRY(np2_new.ensure(sizeof(int) * g.nrows));
        WM_TRY(rowbase_new.ensure(sizeof(long long) * (g.nrows + 1)));
        WM_TRY(cellcnt.ensure(sizeof(int) * (size_t)g.nrows * g.nx));
        WM_TRY(status.ensure(sizeof(unsigned)));
        return WM_OK;
    }
    WmRebinScratch view() const
    {
        WmRebinScratch s;
        s.dir = dir.as<unsigned char>();
        s.ord = ord.as<int>();
        s.P = P.as<int>();
        s.key = key.as<int>();
        s.holes = holes.as<int>();
        s.nup = nup.as<int>();
        s.ndown = ndown.as<int>();
        s.cellcnt = cellcnt.as<int>();
        s.pairs = pairs.as<unsigned long long>();
        s.np2_new = np2_new.as<int>();
        s.rowbase_new = rowbase_new.as<long long>();
        s.status = status.as<unsigned>();
        return s;
    }
    void release()
    {
        for (DevBuf *b : {&dir, &ord, &P, &key, &holes, &nup, &ndown, &cellcnt, &pairs, &np2_new, &rowbase_new, &drow, &status})
            b->release();
    }
};

struct FieldBufs {
    DevBuf uf, uj, df, pjcell, b, r, p, ap, partial, ticket, scal;
    CgScal *scal_host = nullptr;
    int ensure(const WmGeom &g)
    {
        const size_t nf = f_points(g), nc = (size_t)g.nx * g.ny;
        WM_TRY(uf.ensure(sizeof(double) * 6 * nf));
        WM_TRY(uj.ensure(sizeof(double) * 3 * nf));
        WM_TRY(df.ensure(sizeof(double) * 6 * nf));
        WM_TRY(pjcell.ensure(sizeof(double) * 75 * nc));
        WM_TRY(b.ensure(sizeof(double) * 3 * nc));
        WM_TRY(r.ensure(sizeof(double) * 3 * nc));
        WM_TRY(p.ensure(sizeof(double) * 3 * nc));
        WM_TRY(ap.ensure(sizeof(double) * 3 * nc));
        WM_TRY(partial.ensure(sizeof(double) * 3 * wm_field_cg_blocks()));
        if (!ticket.p) {
            WM_TRY(ticket.ensure(sizeof(unsigned)));
            WM_CUDA(cudaMemset(ticket.p, 0, sizeof(unsigned)));
        }
        WM_TRY(scal.ensure(wm_field_scal_bytes()));
        if (!scal_host) WM_CUDA(cudaMallocHost((void **)&scal_host, wm_field_scal_bytes()));
        return WM_OK;
    }
    WmFieldWork work()
    {
        WmFieldWork w;
        w.b = b.as<double>();
        w.r = r.as<double>();
        w.p = p.as<double>();
        w.ap = ap.as<double>();
        w.partial = partial.as<double>();
        w.ticket = ticket.as<unsigned>();
        w.scal = scal.as<CgScal>();
        w.scal_host = scal_host;
        return w;
    }
    void release()
    {
        for (DevBuf *x : {&uf, &uj, &df, &pjcell, &b, &r, &p, &ap, &partial, &ticket, &scal}) x->release();
        if (scal_host) cudaFreeHost(scal_host);
        scal_host = nullptr;
    }
};

template <int NC>
FView<NC, false> soa_view(const DevBuf &b, const WmGeom &g)
{
    return FView<NC, false>{b.as<double>(), g.nxw, g.nyw};
}
template <int NC>
FView<NC, true> aos_view(const DevBuf &b, const WmGeom &g)
{
    return FView<NC, true>{b.as<double>(), g.nxw, g.nyw};
}

int read_status(unsigned *dev_status, cudaStream_t st, unsigned *out)
{
    WM_CUDA(cudaMemcpyAsync(out, dev_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    WM_CUDA(cudaStreamSynchronize(st));
    return WM_OK;
}

int max_of(const int *a, size_t n)
{
    int m = 0;
    for (size_t i = 0; i < n; ++i) m = std::max(m, a[i]);
    return m;
}

}  // namespace

// ========================================================= module-procedure layer
namespace {

struct ModuleState {
    bool particle_ok = false, field_ok = false, sort_ok = false, mom_ok = false, bc_ok = false;
    WmGeom gpart{}, gfield{}, gsort{}, gmom{}, gbc{};
    WmConst kpart{}, kfield{}, kmom{}, kbc{};
    cudaStream_t st = nullptr;
    DevBuf a, b, uf_aos, cc, np2, np2b, mom, phi, energy_partial, energy_out;
    FieldBufs fb;
    RebinBufs rb;
    bool field_work_zeroed = false;
    int last_iters[3] = {0, 0, 0};
    int bc_kind = WM_BC_PERIODIC;  // the boundary module whose *_init ran last

    int stream()
    {
        if (!st) WM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        return WM_OK;
    }
    void release()
    {
        for (DevBuf *x : {&a, &b, &uf_aos, &cc, &np2, &np2b, &mom, &phi, &energy_partial, &energy_out}) x->release();
        fb.release();
        rb.release();
        field_work_zeroed = false;
        if (st) cudaStreamDestroy(st);
        st = nullptr;
    }
};

ModuleState M;

int h2d(DevBuf &d, const void *h, size_t bytes, cudaStream_t st)
{
    WM_TRY(d.ensure(bytes));
    WM_CUDA(cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, st));
    return WM_OK;
}
int d2h(void *h, const DevBuf &d, size_t bytes, cudaStream_t st)
{
    WM_CUDA(cudaMemcpyAsync(h, d.p, bytes, cudaMemcpyDeviceToHost, st));
    return WM_OK;
}
int finish(cudaStream_t st)
{
    WM_CUDA(cudaStreamSynchronize(st));
    WM_CUDA(cudaGetLastError());
    return WM_OK;
}

}  // namespace

extern "C" {

int wm_particle_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, double delx,
                     double delt, double c, const double *q, const double *r)
{
    WM_TRY(make_geom(M.gpart, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye));
    make_const(M.kpart, nsp, delx, delt, c, q, r, 0.501);
    M.particle_ok = true;
    return WM_OK;
}

// The x range nxs..nxe of a call: nxs = nxgs and nxgs + 3 <= nxe <= nxge, nxe below nxge for the
// shock application's growing box (proj/shock/app.f90:277, relocate :613-690); the boundary and
// field procedures take it under the shock's boundary module only (walls_only).  The call's
// geometry follows nxe (nxa = nxe - nxgs + 1 active cells).
static int active_range(WmGeom &g, int nxs, int nxe, bool walls_only)
{
    if (nxs != g.nxgs || nxe > g.nxge || nxe < g.nxgs + 3) return WM_ERR_UNSUPPORTED;
    if (nxe != g.nxge && walls_only && g.bc != WM_BC_SHOCK) return WM_ERR_UNSUPPORTED;
    g.nxa = nxe - g.nxgs + 1;
    return WM_OK;
}

static int push_dropin(const WmGeom &g0, const WmConst &k, double *gp, const double *up, const double *uf, const int *cumcnt,
                       int nxs, int nxe, int half)
{
    WmGeom g = g0;  // cells nxs..nxe (particle.f90:86)
    WM_TRY(active_range(g, nxs, nxe, false));
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    const size_t nup = up_doubles(g) * sizeof(double);
    WM_TRY(h2d(M.a, up, nup, st));
    WM_TRY(h2d(M.b, gp, nup, st));
    WM_TRY(h2d(M.uf_aos, uf, sizeof(double) * 6 * f_points(g), st));
    WM_TRY(h2d(M.cc, cumcnt, sizeof(int) * cc_ints(g), st));
    AoSView va{M.a.as<double>(), g.np}, vb{M.b.as<double>(), g.np};
    WM_TRY(wm_launch_push(g, k, va, vb, aos_view<6>(M.uf_aos, g), M.cc.as<int>(), half, 0, st));
    if (!half) WM_TRY(wm_launch_pid_copy_aos(M.b.as<double>(), M.a.as<double>(), (long long)g.np * g.nrows, st));
    WM_TRY(d2h(gp, M.b, nup, st));
    return finish(st);
}

int wm_particle_solv(double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe)
{
    if (!M.particle_ok) return WM_ERR_NOT_INIT;
    return push_dropin(M.gpart, M.kpart, gp, up, uf, cumcnt, nxs, nxe, 0);
}

int wm_field_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int mnpr, int ncomw,
                  int opsum, int nerr, double delx, double delt, double c, const double *q, const double *r, double gfac)
{
    (void)mnpr;
    (void)ncomw;
    (void)opsum;
    (void)nerr;
    WM_TRY(make_geom(M.gfield, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye));
    make_const(M.kfield, nsp, delx, delt, c, q, r, gfac);
    M.field_ok = true;
    M.field_work_zeroed = false;
    return WM_OK;
}

static int field_work_ready(const WmGeom &g)
{
    WM_TRY(M.stream());
    WM_TRY(M.fb.ensure(g));
    if (!M.field_work_zeroed) {  // field.f90:105-119: df, gkl, uj allocated and zeroed on the first call
        WM_CUDA(cudaMemsetAsync(M.fb.df.p, 0, sizeof(double) * 6 * f_points(g), M.st));
        WM_CUDA(cudaMemsetAsync(M.fb.uj.p, 0, sizeof(double) * 3 * f_points(g), M.st));
        M.field_work_zeroed = true;
    }
    return WM_OK;
}

int wm_field_fdtd_i(double *uf, const double *up, const double *gp, const int *cumcnt, int nxs, int nxe)
{
    if (!M.field_ok) return WM_ERR_NOT_INIT;
    if (!M.bc_ok) return WM_ERR_NOT_INIT;  // the boundary procedures: those of the module initialised last
    WmGeom g = M.gfield;
    g.bc = M.bc_kind;
    WM_TRY(active_range(g, nxs, nxe, true));  // deposit, solve and update over nxs..nxe (field.f90:121-184)
    WM_TRY(field_work_ready(g));
    cudaStream_t st = M.st;
    const size_t nup = up_doubles(g) * sizeof(double);
    const long long npts = (long long)f_points(g);
    WM_TRY(h2d(M.a, up, nup, st));
    WM_TRY(h2d(M.b, gp, nup, st));
    WM_TRY(h2d(M.cc, cumcnt, sizeof(int) * cc_ints(g), st));
    WM_TRY(h2d(M.uf_aos, uf, sizeof(double) * 6 * npts, st));
    WM_TRY(M.rb.ensure(1, g));
    WM_CUDA(cudaMemsetAsync(M.rb.status.p, 0, sizeof(unsigned), st));
    WM_TRY(wm_launch_aos_to_soa(6, npts, M.uf_aos.as<double>(), M.fb.uf.as<double>(), st));
    AoSView va{M.a.as<double>(), g.np}, vb{M.b.as<double>(), g.np};
    WM_TRY(wm_launch_deposit_cells(g, M.kfield, va, vb, M.cc.as<int>(), M.fb.pjcell.as<double>(), M.rb.status.as<unsigned>(), st));
    WM_TRY(wm_launch_deposit_fold(g, soa_view<3>(M.fb.uj, g), M.fb.pjcell.as<double>(), st));
    WmFieldWork w = M.fb.work();
    const int s = wm_field_solve(g, M.kfield, soa_view<6>(M.fb.uf, g), soa_view<3>(M.fb.uj, g), soa_view<6>(M.fb.df, g), w,
                                 M.last_iters, CG_BATCH, st, nullptr, nullptr, nullptr);
    if (s != WM_OK) return s;
    WM_TRY(wm_launch_soa_to_aos(6, npts, M.fb.uf.as<double>(), M.uf_aos.as<double>(), st));
    WM_TRY(d2h(uf, M.uf_aos, sizeof(double) * 6 * npts, st));
    unsigned dev = 0;
    WM_TRY(read_status(M.rb.status.as<unsigned>(), st, &dev));
    WM_TRY(finish(st));
    return map_status(dev);
}

int wm_sort_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye)
{
    WM_TRY(make_geom(M.gsort, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye));
    M.sort_ok = true;
    return WM_OK;
}

int wm_sort_bucket(double *gp, const double *up, int *cumcnt, const int *np2, int nxs, int nxe)
{
    if (!M.sort_ok) return WM_ERR_NOT_INIT;
    WmGeom g = M.gsort;
    WM_TRY(active_range(g, nxs, nxe, false));  // cumcnt(nxs:nxe+1) (sort.f90:57-70): the rest of the rows untouched
    if ((long long)g.np * g.nrows >= (1LL << 32)) return WM_ERR_UNSUPPORTED;
    for (int r = 0; r < g.nrows; ++r)
        if (np2[r] < 0 || np2[r] > g.np) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    const size_t nup = up_doubles(g) * sizeof(double);
    WM_TRY(h2d(M.a, up, nup, st));
    WM_TRY(h2d(M.b, gp, nup, st));
    WM_TRY(h2d(M.np2, np2, sizeof(int) * g.nrows, st));
    WM_TRY(M.cc.ensure(sizeof(int) * cc_ints(g)));
    WM_TRY(M.rb.ensure((long long)g.np * g.nrows, g));
    WmRebinScratch sc = M.rb.view();
    WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
    const int maxc = max_of(np2, (size_t)g.nrows);
    AoSView va{M.a.as<double>(), g.np}, vb{M.b.as<double>(), g.np};
    WM_TRY(wm_launch_wrap_classify(g, 1.0, va, M.np2.as<int>(), maxc, 8, sc, st));
    WM_TRY(wm_launch_slot_as_P(g, va, M.np2.as<int>(), maxc, sc, st));
    WM_TRY(wm_launch_scan_cells(g, sc, M.cc.as<int>(), sc.np2_new, st));
    unsigned dev = 0;
    WM_TRY(read_status(sc.status, st, &dev));
    if (map_status(dev) != WM_OK) return map_status(dev);
    WM_TRY(wm_launch_sort_move(g, va, vb, M.np2.as<int>(), maxc, M.cc.as<int>(), sc, st));
    WM_TRY(d2h(gp, M.b, nup, st));
    if (g.nxa == g.nx) {
        WM_TRY(d2h(cumcnt, M.cc, sizeof(int) * cc_ints(g), st));
    } else {
        const size_t pitch = sizeof(int) * (g.nx + 1);
        WM_CUDA(cudaMemcpy2DAsync(cumcnt, pitch, M.cc.p, pitch, sizeof(int) * (g.nxa + 1), g.nrows, cudaMemcpyDeviceToHost, st));
    }
    return finish(st);
}

int wm_mom_calc_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, double delx,
                     double delt, double c, const double *q, const double *r)
{
    WM_TRY(make_geom(M.gmom, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye));
    make_const(M.kmom, nsp, delx, delt, c, q, r, 0.501);
    M.mom_ok = true;
    return WM_OK;
}

int wm_mom_calc_accl(double *gp, const double *up, const double *uf, const int *cumcnt, int nxs, int nxe)
{
    if (!M.mom_ok) return WM_ERR_NOT_INIT;
    return push_dropin(M.gmom, M.kmom, gp, up, uf, cumcnt, nxs, nxe, 1);
}

int wm_mom_calc_nvt(double *mom, const double *up, const int *np2)
{
    if (!M.mom_ok) return WM_ERR_NOT_INIT;
    const WmGeom &g = M.gmom;
    for (int r = 0; r < g.nrows; ++r)
        if (np2[r] < 0 || np2[r] > g.np) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    WM_TRY(h2d(M.a, up, up_doubles(g) * sizeof(double), st));
    WM_TRY(h2d(M.np2, np2, sizeof(int) * g.nrows, st));
    WM_TRY(M.mom.ensure(sizeof(double) * mom_doubles(g)));
    AoSView va{M.a.as<double>(), g.np};
    WM_TRY(wm_launch_mom_nvt(g, M.kmom, va, M.np2.as<int>(), M.mom.as<double>(), max_of(np2, (size_t)g.nrows), st));
    WM_TRY(d2h(mom, M.mom, sizeof(double) * mom_doubles(g), st));
    return finish(st);
}

static int bc_init(int kind, int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, double delx,
                   double delt, double c)
{
    WM_TRY(make_geom(M.gbc, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye));
    make_const(M.kbc, nsp, delx, delt, c, nullptr, nullptr, 0.501);
    M.gbc.bc = kind;
    M.bc_kind = kind;
    M.bc_ok = true;
    return WM_OK;
}

// particle_x of the walls (inject = 0) or the shock's injection boundary (inject = 1), x range
// nxs..nxe (the whole grid here)
static int walls_x_dropin(double *up, const int *np2, int nxs, int nxe, int inject, double u0)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    WmGeom g = M.gbc;
    WM_TRY(active_range(g, nxs, nxe, false));
    for (int r = 0; r < g.nrows; ++r)
        if (np2[r] < 0 || np2[r] > g.np) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    const size_t nup = up_doubles(g) * sizeof(double);
    WM_TRY(h2d(M.a, up, nup, st));
    WM_TRY(h2d(M.np2, np2, sizeof(int) * g.nrows, st));
    AoSView va{M.a.as<double>(), g.np};
    WM_TRY(wm_launch_walls_x(g, M.kbc, va, M.np2.as<int>(), max_of(np2, (size_t)g.nrows), inject, u0, st));
    WM_TRY(d2h(up, M.a, nup, st));
    return finish(st);
}

int wm_bc_periodic_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nup,
                        int ndown, int mnpi, int mnpr, int ncomw, int nerr, const int *nstat, int nstat_len, double delx,
                        double delt, double c)
{
    (void)nup, (void)ndown, (void)mnpi, (void)mnpr, (void)ncomw, (void)nerr, (void)nstat, (void)nstat_len;
    return bc_init(WM_BC_PERIODIC, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c);
}

int wm_bc_reconnection_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nup,
                            int ndown, int mnpi, int mnpr, int ncomw, int nerr, const int *nstat, int nstat_len, double delx,
                            double delt, double c)
{
    (void)nup, (void)ndown, (void)mnpi, (void)mnpr, (void)ncomw, (void)nerr, (void)nstat, (void)nstat_len;
    return bc_init(WM_BC_RECONNECTION, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c);
}

int wm_bc_shock_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nup, int ndown,
                     int mnpi, int mnpr, int ncomw, int nerr, const int *nstat, int nstat_len, double delx, double delt, double c)
{
    (void)nup, (void)ndown, (void)mnpi, (void)mnpr, (void)ncomw, (void)nerr, (void)nstat, (void)nstat_len;
    return bc_init(WM_BC_SHOCK, ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye, delx, delt, c);
}

int wm_bc_reconnection_particle_x(double *up, const int *np2, int nxs, int nxe)
{
    if (M.bc_kind != WM_BC_RECONNECTION) return WM_ERR_NOT_INIT;
    return walls_x_dropin(up, np2, nxs, nxe, 0, 0.0);
}

int wm_bc_shock_particle_x(double *up, const int *np2, int nxs, int nxe)
{
    if (M.bc_kind != WM_BC_SHOCK) return WM_ERR_NOT_INIT;
    return walls_x_dropin(up, np2, nxs, nxe, 0, 0.0);
}

int wm_bc_shock_injection(double *up, const int *np2, int nxs, int nxe, double u0)
{
    if (M.bc_kind != WM_BC_SHOCK) return WM_ERR_NOT_INIT;
    return walls_x_dropin(up, np2, nxs, nxe, 1, u0);
}

int wm_bc_periodic_particle_x(double *up, const int *np2)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    const WmGeom &g = M.gbc;
    for (int r = 0; r < g.nrows; ++r)
        if (np2[r] < 0 || np2[r] > g.np) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    const size_t nup = up_doubles(g) * sizeof(double);
    WM_TRY(h2d(M.a, up, nup, st));
    WM_TRY(h2d(M.np2, np2, sizeof(int) * g.nrows, st));
    WM_TRY(M.rb.ensure(1, g));
    AoSView va{M.a.as<double>(), g.np};
    WM_TRY(wm_launch_wrap_classify(g, M.kbc.delx, va, M.np2.as<int>(), max_of(np2, (size_t)g.nrows), 1, M.rb.view(), st));
    WM_TRY(d2h(up, M.a, nup, st));
    return finish(st);
}

int wm_bc_periodic_particle_y(double *up, int *np2)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    const WmGeom &g = M.gbc;
    if ((long long)g.np * g.nrows >= (1LL << 31)) return WM_ERR_UNSUPPORTED;
    for (int r = 0; r < g.nrows; ++r)
        if (np2[r] < 0 || np2[r] > g.np) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    const size_t nup = up_doubles(g) * sizeof(double);
    WM_TRY(h2d(M.a, up, nup, st));
    WM_TRY(h2d(M.np2, np2, sizeof(int) * g.nrows, st));
    WM_TRY(M.rb.ensure((long long)g.np * g.nrows, g));
    WmRebinScratch sc = M.rb.view();
    WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
    const int maxc = max_of(np2, (size_t)g.nrows);
    AoSView va{M.a.as<double>(), g.np};
    WM_TRY(wm_launch_wrap_classify(g, M.kbc.delx, va, M.np2.as<int>(), maxc, 2, sc, st));
    unsigned dev = 0;
    WM_TRY(read_status(sc.status, st, &dev));
    if (map_status(dev) != WM_OK) return map_status(dev);
    WM_TRY(wm_launch_place(g, va, M.np2.as<int>(), maxc, sc, M.rb.drow.as<int>(), st));
    WM_TRY(wm_launch_np2_after_y(g, M.np2.as<int>(), sc, sc.np2_new, g.np, st));
    // the output starts as the wrapped input: slots nothing moves into keep their content
    WM_TRY(M.b.ensure(nup));
    WM_CUDA(cudaMemcpyAsync(M.b.p, M.a.p, nup, cudaMemcpyDeviceToDevice, st));
    AoSView vb{M.b.as<double>(), g.np};
    WM_TRY(wm_launch_scatter_by_P(g, va, vb, M.np2.as<int>(), maxc, sc, M.rb.drow.as<int>(), g.np, st));
    WM_TRY(read_status(sc.status, st, &dev));
    if (map_status(dev) != WM_OK) return map_status(dev);
    WM_TRY(d2h(up, M.b, nup, st));
    WM_CUDA(cudaMemcpyAsync(np2, sc.np2_new, sizeof(int) * g.nrows, cudaMemcpyDeviceToHost, st));
    return finish(st);
}

static int check_range_args(WmGeom &g, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    if (nys != g.nys || nye != g.nye || nxgs != g.nxgs || nxge != g.nxge) return WM_ERR_UNSUPPORTED;
    return active_range(g, nxs, nxe, true);
}

// The ghost routines of the three boundary modules share one implementation each; kind selects
// the x treatment (y is periodic in all three).
static int dfield_impl(int kind, double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    WmGeom g = M.gbc;
    g.bc = kind;
    WM_TRY(check_range_args(g, nxs, nxe, nys, nye, nxgs, nxge));
    WM_TRY(M.stream());
    const size_t bytes = sizeof(double) * 6 * f_points(g);
    WM_TRY(h2d(M.uf_aos, df, bytes, M.st));
    WM_TRY(wm_launch_dfield_bc(g, aos_view<6>(M.uf_aos, g), M.st));
    WM_TRY(d2h(df, M.uf_aos, bytes, M.st));
    return finish(M.st);
}

static int curre_impl(int kind, double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    WmGeom g = M.gbc;
    g.bc = kind;
    WM_TRY(check_range_args(g, nxs, nxe, nys, nye, nxgs, nxge));
    WM_TRY(M.stream());
    const size_t bytes = sizeof(double) * 3 * f_points(g);
    WM_TRY(h2d(M.uf_aos, uj, bytes, M.st));
    WM_TRY(wm_launch_curre_bc(g, aos_view<3>(M.uf_aos, g), M.st));
    WM_TRY(d2h(uj, M.uf_aos, bytes, M.st));
    return finish(M.st);
}

static int phi_impl(int kind, double *phi, int nxs, int nxe, int nys, int nye, int l)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    WmGeom g = M.gbc;
    g.bc = kind;
    if (nys != g.nys || nye != g.nye) return WM_ERR_UNSUPPORTED;
    WM_TRY(active_range(g, nxs, nxe, true));  // phi(nxs-1:nxe+1, nys-1:nye+1)
    if (l < 1 || l > 3) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    const size_t bytes = sizeof(double) * (size_t)(g.nxa + 2) * (g.ny + 2);
    WM_TRY(h2d(M.phi, phi, bytes, M.st));
    WM_TRY(wm_launch_phi_bc(g.nxa, g.ny, M.phi.as<double>(), kind, l, M.st));
    WM_TRY(d2h(phi, M.phi, bytes, M.st));
    return finish(M.st);
}

static int mom_impl(int kind, double *mom)
{
    if (!M.bc_ok) return WM_ERR_NOT_INIT;
    WmGeom g = M.gbc;
    g.bc = kind;
    WM_TRY(M.stream());
    const size_t bytes = sizeof(double) * mom_doubles(g);
    WM_TRY(h2d(M.mom, mom, bytes, M.st));
    WM_TRY(wm_launch_mom_bc(g, M.mom.as<double>(), M.st));
    WM_TRY(d2h(mom, M.mom, bytes, M.st));
    return finish(M.st);
}

int wm_bc_periodic_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    return dfield_impl(WM_BC_PERIODIC, df, nxs, nxe, nys, nye, nxgs, nxge);
}
int wm_bc_periodic_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    return curre_impl(WM_BC_PERIODIC, uj, nxs, nxe, nys, nye, nxgs, nxge);
}
int wm_bc_periodic_phi(double *phi, int nxs, int nxe, int nys, int nye, int l)
{
    return phi_impl(WM_BC_PERIODIC, phi, nxs, nxe, nys, nye, l);
}
int wm_bc_periodic_mom(double *mom) { return mom_impl(WM_BC_PERIODIC, mom); }

int wm_bc_reconnection_particle_y(double *up, int *np2)
{
    if (M.bc_kind != WM_BC_RECONNECTION) return WM_ERR_NOT_INIT;
    return wm_bc_periodic_particle_y(up, np2);  // the same procedure (boundary_reconnection.f90:102-251)
}
int wm_bc_reconnection_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    return dfield_impl(WM_BC_RECONNECTION, df, nxs, nxe, nys, nye, nxgs, nxge);
}
int wm_bc_reconnection_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    return curre_impl(WM_BC_RECONNECTION, uj, nxs, nxe, nys, nye, nxgs, nxge);
}
int wm_bc_reconnection_phi(double *phi, int nxs, int nxe, int nys, int nye, int l)
{
    return phi_impl(WM_BC_RECONNECTION, phi, nxs, nxe, nys, nye, l);
}
int wm_bc_reconnection_mom(double *mom) { return mom_impl(WM_BC_RECONNECTION, mom); }

int wm_bc_shock_particle_y(double *up, int *np2)
{
    if (M.bc_kind != WM_BC_SHOCK) return WM_ERR_NOT_INIT;
    return wm_bc_periodic_particle_y(up, np2);  // the same procedure (boundary_shock.f90:103-252)
}
int wm_bc_shock_dfield(double *df, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    return dfield_impl(WM_BC_SHOCK, df, nxs, nxe, nys, nye, nxgs, nxge);
}
int wm_bc_shock_curre(double *uj, int nxs, int nxe, int nys, int nye, int nxgs, int nxge)
{
    return curre_impl(WM_BC_SHOCK, uj, nxs, nxe, nys, nye, nxgs, nxge);
}
int wm_bc_shock_phi(double *phi, int nxs, int nxe, int nys, int nye, int l)
{
    return phi_impl(WM_BC_SHOCK, phi, nxs, nxe, nys, nye, l);
}
int wm_bc_shock_mom(double *mom) { return mom_impl(WM_BC_SHOCK, mom); }

int wm_energy_sums(const double *up, const double *uf, const int *np2, double *out)
{
    if (!M.particle_ok) return WM_ERR_NOT_INIT;
    const WmGeom &g = M.gpart;
    for (int r = 0; r < g.nrows; ++r)
        if (np2[r] < 0 || np2[r] > g.np) return WM_ERR_BAD_ARG;
    WM_TRY(M.stream());
    cudaStream_t st = M.st;
    const long long npts = (long long)f_points(g);
    WM_TRY(h2d(M.a, up, up_doubles(g) * sizeof(double), st));
    WM_TRY(h2d(M.np2, np2, sizeof(int) * g.nrows, st));
    WM_TRY(h2d(M.uf_aos, uf, sizeof(double) * 6 * npts, st));
    WM_TRY(M.b.ensure(sizeof(double) * 6 * npts));
    WM_TRY(wm_launch_aos_to_soa(6, npts, M.uf_aos.as<double>(), M.b.as<double>(), st));
    const int nb = 152 * 2;
    WM_TRY(M.energy_partial.ensure(sizeof(double) * nb * (g.nsp + 2)));
    WM_TRY(M.energy_out.ensure(sizeof(double) * (g.nsp + 2)));
    AoSView va{M.a.as<double>(), g.np};
    double *part = M.energy_partial.as<double>();
    WM_TRY(wm_launch_energy_particles(g, M.kpart, va, M.np2.as<int>(), part, nb, st));
    WM_TRY(wm_launch_energy_fields(g, FView<6, false>{M.b.as<double>(), g.nxw, g.nyw}, part + (size_t)nb * g.nsp, nb, st));
    WM_TRY(wm_launch_sum_partials(part, nb, g.nsp + 2, M.energy_out.as<double>(), st));
    std::vector<double> tmp(g.nsp + 2);
    WM_CUDA(cudaMemcpyAsync(tmp.data(), M.energy_out.p, sizeof(double) * (g.nsp + 2), cudaMemcpyDeviceToHost, st));
    WM_TRY(finish(st));
    for (int s = 0; s < g.nsp; ++s) out[s] = tmp[s];
    out[g.nsp] = tmp[g.nsp + 1] / (8 * PI_REF);     // efield
    out[g.nsp + 1] = tmp[g.nsp] / (8 * PI_REF);     // bfield
    return WM_OK;
}

int wm_field_cg_iters(int *iters3)
{
    for (int l = 0; l < 3; ++l) iters3[l] = M.last_iters[l];
    return WM_OK;
}

int wm_field_get_work(double *df, double *uj)
{
    if (!M.field_ok) return WM_ERR_NOT_INIT;
    const WmGeom &g = M.gfield;
    WM_TRY(field_work_ready(g));
    const long long npts = (long long)f_points(g);
    WM_TRY(M.uf_aos.ensure(sizeof(double) * 6 * npts));
    if (df) {
        WM_TRY(wm_launch_soa_to_aos(6, npts, M.fb.df.as<double>(), M.uf_aos.as<double>(), M.st));
        WM_CUDA(cudaMemcpyAsync(df, M.uf_aos.p, sizeof(double) * 6 * npts, cudaMemcpyDeviceToHost, M.st));
        WM_TRY(finish(M.st));
    }
    if (uj) {
        WM_TRY(wm_launch_soa_to_aos(3, npts, M.fb.uj.as<double>(), M.uf_aos.as<double>(), M.st));
        WM_CUDA(cudaMemcpyAsync(uj, M.uf_aos.p, sizeof(double) * 3 * npts, cudaMemcpyDeviceToHost, M.st));
        WM_TRY(finish(M.st));
    }
    return WM_OK;
}

int wm_field_set_work(const double *df)
{
    if (!M.field_ok) return WM_ERR_NOT_INIT;
    const WmGeom &g = M.gfield;
    WM_TRY(field_work_ready(g));
    const long long npts = (long long)f_points(g);
    WM_TRY(h2d(M.uf_aos, df, sizeof(double) * 6 * npts, M.st));
    WM_TRY(wm_launch_aos_to_soa(6, npts, M.uf_aos.as<double>(), M.fb.df.as<double>(), M.st));
    return finish(M.st);
}

int wm_finalize(void)
{
    if (M.st) cudaStreamSynchronize(M.st);
    M.release();
    M.particle_ok = M.field_ok = M.sort_ok = M.mom_ok = M.bc_ok = false;
    return WM_OK;
}

const char *wm_status_string(int s)
{
    switch (s) {
    case WM_OK: return "ok";
    case WM_ERR_CG_MAXITER: return "CG reached ite_max";
    case WM_ERR_OVERFLOW: return "particle row overflow (np2 > np)";
    case WM_ERR_BAD_ARG: return "bad argument";
    case WM_ERR_CELL: return "particle outside the grid or moved more than one cell";
    case WM_ERR_CUDA: return "CUDA error";
    case WM_ERR_NOT_INIT: return "module not initialised";
    case WM_ERR_UNSUPPORTED: return "unsupported option";
    case WM_ERR_IO: return "snapshot/output file error";
    default: return "unknown status";
    }
}

const char *wm_build_info(void) { return "wumingpic2d_gb300: sm_103a; precision paths: fp64, mixed"; }

}  // extern "C"
