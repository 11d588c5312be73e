// wm_sim.cu -- the resident simulation: particles and fields stay on the GPU across steps.
//
// Device state (FP64 path):
//   particles  two SoA sets A (up) and B (gp) of x, y, ux, uy, uz (f64) and pid (i64), rows
//              (species-major, then y) stored back to back at rowbase[row], each row sorted by
//              cell with cumcnt in the reference layout;
//   fields     uf, df (6 planes) and uj (3 planes) on the ghosted (nx+4) x (ny+4) grid;
//   work       per-cell partial currents, CG vectors, rebin scratch.
// One step = the main-loop body of proj/weibel/app.f90:102-107:
//   push A->B, deposit(A,B)->uj, field solve, then particle_x + particle_y + sort__bucket fused:
//   classify B (wrap, direction, destination cell), particle_y slots, cell counts -> cumcnt,
//   and one gather B->A into the new cell-sorted order.
// Mixed path: FP32 particles (cell implicit, FP32 offsets and momenta); push + deposit fused,
// FP64 fold, field solve; the new cell order is kept as a slot permutation that the next push
// reads through (or, with WM_REBIN_MOVE, the particles are moved into it), materialize() writes
// the cell-sorted state out for the calls that need it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "wm_launch.cuh"
#include "wm_pio.cuh"
#include "wm_rng.cuh"

namespace {

__global__ void k_unpack(WmGeom g, const double *__restrict__ stage, int pitch, const int *__restrict__ np2, SoAView dst, int row0)
{
    const int row = row0 + blockIdx.y;
    const int n = np2[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const double *a = stage + 6 * ((long long)row * pitch + s);
        const long long p = dst.idx(row, s);
        dst.X(p) = a[0];
        dst.Y(p) = a[1];
        dst.UX(p) = a[2];
        dst.UY(p) = a[3];
        dst.UZ(p) = a[4];
        dst.setpid(p, __double_as_longlong(a[5]));
    }
}

__global__ void k_pack(WmGeom g, SoAView src, const int *__restrict__ np2, int pitch, double *__restrict__ stage, int row0)
{
    const int row = row0 + blockIdx.y;
    const int n = np2[row];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < pitch; s += gridDim.x * blockDim.x) {
        double *a = stage + 6 * ((long long)row * pitch + s);
        if (s < n) {
            const long long p = src.idx(row, s);
            a[0] = src.X(p);
            a[1] = src.Y(p);
            a[2] = src.UX(p);
            a[3] = src.UY(p);
            a[4] = src.UZ(p);
            a[5] = __longlong_as_double(src.getpid(p));
        } else {
            for (int k = 0; k < 6; ++k) a[k] = 0.0;
        }
    }
}

// Pitched copy by the SMs, 16 bytes per access (width and pitches multiples of 16, bases
// 16-byte aligned).  Between device memory and mapped page-locked host memory on a Grace host
// the SMs' loads and stores reach the link's rate, about twice what a pitched copy-engine
// transfer of the same rows gave (rows of a few MB, thousands of rows).
__global__ void k_copy2d(uint4 *__restrict__ dst, size_t dpitch16, const uint4 *__restrict__ src, size_t spitch16, size_t width16,
                         int rows)
{
    for (int r = blockIdx.y; r < rows; r += gridDim.y) {
        const uint4 *s = src + (size_t)r * spitch16;
        uint4 *d = dst + (size_t)r * dpitch16;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < width16; i += (size_t)gridDim.x * blockDim.x) d[i] = s[i];
    }
}

struct Mark {
    const char *name;
    cudaEvent_t ev;
};

}  // namespace

// dst/src pitched rows where one side is host memory: with the SMs when the host buffer is
// mapped into the device's address space (wm_host_alloc, or registered page-locked memory) and
// every size is a multiple of 16 bytes, else with cudaMemcpy2DAsync.
static bool rows_mapped(const void *host, const void *dst, size_t dpitch, const void *src, size_t spitch, size_t width)
{
    void *mapped = nullptr;
    const bool aligned = ((dpitch | spitch | width | (uintptr_t)dst | (uintptr_t)src) & 15) == 0;
    if (aligned && width > 0 && cudaHostGetDevicePointer(&mapped, (void *)host, 0) == cudaSuccess && mapped == host) return true;
    cudaGetLastError();  // a failed mapping query is not an error of the caller
    return false;
}

// k_copy2d over `rows` rows with up to gx x gy CTAs.  Measured on the 2048^2 x 64 ppc state:
// host -> device chunks of 256 rows with 16 x 256 CTAs overlapped with the unpack took 125 ms
// (one full-grid copy then the unpack: 134 ms); device -> host, one full-grid copy after the pack
// took 149 ms, chunks overlapped with the pack 154-158 ms at every grid size tried.
static int launch_copy2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int rows, cudaStream_t st, int gx = 16,
                         int gy = 65535)
{
    if (rows <= 0) return WM_OK;
    const size_t w16 = width / 16;
    dim3 grid((unsigned)std::min<size_t>((w16 + 255) / 256, gx), (unsigned)std::min(rows, gy));
    k_copy2d<<<grid, 256, 0, st>>>((uint4 *)dst, dpitch / 16, (const uint4 *)src, spitch / 16, w16, rows);
    return wm_check_launch("k_copy2d");
}

static int copy_rows(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int rows, bool to_host, cudaStream_t st)
{
    if (rows > 0 && rows_mapped(to_host ? dst : src, dst, dpitch, src, spitch, width)) return launch_copy2d(dst, dpitch, src, spitch, width, rows, st);
    WM_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice, st));
    return WM_OK;
}

struct wm_sim {
    WmGeom g{};
    WmConst k{};
    int precision = WM_PREC_FP64;
    double u0 = 0.0;  // shock: upstream four-velocity of the injection boundary
    long long cap_req = 0, cap = 0, ntot = 0;
    cudaStream_t st = nullptr;
    DevBuf A[6], B[6];
    DevBuf rowbase[2], np2[2], cumcnt, stage, uf_aos, energy_partial, energy_out, jtile, fcc, stage2;
    DevBuf cumcnt_alt, mx_cnt9, mx_off9;  // mixed path: new cumcnt, per-cell direction counts and offsets
    DevBuf mx_ovf;                        // mixed path: tiles of the push to recompute (queue overflow)
    // Mixed path, rebin by permutation (the default): after a step, set A holds the push output
    // and slot p of the cell-sorted order is at slot mx_perm[p] of A ("permuted"), its id at slot
    // mx_idperm[idp][p] of A[5] (the ids do not move while permuted); the next push reads through
    // mx_perm, and materialize() writes the cell-sorted order out when anything else needs it.
    // rebin_move = true moves the particles every step instead (k_mixed_move).
    DevBuf mx_perm, mx_idperm[2];
    int idp = 0;
    bool permuted = false, rebin_move = false;
    DevBuf mom_dev, out_dev, out_cnt;     // moments and the file-ordered data of the paraio outputs
    // shock application: particles entering at the right boundary every step (off until set)
    bool inject_on = false;
    WmInjectArgs inj{};
    long long it = 0;  // steps taken: the counter of the injection draws
    // the shock box's expansion (proj/shock/app.f90:123-125, relocate :613-690): every
    // expand_every steps (0: never), after the injection, nxe (g.nxa) grows by one cell and
    // inj_n0 particles per row and species enter the new cell
    int expand_every = 0, inj_n0 = 0;
    bool expanding_now() const { return inject_on && expand_every > 0 && (it + 1) % expand_every == 0 && g.nxa < g.nx; }
    // the injection boundary at the active nxe: cell nxe-1 counts the new particles, x = nxe dx
    void sync_inject_boundary()
    {
        inj.cell = g.nxa - 2;
        inj.xe = (g.nxgs + g.nxa - 1) * k.delx;
        inj.n_expand = expanding_now() ? inj_n0 : 0;
    }
    // after this step's injection: the expansion's particles (on stream s), then, once the field
    // update has run (finish_expansion), nxe moves on and the new boundary columns take the
    // upstream field
    template <class PV>
    int expand_write(PV dst, int *np2_new, int *cumcnt_new, cudaStream_t s, unsigned *perm = nullptr, unsigned *idperm = nullptr,
                     const long long *phys0 = nullptr)
    {
        if (inj.n_expand == 0) return WM_OK;
        return wm_launch_expand_particles(g, inj, dst, np2_new, cumcnt_new, inj_rows.as<int>(), inj_ninc.as<long long>(),
                                          inj_nptot.as<long long>(), s, perm, idperm, phys0);
    }
    int finish_expansion()
    {
        if (inj.n_expand == 0) return WM_OK;
        g.nxa += 1;
        inj.cell = g.nxa - 2;
        inj.xe = (g.nxgs + g.nxa - 1) * k.delx;
        inj.n_expand = 0;
        return wm_launch_inject_fields(g, inj, uf(), st);
    }
    DevBuf inj_rows, inj_ninc, inj_nptot, inj_tmp;
    // host -> device particle rows in chunks on a second stream, overlapped with the unpack
    // kernels on the main one (host buffers mapped into the device's address space)
    static constexpr int XFER_CHUNKS = 16;
    cudaStream_t st2 = nullptr;
    cudaEvent_t xev[XFER_CHUNKS + 1] = {};
    int xfer_setup()
    {
        if (!st2) {
            int least = 0, greatest = 0;
            WM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            WM_CUDA(cudaStreamCreateWithPriority(&st2, cudaStreamNonBlocking, least));
        }
        for (cudaEvent_t &e : xev)
            if (!e) WM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        return WM_OK;
    }
    // learned CG guess (off until wm_sim_set_guess)
    DevBuf cnn_params, cnn_wf[WM_CNN_LAYERS], cnn_x, cnn_a0, cnn_a1, cnn_pred, cnn_partial, cnn_scale, guess_cand, guess_stats;
    WmCnnNet net{};
    WmGuess gdesc{};
    bool guess_on = false;
    int cur = 0;  // index of the current rowbase/np2
    // field and rebin work
    DevBuf f_uf, f_uj, f_df, f_pj, f_b, f_r, f_p, f_ap, f_partial, f_ticket, f_scal;
    CgScal *scal_host = nullptr;
    DevBuf rb_dir, rb_ord, rb_P, rb_key, rb_holes, rb_nup, rb_ndown, rb_cellcnt, rb_pairs, rb_status;
    unsigned *status_host = nullptr;
    int iters[3] = {0, 0, 0};
    int max_row = 1;
    bool loaded = false;
    // timing
    bool timing = false;
    std::vector<Mark> marks;
    size_t nmarks = 0;
    // the mixed step's rebin runs on a second stream beside the field solve: its events, and the
    // timing marks recorded on that stream
    cudaEvent_t rb_push_done = nullptr, rb_done = nullptr;
    std::vector<Mark> smarks;
    size_t nsmarks = 0;
    std::vector<const char *> t_names;
    std::vector<double> t_ms;
    long long launches = 0;

    SoAView view(DevBuf *S, int rb) const
    {
        SoAView v;
        v.x = S[0].as<double>();
        v.y = S[1].as<double>();
        v.ux = S[2].as<double>();
        v.uy = S[3].as<double>();
        v.uz = S[4].as<double>();
        v.pid = S[5].as<long long>();
        v.rowbase = rowbase[rb].as<long long>();
        return v;
    }
    bool mixed() const { return precision == WM_PREC_MIXED; }
    // Mixed path: the push does not touch the ids; the sort gathers them from the id buffer of the
    // old order (pid_cur) into the other one, so the two id buffers alternate every step.
    int pid_cur = 0;  // 0: A[5] holds the ids of the current order, 1: B[5]
    MixedView mview(DevBuf *S, int rb, int pidw = -1) const
    {
        MixedView v;
        v.xyuv = S[0].as<float4>();
        v.uz = S[4].as<float>();
        v.pid = (pidw < 0 ? S[5] : (pidw == 0 ? A[5] : B[5])).as<long long>();
        v.rowbase = rowbase[rb].as<long long>();
        return v;
    }
    WmRebinScratch scratch() const
    {
        WmRebinScratch s;
        s.dir = rb_dir.as<unsigned char>();
        s.ord = rb_ord.as<int>();
        s.P = rb_P.as<int>();
        s.key = rb_key.as<int>();
        s.holes = rb_holes.as<int>();
        s.nup = rb_nup.as<int>();
        s.ndown = rb_ndown.as<int>();
        s.cellcnt = rb_cellcnt.as<int>();
        s.pairs = rb_pairs.as<unsigned long long>();
        s.np2_new = np2[1 - cur].as<int>();
        s.rowbase_new = rowbase[1 - cur].as<long long>();
        s.status = rb_status.as<unsigned>();
        return s;
    }
    WmFieldWork work()
    {
        WmFieldWork w;
        w.b = f_b.as<double>();
        w.r = f_r.as<double>();
        w.p = f_p.as<double>();
        w.ap = f_ap.as<double>();
        w.partial = f_partial.as<double>();
        w.ticket = f_ticket.as<unsigned>();
        w.scal = f_scal.as<CgScal>();
        w.scal_host = scal_host;
        return w;
    }
    FView<6, false> uf() const { return FView<6, false>{f_uf.as<double>(), g.nxw, g.nyw}; }
    FView<6, false> df() const { return FView<6, false>{f_df.as<double>(), g.nxw, g.nyw}; }
    FView<3, false> uj() const { return FView<3, false>{f_uj.as<double>(), g.nxw, g.nyw}; }
    const WmGuess *guess() const { return guess_on ? &gdesc : nullptr; }
    static int guess_run(void *ctx, cudaStream_t stream)
    {
        wm_sim *s = static_cast<wm_sim *>(ctx);
        const WmCnnWork w{s->cnn_x.p, s->cnn_a0.p, s->cnn_a1.p, s->cnn_pred.as<float>(), s->cnn_partial.as<double>(), s->cnn_scale.as<double>()};
        return wm_cnn_infer_guess(s->g, s->net, s->uf(), s->uj(), w, s->guess_cand.as<double>(), stream, s->rb_status.as<unsigned>());
    }

    void mark(const char *name)
    {
        if (!timing) return;
        if (nmarks == marks.size()) {
            Mark m{name, nullptr};
            cudaEventCreate(&m.ev);
            marks.push_back(m);
        }
        marks[nmarks].name = name;
        cudaEventRecord(marks[nmarks].ev, st);
        ++nmarks;
    }
    static void mark_cb(void *self, const char *name) { static_cast<wm_sim *>(self)->mark(name); }
    void smark(const char *name)  // a timing mark on the rebin's stream
    {
        if (!timing) return;
        if (nsmarks == smarks.size()) {
            Mark m{name, nullptr};
            cudaEventCreate(&m.ev);
            smarks.push_back(m);
        }
        smarks[nsmarks].name = name;
        cudaEventRecord(smarks[nsmarks].ev, st2);
        ++nsmarks;
    }
    // phase events of the host-buffer path (load and store), recorded only with timing on
    std::vector<Mark> phases;
    size_t nphases = 0;
    void pmark(const char *name)
    {
        if (!timing) return;
        if (nphases == phases.size()) {
            Mark m{name, nullptr};
            cudaEventCreate(&m.ev);
            phases.push_back(m);
        }
        phases[nphases].name = name;
        cudaEventRecord(phases[nphases].ev, st);
        ++nphases;
    }

    int alloc(long long capacity)
    {
        const size_t nf = (size_t)g.nxw * g.nyw, nc = (size_t)g.nx * g.ny;
        cap = capacity;
        for (int c = 0; c < 6; ++c) {  // mixed: the (dx, dy, ux, uy) records in [0], the uz plane in [4], the i64 pid
            const size_t esz = !mixed() ? 8 : c == 0 ? 16 : c == 4 ? 4 : c == 5 ? 8 : 0;
            if (esz == 0) continue;
            WM_TRY(A[c].ensure(esz * (size_t)cap));
            WM_TRY(B[c].ensure(esz * (size_t)cap));
        }
        if (mixed()) {
            WM_TRY(jtile.ensure(sizeof(float) * wm_mixed_jtile_floats(g)));
            WM_TRY(fcc.ensure(sizeof(float) * wm_mixed_fcc_floats(g)));
            WM_TRY(cumcnt_alt.ensure(sizeof(int) * (size_t)(g.nx + 1) * g.nrows));
            WM_TRY(mx_cnt9.ensure(sizeof(int) * 9 * (size_t)g.nx * g.nrows));
            WM_TRY(mx_ovf.ensure(sizeof(unsigned) * wm_mixed_ovf_words(g)));
            WM_TRY(mx_off9.ensure(sizeof(int) * 9 * (size_t)g.nx * g.nrows));
            if (cap < (1LL << 32)) {
                WM_TRY(mx_perm.ensure(sizeof(unsigned) * (size_t)cap));
                for (DevBuf &b : mx_idperm) WM_TRY(b.ensure(sizeof(unsigned) * (size_t)cap));
            }
        }
        permuted = false;
        for (int c = 0; c < 2; ++c) {
            WM_TRY(rowbase[c].ensure(sizeof(long long) * (g.nrows + 1)));
            WM_TRY(np2[c].ensure(sizeof(int) * g.nrows));
        }
        WM_TRY(cumcnt.ensure(sizeof(int) * (size_t)(g.nx + 1) * g.nrows));
        WM_TRY(f_uf.ensure(sizeof(double) * 6 * nf));
        WM_TRY(f_df.ensure(sizeof(double) * 6 * nf));
        WM_TRY(f_uj.ensure(sizeof(double) * 3 * nf));
        WM_TRY(f_pj.ensure(sizeof(double) * 75 * nc));
        WM_TRY(f_b.ensure(sizeof(double) * 3 * nc));
        WM_TRY(f_r.ensure(sizeof(double) * 3 * nc));
        WM_TRY(f_p.ensure(sizeof(double) * 3 * nc));
        WM_TRY(f_ap.ensure(sizeof(double) * 3 * nc));
        WM_TRY(f_partial.ensure(sizeof(double) * 6 * wm_field_cg_blocks()));  // 6 sums: the two guesses' residuals
        WM_TRY(f_ticket.ensure(sizeof(unsigned)));
        WM_CUDA(cudaMemsetAsync(f_ticket.p, 0, sizeof(unsigned), st));
        WM_TRY(f_scal.ensure(wm_field_scal_bytes()));
        WM_TRY(rb_dir.ensure((size_t)cap));
        WM_TRY(rb_ord.ensure(4 * (size_t)cap));
        WM_TRY(rb_P.ensure(4 * (size_t)cap));
        WM_TRY(rb_key.ensure(4 * (size_t)cap));
        WM_TRY(rb_holes.ensure(4 * (size_t)cap));
        WM_TRY(rb_pairs.ensure(8 * (size_t)cap));
        WM_TRY(rb_nup.ensure(sizeof(int) * g.nrows));
        WM_TRY(rb_ndown.ensure(sizeof(int) * g.nrows));
        WM_TRY(rb_cellcnt.ensure(sizeof(int) * (size_t)g.nrows * g.nx));
        WM_TRY(rb_status.ensure(sizeof(unsigned)));
        WM_TRY(energy_partial.ensure(sizeof(double) * 304 * (g.nsp + 2)));
        WM_TRY(energy_out.ensure(sizeof(double) * (g.nsp + 2)));
        return WM_OK;
    }

    size_t device_bytes() const
    {
        size_t t = 0;
        for (int c = 0; c < 6; ++c) t += A[c].bytes + B[c].bytes;
        for (const DevBuf *b : {&rowbase[0], &rowbase[1], &np2[0], &np2[1], &cumcnt, &stage, &uf_aos, &jtile, &fcc, &cumcnt_alt, &mx_cnt9, &mx_off9, &mx_ovf, &mx_perm, &mx_idperm[0], &mx_idperm[1], &f_uf, &f_uj, &f_df, &f_pj,
                                &f_b, &f_r, &f_p, &f_ap, &f_partial, &rb_dir, &rb_ord, &rb_P, &rb_key, &rb_holes, &rb_nup,
                                &rb_ndown, &rb_cellcnt, &rb_pairs})
            t += b->bytes;
        return t;
    }

    void release()
    {
        if (st) cudaStreamSynchronize(st);
        for (int c = 0; c < 6; ++c) {
            A[c].release();
            B[c].release();
        }
        for (DevBuf *b : {&rowbase[0], &rowbase[1], &np2[0], &np2[1], &cumcnt, &stage, &uf_aos, &energy_partial, &energy_out, &jtile, &fcc, &cumcnt_alt, &mx_cnt9, &mx_off9, &mx_ovf, &mx_perm, &mx_idperm[0], &mx_idperm[1], &stage2,
                          &mom_dev, &out_dev, &out_cnt, &inj_rows, &inj_ninc, &inj_nptot, &inj_tmp,
                          &f_uf, &f_uj, &f_df, &f_pj, &f_b, &f_r, &f_p, &f_ap, &f_partial, &f_ticket, &f_scal, &rb_dir, &rb_ord,
                          &rb_P, &rb_key, &rb_holes, &rb_nup, &rb_ndown, &rb_cellcnt, &rb_pairs, &rb_status})
            b->release();
        for (DevBuf *b : {&cnn_params, &cnn_x, &cnn_a0, &cnn_a1, &cnn_pred, &cnn_partial, &cnn_scale, &guess_cand, &guess_stats})
            b->release();
        for (DevBuf &b : cnn_wf) b.release();
        guess_on = false;
        for (Mark &m : marks) cudaEventDestroy(m.ev);
        marks.clear();
        for (Mark &m : smarks) cudaEventDestroy(m.ev);
        smarks.clear();
        for (cudaEvent_t *e : {&rb_push_done, &rb_done})
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
        for (Mark &m : phases) cudaEventDestroy(m.ev);
        phases.clear();
        if (scal_host) cudaFreeHost(scal_host);
        if (status_host) cudaFreeHost(status_host);
        scal_host = nullptr;
        status_host = nullptr;
        if (st) cudaStreamDestroy(st);
        st = nullptr;
        if (st2) {
            cudaStreamSynchronize(st2);
            cudaStreamDestroy(st2);
        }
        st2 = nullptr;
        for (cudaEvent_t &e : xev) {
            if (e) cudaEventDestroy(e);
            e = nullptr;
        }
    }

    int check_status()
    {
        WM_CUDA(cudaMemcpyAsync(status_host, rb_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        WM_CUDA(cudaStreamSynchronize(st));
        const unsigned d = *status_host;
        if (d & WMDEV_TIMEOUT) return WM_ERR_CUDA;  // a bounded wait inside a kernel ran out
        if (d & WMDEV_OVERFLOW) return WM_ERR_OVERFLOW;
        if (d & (WMDEV_CELL | WMDEV_ROWJUMP)) return WM_ERR_CELL;
        return WM_OK;
    }

    // Upload a reference-layout particle array (np slots per row, np2 used) into set S.
    // up: host rows of `host_pitch` slots (6 doubles each); the reference layout has np slots
    // up == nullptr: the rows are already in `stage` with pitch = the largest row count
    int upload_particles(const double *up, const int *np2_h, DevBuf *S, int host_pitch)
    {
        const int maxc = std::max(1, *std::max_element(np2_h, np2_h + g.nrows));
        if (maxc > g.np || maxc > host_pitch) return WM_ERR_BAD_ARG;
        permuted = false;  // the state is replaced
        const size_t rowb = sizeof(double) * 6 * maxc, hrowb = sizeof(double) * 6 * host_pitch;
        bool piped = false;
        if (up) {
            WM_TRY(stage.ensure(rowb * g.nrows));
            piped = rows_mapped(up, stage.p, rowb, up, hrowb, rowb);
            if (!piped) WM_TRY(copy_rows(stage.p, rowb, up, hrowb, rowb, g.nrows, false, st));
        }
        WM_CUDA(cudaMemcpyAsync(np2[cur].p, np2_h, sizeof(int) * g.nrows, cudaMemcpyHostToDevice, st));
        WM_TRY(wm_launch_rowbase(g.nrows, np2[cur].as<int>(), rowbase[cur].as<long long>(), st));
        WmRebinScratch sc = scratch();
        if (mixed()) WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
        // mixed: offsets against int(x) and the row, also the load-sort keys and counts
        auto unpack = [&](int r0, int nr) -> int {
            if (mixed()) return wm_launch_mixed_unpack(g, stage.as<double>(), maxc, np2[cur].as<int>(), mview(S, cur), sc, st, r0, nr);
            dim3 grid(std::min(wm_div_up(maxc, 256), 64u), nr);
            k_unpack<<<grid, 256, 0, st>>>(g, stage.as<double>(), maxc, np2[cur].as<int>(), view(S, cur), r0);
            return wm_check_launch("k_unpack");
        };
        if (piped) {  // chunk c's copy on st2, its unpack on st once the copy is in
            WM_TRY(xfer_setup());
            WM_CUDA(cudaEventRecord(xev[XFER_CHUNKS], st));
            WM_CUDA(cudaStreamWaitEvent(st2, xev[XFER_CHUNKS], 0));
            const int per = (g.nrows + XFER_CHUNKS - 1) / XFER_CHUNKS;
            for (int c = 0, r0 = 0; r0 < g.nrows; ++c, r0 += per) {
                const int nr = std::min(per, g.nrows - r0);
                WM_TRY(launch_copy2d((char *)stage.p + r0 * rowb, rowb, (const char *)up + r0 * hrowb, hrowb, rowb, nr, st2, 16, 256));
                WM_CUDA(cudaEventRecord(xev[c], st2));
                WM_CUDA(cudaStreamWaitEvent(st, xev[c], 0));
                WM_TRY(unpack(r0, nr));
            }
        } else {
            pmark("copy_in_h2d");
            WM_TRY(unpack(0, g.nrows));
        }
        max_row = maxc;
        pmark("copy_in_particles");
        return WM_OK;
    }

    int upload_fields(const double *uf_h)
    {
        const long long npts = (long long)g.nxw * g.nyw;
        WM_TRY(uf_aos.ensure(sizeof(double) * 6 * npts));
        WM_CUDA(cudaMemcpyAsync(uf_aos.p, uf_h, sizeof(double) * 6 * npts, cudaMemcpyHostToDevice, st));
        return wm_launch_aos_to_soa(6, npts, uf_aos.as<double>(), f_uf.as<double>(), st);
    }

    // sort__bucket of set B into set A (load path)
    int sort_B_into_A()
    {
        WmRebinScratch sc = scratch();
        if (mixed()) {  // keys and counts came from the unpack
            MixedView vb = mview(B, cur);
            WM_TRY(wm_launch_slot_as_P(g, vb, np2[cur].as<int>(), max_row, sc, st));
            WM_TRY(wm_launch_scan_cells(g, sc, cumcnt.as<int>(), sc.np2_new, st));
            WM_TRY(check_status());
            WM_TRY(wm_launch_rowbase(g.nrows, sc.np2_new, sc.rowbase_new, st));
            WM_TRY(wm_launch_sort_move(g, vb, mview(A, 1 - cur), np2[cur].as<int>(), max_row, cumcnt.as<int>(), sc, st));
            cur = 1 - cur;
            pid_cur = 0;
            return WM_OK;
        }
        WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
        SoAView vb = view(B, cur);
        WM_TRY(wm_launch_wrap_classify(g, k.delx, vb, np2[cur].as<int>(), max_row, 8, sc, st));
        WM_TRY(wm_launch_slot_as_P(g, vb, np2[cur].as<int>(), max_row, sc, st));
        WM_TRY(wm_launch_scan_cells(g, sc, cumcnt.as<int>(), sc.np2_new, st));
        WM_TRY(check_status());
        WM_TRY(wm_launch_rowbase(g.nrows, sc.np2_new, sc.rowbase_new, st));
        WM_TRY(wm_launch_sort_move(g, vb, view(A, 1 - cur), np2[cur].as<int>(), max_row, cumcnt.as<int>(), sc, st));
        cur = 1 - cur;
        return WM_OK;
    }

    // The mixed-precision step: FP32 push + deposit with the wrap, keys and counts fused in one
    // kernel; FP64 current fold, field solve and the same particle_y / sort permutation.
    // Injection, first half (after the new row counts exist): this step's counts per row and the
    // new row bases with room behind each row for them.  Without injection: the plain row bases.
    int rowbases(WmRebinScratch &sc) { return rowbases(sc, st); }
    int rowbases(WmRebinScratch &sc, cudaStream_t s)
    {
        if (!inject_on) return wm_launch_rowbase(g.nrows, sc.np2_new, sc.rowbase_new, s);
        inj.it = (int)it;
        inj.cap = cap;
        sync_inject_boundary();
        WM_TRY(wm_launch_inject_counts(g, inj, sc.np2_new, inj_rows.as<int>(), inj_ninc.as<long long>(), inj_nptot.as<long long>(),
                                       sc.status, s));
        WM_TRY(wm_launch_inject_reserve(g, inj, sc.np2_new, inj_rows.as<int>(), inj_tmp.as<int>(), s));
        return wm_launch_rowbase(g.nrows, inj_tmp.as<int>(), sc.rowbase_new, s);
    }
    // second half (after the move): the new particles behind the sorted ones, np2 and cumcnt
    // advanced (proj/shock/app.f90:829-848), and the upstream field at the boundary columns
    template <class PV>
    int inject_write(PV dst, int *cumcnt_new, WmRebinScratch &sc)
    {
        if (!inject_on) return WM_OK;
        WM_TRY(wm_launch_inject_particles(g, inj, dst, sc.np2_new, cumcnt_new, inj_rows.as<int>(), inj_ninc.as<long long>(),
                                          inj_nptot.as<long long>(), st));
        WM_TRY(expand_write(dst, sc.np2_new, cumcnt_new, st));
        WM_TRY(wm_launch_inject_fields(g, inj, uf(), st));
        return finish_expansion();
    }

    // The cell-sorted state in set A again (ids in A[5]): gather the push output through mx_perm
    // and the ids through mx_idperm into set B and exchange the two sets.
    int materialize()
    {
        if (!permuted) return WM_OK;
        WM_TRY(wm_launch_mixed_gather(g, mview(A, cur), mview(B, cur), mx_perm.as<unsigned>(), mx_idperm[idp].as<unsigned>(), np2[cur].as<int>(),
                                      max_row, st));
        ++launches;
        for (int c = 0; c < 6; ++c) std::swap(A[c], B[c]);
        permuted = false;
        pid_cur = 0;
        return WM_OK;
    }

    int step_mixed()
    {
        if (!rebin_move && cap < (1LL << 32)) return step_mixed_perm();
        WM_TRY(materialize());
        WmRebinScratch sc = scratch();
        long long nl = 0;
        WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
        mark("start");
        MixedView va = mview(A, cur), vb = mview(B, cur);
        WM_TRY(wm_launch_mixed_fields(g, uf(), fcc.as<float>(), st));
        ++nl;
        mark("fields");
        WM_TRY(wm_launch_mixed_push_deposit(g, k, va, vb, nullptr, fcc.as<float>(), cumcnt.as<int>(), sc, mx_cnt9.as<int>(), jtile.as<float>(), mx_ovf.as<unsigned>(), st));
        ++nl;
        mark("push_deposit");
        WM_TRY(wm_launch_mixed_jfold(g, jtile.as<float>(), uj(), st));
        ++nl;
        mark("deposit");
        WmFieldWork w = work();
        const int s = wm_field_solve(g, k, uf(), uj(), df(), w, iters, 4, st, timing ? &wm_sim::mark_cb : nullptr, this, &nl, guess());
        if (s != WM_OK) return s;
        // the push counted each cell's particles per direction: destination counts and offsets,
        // the new cumcnt (into the second buffer) and row bases, then one move into the new order
        WM_TRY(wm_launch_mixed_incoming(g, mx_cnt9.as<int>(), mx_off9.as<int>(), sc, st));
        WM_TRY(wm_launch_scan_cells(g, sc, cumcnt_alt.as<int>(), sc.np2_new, st));
        WM_TRY(rowbases(sc));
        nl += inject_on ? 5 : 3;
        mark("scan");
        WM_TRY(wm_launch_mixed_move(g, mview(B, cur, pid_cur), mview(A, 1 - cur, 1 - pid_cur), cumcnt.as<int>(), cumcnt_alt.as<int>(),
                                    mx_off9.as<int>(), sc, st));
        ++nl;
        mark("sort_move");
        WM_TRY(inject_write(mview(A, 1 - cur, 1 - pid_cur), cumcnt_alt.as<int>(), sc));
        if (inject_on) {
            nl += 3;
            mark("inject");
        }
        std::swap(cumcnt, cumcnt_alt);
        cur = 1 - cur;
        pid_cur = 1 - pid_cur;
        ++it;
        launches += nl;
        return check_status();
    }

    // The same step with the rebin as a permutation: the push reads its particles through mx_perm
    // (when the state is permuted) and writes them to set B in the cell order of the step's start;
    // k_mixed_perm records where each particle of the new order is (and where its id is: the ids
    // stay in A[5]); the position sets then exchange roles.  The particles, their order and every
    // result are those of the move.
    int step_mixed_perm()
    {
        WmRebinScratch sc = scratch();
        long long nl = 0;
        WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
        mark("start");
        if (pid_cur != 0) {  // the ids of the current order live with the positions in set A
            std::swap(A[5], B[5]);
            pid_cur = 0;
        }
        const bool gather = permuted;
        MixedView va = mview(A, cur), vb = mview(B, cur);
        WM_TRY(wm_launch_mixed_fields(g, uf(), fcc.as<float>(), st));
        ++nl;
        mark("fields");
        WM_TRY(wm_launch_mixed_push_deposit(g, k, va, vb, gather ? mx_perm.as<unsigned>() : nullptr, fcc.as<float>(), cumcnt.as<int>(), sc,
                                            mx_cnt9.as<int>(), jtile.as<float>(), mx_ovf.as<unsigned>(), st));
        ++nl;
        mark("push_deposit");
        // The rebin needs the push's counts and codes only: destination counts, scan, row bases and
        // the permutations run on the second stream while this one folds the current and solves
        // the fields (FP64-bound work beside memory-bound work); the next push waits for both.
        WM_TRY(xfer_setup());
        if (!rb_push_done) WM_CUDA(cudaEventCreateWithFlags(&rb_push_done, cudaEventDisableTiming));
        if (!rb_done) WM_CUDA(cudaEventCreateWithFlags(&rb_done, cudaEventDisableTiming));
        WM_CUDA(cudaEventRecord(rb_push_done, st));
        WM_CUDA(cudaStreamWaitEvent(st2, rb_push_done, 0));
        smark("start");
        int rs = wm_launch_mixed_incoming(g, mx_cnt9.as<int>(), mx_off9.as<int>(), sc, st2);
        if (rs == WM_OK) rs = wm_launch_scan_cells(g, sc, cumcnt_alt.as<int>(), sc.np2_new, st2);
        if (rs == WM_OK) rs = rowbases(sc, st2);
        smark("scan");
        if (rs == WM_OK)
            rs = wm_launch_mixed_perm(g, rowbase[cur].as<long long>(), sc.rowbase_new, cumcnt.as<int>(), cumcnt_alt.as<int>(), mx_off9.as<int>(),
                                      sc, mx_perm.as<unsigned>(), gather ? mx_idperm[idp].as<unsigned>() : nullptr,
                                      mx_idperm[1 - idp].as<unsigned>(), st2);
        smark("sort_perm");
        if (rs == WM_OK && inject_on)  // the new particles past the push output (positions in B, ids in A[5]), their slots in the permutations
            rs = wm_launch_inject_particles(g, inj, mview(B, 1 - cur, 0), sc.np2_new, cumcnt_alt.as<int>(), inj_rows.as<int>(),
                                            inj_ninc.as<long long>(), inj_nptot.as<long long>(), st2, mx_perm.as<unsigned>(),
                                            mx_idperm[1 - idp].as<unsigned>(), rowbase[cur].as<long long>() + g.nrows);
        if (rs == WM_OK && inject_on)  // the box's expansion: its particles past the injected ones
            rs = expand_write(mview(B, 1 - cur, 0), sc.np2_new, cumcnt_alt.as<int>(), st2, mx_perm.as<unsigned>(),
                              mx_idperm[1 - idp].as<unsigned>(), rowbase[cur].as<long long>() + g.nrows);
        WM_CUDA(cudaEventRecord(rb_done, st2));
        nl += (inject_on ? 7 : 4);
        WM_TRY(wm_launch_mixed_jfold(g, jtile.as<float>(), uj(), st));
        ++nl;
        mark("deposit");
        WmFieldWork w = work();
        const int s = wm_field_solve(g, k, uf(), uj(), df(), w, iters, 4, st, timing ? &wm_sim::mark_cb : nullptr, this, &nl, guess());
        WM_CUDA(cudaStreamWaitEvent(st, rb_done, 0));  // (also when the solve failed: no work of this step left in flight)
        if (s != WM_OK) return s;
        WM_TRY(rs);
        if (inject_on) {  // the upstream field at the boundary columns, after the solve's field update
            WM_TRY(wm_launch_inject_fields(g, inj, uf(), st));
            ++nl;
            if (inj.n_expand) nl += 3;
            WM_TRY(finish_expansion());
        }
        mark("rebin_wait");
        // set B now holds the pushed particles in the old cell order: it becomes set A (the ids
        // stay in A[5], reached through the new idperm)
        for (int c = 0; c < 5; ++c) std::swap(A[c], B[c]);
        idp = 1 - idp;
        std::swap(cumcnt, cumcnt_alt);
        cur = 1 - cur;
        permuted = true;
        ++it;
        launches += nl;
        return check_status();
    }

    int step_once()
    {
        if (mixed()) return step_mixed();
        WmRebinScratch sc = scratch();
        long long nl = 0;
        WM_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(unsigned), st));
        mark("start");
        SoAView va = view(A, cur), vb = view(B, cur);
        WM_TRY(wm_launch_push(g, k, va, vb, uf(), cumcnt.as<int>(), 0, 1, st));
        ++nl;
        if (g.bc == WM_BC_SHOCK) {  // proj/shock/app.f90:112-117: the injection boundary before the field solve
            WM_TRY(wm_launch_walls_x(g, k, vb, np2[cur].as<int>(), max_row, 1, u0, st));
            ++nl;
        }
        mark("push");
        WM_TRY(wm_launch_deposit_cells(g, k, va, vb, cumcnt.as<int>(), f_pj.as<double>(), sc.status, st));
        WM_TRY(wm_launch_deposit_fold(g, uj(), f_pj.as<double>(), st));
        nl += 2;
        mark("deposit");
        WmFieldWork w = work();
        const int s = wm_field_solve(g, k, uf(), uj(), df(), w, iters, 4, st, timing ? &wm_sim::mark_cb : nullptr, this, &nl, guess());
        if (s != WM_OK) return s;
        // particle_x of the application (periodic wrap, the reconnection walls, none in the shock
        // loop), particle_y, and the sort keys
        const int xmode = g.bc == WM_BC_PERIODIC ? 1 : (g.bc == WM_BC_RECONNECTION ? 16 : 0);
        WM_TRY(wm_launch_wrap_classify(g, k.delx, vb, np2[cur].as<int>(), max_row, xmode | 2 | 4, sc, st));
        nl += 1;
        mark("classify");
        WM_TRY(wm_launch_scan_cells(g, sc, cumcnt.as<int>(), sc.np2_new, st));
        WM_TRY(rowbases(sc));
        nl += inject_on ? 4 : 2;
        mark("scan");
        WM_TRY(wm_launch_place_sort(g, vb, view(A, 1 - cur), np2[cur].as<int>(), max_row, cumcnt.as<int>(), sc, st));
        nl += 3;
        mark("sort_move");
        WM_TRY(inject_write(view(A, 1 - cur), cumcnt.as<int>(), sc));
        if (inject_on) {
            nl += 3;
            mark("inject");
        }
        cur = 1 - cur;
        ++it;
        launches += nl;
        return check_status();
    }
};

extern "C" {

int wm_sim_create(const wm_sim_config *cfg, wm_sim **out)
{
    if (!cfg || !out) return WM_ERR_BAD_ARG;
    *out = nullptr;
    if (cfg->precision != WM_PREC_FP64 && cfg->precision != WM_PREC_MIXED) return WM_ERR_BAD_ARG;
    if (cfg->nsp < 1 || cfg->nsp > WM_MAX_SP || cfg->nx < 4 || cfg->ny < 4 || cfg->np < 1) return WM_ERR_BAD_ARG;
    if (cfg->cg_itemax < 1 || !(cfg->cg_err > 0)) return WM_ERR_BAD_ARG;
    if (cfg->bc != WM_BC_PERIODIC && cfg->bc != WM_BC_RECONNECTION && cfg->bc != WM_BC_SHOCK) return WM_ERR_BAD_ARG;
    wm_sim *s = new wm_sim();
    WmGeom &g = s->g;
    g.bc = cfg->bc;
    s->u0 = cfg->u0;
    s->k.u0 = cfg->u0;
    g.ndim = 6;
    g.np = cfg->np;
    g.nsp = cfg->nsp;
    g.nxgs = 2;
    g.nxge = 2 + cfg->nx - 1;
    g.nygs = 2;
    g.nyge = 2 + cfg->ny - 1;
    g.nys = g.nygs;
    g.nye = g.nyge;
    g.nx = cfg->nx;
    g.ny = cfg->ny;
    g.nrows = g.nsp * g.ny;
    g.nxw = g.nx + 4;
    g.nyw = g.ny + 4;
    g.nxa = g.nx;  // the whole box unless the shock's expansion is set
    WmConst &k = s->k;
    k.delx = cfg->delx;
    k.delt = cfg->delt;
    k.c = cfg->c;
    k.gfac = cfg->gfac;
    for (int i = 0; i < WM_MAX_SP; ++i) {
        k.q[i] = i < cfg->nsp ? cfg->q[i] : 0.0;
        k.r[i] = i < cfg->nsp ? cfg->r[i] : 1.0;
    }
    k.cg_err = cfg->cg_err;
    k.cg_itemax = cfg->cg_itemax;
    s->precision = cfg->precision;
    s->cap_req = cfg->capacity;
    // the main stream at the highest priority: the mixed step's rebin runs beside the field solve on
    // a second stream of the lowest, so the solve's blocks are scheduled first
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (cudaStreamCreateWithPriority(&s->st, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
        cudaMallocHost((void **)&s->scal_host, wm_field_scal_bytes()) != cudaSuccess ||
        cudaMallocHost((void **)&s->status_host, sizeof(unsigned)) != cudaSuccess) {
        s->release();
        delete s;
        return WM_ERR_CUDA;
    }
    *out = s;
    return WM_OK;
}

int wm_sim_destroy(wm_sim *s)
{
    if (!s) return WM_ERR_BAD_ARG;
    s->release();
    delete s;
    return WM_OK;
}

// Check the row counts of a state about to be loaded and size the device buffers for it.
static int sim_prepare(wm_sim *s, const int *np2_h)
{
    const WmGeom &g = s->g;
    long long ntot = 0;
    for (int r = 0; r < g.nrows; ++r) {
        if (np2_h[r] < 0 || np2_h[r] > g.np) return WM_ERR_BAD_ARG;
        ntot += np2_h[r];
    }
    if (ntot >= (1LL << 32)) return WM_ERR_UNSUPPORTED;
    long long cap = std::max<long long>(ntot, 1);
    if (s->cap_req > cap) cap = s->cap_req;
    if (!s->loaded || cap > s->cap) WM_TRY(s->alloc(cap));
    s->ntot = ntot;
    return WM_OK;
}

static int sim_finish_load(wm_sim *s)
{
    const WmGeom &g = s->g;
    if (!s->loaded) {
        const size_t nf = (size_t)g.nxw * g.nyw;
        WM_CUDA(cudaMemsetAsync(s->f_df.p, 0, sizeof(double) * 6 * nf, s->st));
        WM_CUDA(cudaMemsetAsync(s->f_uj.p, 0, sizeof(double) * 3 * nf, s->st));
    }
    s->loaded = true;
    WM_CUDA(cudaStreamSynchronize(s->st));
    return WM_OK;
}

static int sim_load_common(wm_sim *s, const double *up, const double *uf, const int *np2_h, const int *cumcnt_h,
                           int host_pitch = -1)
{
    if (host_pitch < 0) host_pitch = s->g.np;
    const WmGeom &g = s->g;
    WM_TRY(sim_prepare(s, np2_h));
    if (cumcnt_h) {  // already sorted: upload straight into A
        WM_TRY(s->upload_particles(up, np2_h, s->A, host_pitch));
        s->pid_cur = 0;
        WM_CUDA(cudaMemcpyAsync(s->cumcnt.p, cumcnt_h, sizeof(int) * (size_t)(g.nx + 1) * g.nrows, cudaMemcpyHostToDevice, s->st));
    } else {
        WM_TRY(s->upload_particles(up, np2_h, s->B, host_pitch));
        WM_TRY(s->sort_B_into_A());
    }
    WM_TRY(s->upload_fields(uf));
    s->pmark("copy_in_fields");
    return sim_finish_load(s);
}

// A generated state: rows of n_row particles per species written into the stage by
// k_init_particles, unpacked and cell-sorted on the device; fields by k_init_fields (or zero).
static int sim_init_generated(wm_sim *s, WmInitArgs &a, bool fields)
{
    const WmGeom &g = s->g;
    if (a.n_row < 1 || a.n_row > g.np) return WM_ERR_BAD_ARG;
    std::vector<int> np2_h(g.nrows, a.n_row);
    WM_TRY(sim_prepare(s, np2_h.data()));
    a.delx = s->k.delx;
    a.c = s->k.c;
    WM_TRY(s->stage.ensure(sizeof(double) * 6 * (size_t)a.n_row * g.nrows));
    WM_TRY(wm_launch_init_particles(g, a, s->stage.as<double>(), s->st));
    WM_TRY(s->upload_particles(nullptr, np2_h.data(), s->B, a.n_row));
    WM_TRY(s->sort_B_into_A());
    if (fields) {
        WM_TRY(wm_launch_init_fields(g, a, s->uf(), s->st));
    } else {
        WM_CUDA(cudaMemsetAsync(s->f_uf.p, 0, sizeof(double) * 6 * (size_t)g.nxw * g.nyw, s->st));
    }
    s->it = 0;
    if (s->loaded) {  // a fresh state: the CG starts from zero as after a first load
        const size_t nf = (size_t)g.nxw * g.nyw;
        WM_CUDA(cudaMemsetAsync(s->f_df.p, 0, sizeof(double) * 6 * nf, s->st));
        WM_CUDA(cudaMemsetAsync(s->f_uj.p, 0, sizeof(double) * 3 * nf, s->st));
    }
    return sim_finish_load(s);
}

int wm_sim_init_weibel(wm_sim *s, int ppc, double v_drift, double vth_e, double vth_i, uint64_t seed)
{
    if (!s || ppc < 1 || !(fabs(v_drift) < 1.0) || s->g.nsp != 2) return WM_ERR_BAD_ARG;
    WmInitArgs a{};
    a.tag = WM_RNG_WEIBEL;
    a.n_row = (int)std::min<long long>((long long)ppc * s->g.nx, 1LL << 30);
    a.seed = seed;
    a.vth_e = vth_e;
    a.vth_i = vth_i;
    a.ud = v_drift / sqrt(1.0 - v_drift * v_drift);
    return sim_init_generated(s, a, false);
}

int wm_sim_init_harris(wm_sim *s, int nbg, int ncs, double lcs, double b0, double e1, double vte, double vti, double rtemp,
                       uint64_t seed)
{
    if (!s || nbg < 0 || ncs < 0 || !(lcs > 0) || s->g.nsp != 2 || s->g.bc != WM_BC_RECONNECTION) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    const double delx = s->k.delx;
    WmInitArgs a{};
    a.tag = WM_RNG_HARRIS;
    a.n_row = (int)(nbg * (g.nx - 1) + ncs * 2 * lcs);  // proj/reconnection/app.f90:309
    a.seed = seed;
    a.vth_e = vte;
    a.vth_i = vti;
    a.ibg = nbg * (g.nxge - g.nxgs - 2);
    a.lcs = lcs;
    a.x0 = 0.5 * (g.nxge + g.nxgs) * delx;
    a.y0 = 0.5 * (g.nyge - g.nygs) * delx;
    a.tanh_edge = tanh(0.5 * (g.nxge - g.nxgs - 2) * delx / lcs);
    a.b0 = b0;
    a.e1 = e1;
    a.ncs = ncs;
    a.nbg = nbg;
    a.f1 = 1.0 / ((1.0 + rtemp) * s->k.q[0]);
    a.f2 = rtemp / ((1.0 + rtemp) * s->k.q[1]);
    return sim_init_generated(s, a, true);
}

int wm_sim_init_shock(wm_sim *s, int n0, double u0, double vth_e, double vth_i, double b0, double theta_bn, double phi_bn,
                      double l_damp_ini, double xrs, double xre, uint64_t seed)
{
    if (!s || n0 < 1 || s->g.nsp != 2 || s->g.bc != WM_BC_SHOCK) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    const double c = s->k.c;
    WmInitArgs a{};
    a.tag = WM_RNG_SHOCK;
    a.n_row = n0 * (g.nxa - 2);  // np2 = n0*(nxe-nxs-1), proj/shock/app.f90:335, nxs = nxgs, nxe = nxgs + nxa - 1
    a.seed = seed;
    a.vth_e = vth_e;
    a.vth_i = vth_i;
    a.v0 = u0 / sqrt(1 + (u0 * u0) / (c * c));
    a.l_damp_ini = l_damp_ini;
    a.nxgs_delx = g.nxgs * s->k.delx;
    a.xrs = xrs;
    a.xre = xre;
    a.bx = b0 * cos(theta_bn);
    a.by = b0 * sin(theta_bn) * cos(phi_bn);
    a.bz = b0 * sin(theta_bn) * sin(phi_bn);
    return sim_init_generated(s, a, true);
}

int wm_sim_set_injection(wm_sim *s, int on, int n0, double vth_e, double vth_i, double b0, double theta_bn, double phi_bn,
                         double l_damp_ini, uint64_t seed)
{
    if (!s) return WM_ERR_BAD_ARG;
    if (!on) {
        s->inject_on = false;
        return WM_OK;
    }
    const WmGeom &g = s->g;
    if (g.bc != WM_BC_SHOCK || g.nsp != 2 || n0 < 1) return WM_ERR_BAD_ARG;
    if (g.ny > WM_INJECT_MAX_ROWS) return WM_ERR_UNSUPPORTED;
    const double c = s->k.c, delt = s->k.delt, delx = s->k.delx, u0 = s->u0;
    WmInjectArgs a{};
    a.seed = seed;
    a.v0 = u0 / sqrt(1 + (u0 * u0) / (c * c));  // proj/shock/app.f90:318-319
    a.delt = delt;
    a.c = c;
    a.delx = delx;
    a.pflux = n0 * fabs(a.v0) * delt * delx * (g.nyge - g.nygs + 1);  // app.f90:725
    a.x0 = fabs(a.v0) * delt;
    a.xe = (g.nxgs + g.nxa - 1) * delx;
    a.vth_e = vth_e;
    a.vth_i = vth_i;
    a.l_damp_ini = l_damp_ini;
    a.nxgs_delx = g.nxgs * delx;
    a.cell = g.nxa - 2;  // nxe-1
    a.by0 = b0 * sin(theta_bn) * cos(phi_bn);
    a.bz0 = b0 * sin(theta_bn) * sin(phi_bn);
    WM_TRY(s->inj_rows.ensure(sizeof(int) * g.ny));
    WM_TRY(s->inj_ninc.ensure(sizeof(long long) * g.ny));
    WM_TRY(s->inj_nptot.ensure(sizeof(long long) * 2));
    WM_TRY(s->inj_tmp.ensure(sizeof(int) * g.nrows));
    s->inj = a;
    s->inj_n0 = n0;
    s->inject_on = true;
    return WM_OK;
}

int wm_sim_set_expansion(wm_sim *s, int n_x_ini, int intvl_expand)
{
    if (!s || s->g.bc != WM_BC_SHOCK || n_x_ini < 3 || n_x_ini > s->g.nx - 1 || intvl_expand < 0) return WM_ERR_BAD_ARG;
    s->g.nxa = n_x_ini + 1;  // nxe = nxgs + n_x_ini (proj/shock/app.f90:277)
    s->expand_every = intvl_expand;
    s->sync_inject_boundary();
    return WM_OK;
}

int wm_sim_get_nxe(wm_sim *s, int *nxe)
{
    if (!s || !nxe) return WM_ERR_BAD_ARG;
    *nxe = s->g.nxgs + s->g.nxa - 1;
    return WM_OK;
}

int wm_sim_set_step(wm_sim *s, int64_t it)
{
    if (!s || it < 0) return WM_ERR_BAD_ARG;
    s->it = it;
    return WM_OK;
}

int wm_sim_get_step(wm_sim *s, int64_t *it)
{
    if (!s || !it) return WM_ERR_BAD_ARG;
    *it = s->it;
    return WM_OK;
}

int wm_sim_load(wm_sim *s, const double *up, const double *uf, const int *np2_h)
{
    if (!s || !up || !uf || !np2_h) return WM_ERR_BAD_ARG;
    return sim_load_common(s, up, uf, np2_h, nullptr);
}

// Row counts of the current state (host copy) and their maximum.
static int sim_row_counts(wm_sim *s, std::vector<int> &cnt, int &maxc)
{
    const WmGeom &g = s->g;
    cnt.resize(g.nrows);
    WM_CUDA(cudaMemcpyAsync(cnt.data(), s->np2[s->cur].p, sizeof(int) * g.nrows, cudaMemcpyDeviceToHost, s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    maxc = std::max(1, *std::max_element(cnt.begin(), cnt.end()));
    return WM_OK;
}

// The current particles as reference-layout rows in s->stage: 6 doubles per slot, `pitch` slots
// per row, slots past a row's count zero.
static int sim_pack_rows(wm_sim *s, int pitch, int r0, int nr)
{
    const WmGeom &g = s->g;
    WM_TRY(s->materialize());
    if (s->mixed())
        return wm_launch_mixed_pack(g, s->mview(s->A, s->cur, s->pid_cur), s->np2[s->cur].as<int>(), s->cumcnt.as<int>(), pitch,
                                    s->stage.as<double>(), s->st, r0, nr);
    dim3 grid(std::min(wm_div_up(pitch, 256), 64u), nr);
    k_pack<<<grid, 256, 0, s->st>>>(g, s->view(s->A, s->cur), s->np2[s->cur].as<int>(), pitch, s->stage.as<double>(), r0);
    return wm_check_launch("k_pack");
}

static int sim_pack_stage(wm_sim *s, int pitch)
{
    WM_TRY(s->stage.ensure(sizeof(double) * 6 * (size_t)pitch * s->g.nrows));
    return sim_pack_rows(s, pitch, 0, s->g.nrows);
}

int wm_sim_store(wm_sim *s, double *up, double *uf, int *np2_h, int *cumcnt_h)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    const WmGeom &g = s->g;
    std::vector<int> cnt;
    int maxc;
    WM_TRY(sim_row_counts(s, cnt, maxc));
    if (up && maxc > g.np) return WM_ERR_OVERFLOW;  // a row does not fit the host array's np slots
    s->pmark("store_start");
    if (up) {
        const size_t rowb = sizeof(double) * 6 * maxc, hrowb = sizeof(double) * 6 * g.np;
        if (s->mixed() && rows_mapped(up, up, hrowb, up, hrowb, rowb)) {
            // host rows mapped into the device's address space: the pack writes them directly,
            // reading a permuted state through its permutations (the link is the bound; a staged
            // pack then a copy, or a gather into cell order first, costs those on top)
            s->pmark("copy_out_pack");
            if (s->permuted)
                WM_TRY(wm_launch_mixed_pack(g, s->mview(s->A, s->cur), s->np2[s->cur].as<int>(), s->cumcnt.as<int>(), maxc, up, s->st, 0,
                                            -1, g.np, s->mx_perm.as<unsigned>(), s->mx_idperm[s->idp].as<unsigned>()));
            else
                WM_TRY(wm_launch_mixed_pack(g, s->mview(s->A, s->cur, s->pid_cur), s->np2[s->cur].as<int>(), s->cumcnt.as<int>(), maxc, up,
                                            s->st, 0, -1, g.np));
        } else {
            WM_TRY(s->stage.ensure(rowb * g.nrows));
            WM_TRY(sim_pack_stage(s, maxc));
            s->pmark("copy_out_pack");
            WM_TRY(copy_rows(up, hrowb, s->stage.p, rowb, rowb, g.nrows, true, s->st));
        }
        s->pmark("copy_out_d2h");
    }
    if (uf) {
        const long long npts = (long long)g.nxw * g.nyw;
        WM_TRY(s->uf_aos.ensure(sizeof(double) * 6 * npts));
        WM_TRY(wm_launch_soa_to_aos(6, npts, s->f_uf.as<double>(), s->uf_aos.as<double>(), s->st));
        WM_CUDA(cudaMemcpyAsync(uf, s->uf_aos.p, sizeof(double) * 6 * npts, cudaMemcpyDeviceToHost, s->st));
    }
    if (cumcnt_h)
        WM_CUDA(cudaMemcpyAsync(cumcnt_h, s->cumcnt.p, sizeof(int) * (size_t)(g.nx + 1) * g.nrows, cudaMemcpyDeviceToHost, s->st));
    s->pmark("copy_out_fields");
    WM_CUDA(cudaStreamSynchronize(s->st));
    if (np2_h) std::memcpy(np2_h, cnt.data(), sizeof(int) * g.nrows);
    return WM_OK;
}

int wm_sim_step(wm_sim *s, int nsteps)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    s->nmarks = 0;
    s->nsmarks = 0;
    s->launches = 0;
    s->t_names.clear();
    s->t_ms.clear();
    for (int i = 0; i < nsteps; ++i) WM_TRY(s->step_once());
    if (s->timing && s->nsmarks > 1) {  // the rebin's kernels on the second stream (beside the field solve)
        WM_CUDA(cudaStreamSynchronize(s->st));
        for (size_t m = 1; m < s->nsmarks; ++m) {
            if (std::strcmp(s->smarks[m].name, "start") == 0) continue;
            float ms = 0.f;
            WM_CUDA(cudaEventElapsedTime(&ms, s->smarks[m - 1].ev, s->smarks[m].ev));
            size_t idx = 0;
            while (idx < s->t_names.size() && std::strcmp(s->t_names[idx], s->smarks[m].name) != 0) ++idx;
            if (idx == s->t_names.size()) {
                s->t_names.push_back(s->smarks[m].name);
                s->t_ms.push_back(0.0);
            }
            s->t_ms[idx] += ms;
        }
    }
    if (s->timing && s->nmarks > 1) {
        WM_CUDA(cudaStreamSynchronize(s->st));
        for (size_t m = 1; m < s->nmarks; ++m) {
            if (std::strcmp(s->marks[m].name, "start") == 0) continue;
            float ms = 0.f;
            WM_CUDA(cudaEventElapsedTime(&ms, s->marks[m - 1].ev, s->marks[m].ev));
            size_t idx = 0;
            while (idx < s->t_names.size() && std::strcmp(s->t_names[idx], s->marks[m].name) != 0) ++idx;
            if (idx == s->t_names.size()) {
                s->t_names.push_back(s->marks[m].name);
                s->t_ms.push_back(0.0);
            }
            s->t_ms[idx] += ms;
        }
    }
    return WM_OK;
}

int wm_sim_step_host(wm_sim *s, double *up, double *uf, int *np2_h, int *cumcnt_h, int nsteps)
{
    if (!s || !up || !uf || !np2_h || !cumcnt_h) return WM_ERR_BAD_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    s->nphases = 0;
    s->pmark("start");
    WM_TRY(sim_load_common(s, up, uf, np2_h, cumcnt_h));  // ends with a stream synchronisation
    const auto t1 = std::chrono::steady_clock::now();
    WM_TRY(wm_sim_step(s, nsteps));
    WM_CUDA(cudaStreamSynchronize(s->st));
    const auto t2 = std::chrono::steady_clock::now();
    WM_TRY(wm_sim_store(s, up, uf, np2_h, cumcnt_h));
    const auto t3 = std::chrono::steady_clock::now();
    if (s->timing) {  // wall-clock phases of this call, after the steps' own kernel times
        const auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
        s->t_names.push_back("host_copy_in");
        s->t_ms.push_back(ms(t0, t1));
        s->t_names.push_back("host_steps");
        s->t_ms.push_back(ms(t1, t2));
        s->t_names.push_back("host_copy_out");
        s->t_ms.push_back(ms(t2, t3));
        // GPU-side phases (events on the stream): each interval is named by the mark that ends it;
        // the one ending at store_start holds the steps and is left out
        for (size_t m = 1; m < s->nphases; ++m) {
            if (std::strcmp(s->phases[m].name, "store_start") == 0) continue;
            float e = 0.f;
            WM_CUDA(cudaEventElapsedTime(&e, s->phases[m - 1].ev, s->phases[m].ev));
            s->t_names.push_back(s->phases[m].name);
            s->t_ms.push_back(e);
        }
    }
    return WM_OK;
}

int wm_sim_energy(wm_sim *s, double *out)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    const WmGeom &g = s->g;
    const int nb = 304;
    double *part = s->energy_partial.as<double>();
    WM_TRY(s->materialize());
    if (s->mixed())
        WM_TRY(wm_launch_energy_particles(g, s->k, s->mview(s->A, s->cur), s->np2[s->cur].as<int>(), part, nb, s->st));
    else
        WM_TRY(wm_launch_energy_particles(g, s->k, s->view(s->A, s->cur), s->np2[s->cur].as<int>(), part, nb, s->st));
    WM_TRY(wm_launch_energy_fields(g, s->uf(), part + (size_t)nb * g.nsp, nb, s->st));
    WM_TRY(wm_launch_sum_partials(part, nb, g.nsp + 2, s->energy_out.as<double>(), s->st));
    std::vector<double> tmp(g.nsp + 2);
    WM_CUDA(cudaMemcpyAsync(tmp.data(), s->energy_out.p, sizeof(double) * (g.nsp + 2), cudaMemcpyDeviceToHost, s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    const double pi = 3.14159265358979311599796346854418516;
    for (int i = 0; i < g.nsp; ++i) out[i] = tmp[i];
    out[g.nsp] = tmp[g.nsp + 1] / (8 * pi);
    out[g.nsp + 1] = tmp[g.nsp] / (8 * pi);
    return WM_OK;
}

// mom_calc__accl + mom_calc__nvt + boundary__mom of the current state into s->mom_dev
// (reference layout mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp)).
static int sim_moments_device(wm_sim *s)
{
    const WmGeom &g = s->g;
    const size_t nm = (size_t)7 * (g.nx + 2) * (g.ny + 2) * g.nsp;
    WM_TRY(s->mom_dev.ensure(sizeof(double) * nm));
    WM_TRY(s->materialize());
    if (s->mixed()) {
        // moment steps are rare: expand the mixed state to FP64 rows (pitch = largest row) and run
        // the FP64 half-step push and moment deposit on that copy
        std::vector<int> cnt(g.nrows);
        WM_CUDA(cudaMemcpyAsync(cnt.data(), s->np2[s->cur].p, sizeof(int) * g.nrows, cudaMemcpyDeviceToHost, s->st));
        WM_CUDA(cudaStreamSynchronize(s->st));
        const int pitch = std::max(1, *std::max_element(cnt.begin(), cnt.end()));
        const size_t nstage = (size_t)6 * pitch * g.nrows;
        WM_TRY(s->stage.ensure(sizeof(double) * nstage));
        WM_TRY(s->stage2.ensure(sizeof(double) * nstage));
        WM_TRY(wm_launch_mixed_pack(g, s->mview(s->A, s->cur, s->pid_cur), s->np2[s->cur].as<int>(), s->cumcnt.as<int>(), pitch,
                                    s->stage.as<double>(), s->st));
        AoSView va{s->stage.as<double>(), pitch}, vb{s->stage2.as<double>(), pitch};
        WM_TRY(wm_launch_push(g, s->k, va, vb, s->uf(), s->cumcnt.as<int>(), 1, 0, s->st));
        WM_TRY(wm_launch_mom_nvt(g, s->k, vb, s->np2[s->cur].as<int>(), s->mom_dev.as<double>(), pitch, s->st));
    } else {
        SoAView va = s->view(s->A, s->cur), vb = s->view(s->B, s->cur);
        WM_TRY(wm_launch_push(g, s->k, va, vb, s->uf(), s->cumcnt.as<int>(), 1, 0, s->st));
        WM_TRY(wm_launch_mom_nvt(g, s->k, vb, s->np2[s->cur].as<int>(), s->mom_dev.as<double>(), s->max_row, s->st));
    }
    return wm_launch_mom_bc(g, s->mom_dev.as<double>(), s->st);
}

int wm_sim_moments(wm_sim *s, double *mom)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    if (!mom) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    WM_TRY(sim_moments_device(s));
    WM_CUDA(cudaMemcpyAsync(mom, s->mom_dev.p, sizeof(double) * 7 * (g.nx + 2) * (g.ny + 2) * g.nsp, cudaMemcpyDeviceToHost, s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    return WM_OK;
}

// ------------------------------------------------- snapshot and output files from the GPU
// The module parameters paraio__init would hold for this simulation (one rank, ndim = 6).
static wmpio::Params sim_pio_params(const wm_sim *s)
{
    const WmGeom &g = s->g;
    wmpio::Params P;
    P.ndim = 6;
    P.np = g.np;
    P.nsp = g.nsp;
    P.nxgs = g.nxgs;
    P.nxge = g.nxge;
    P.nygs = g.nygs;
    P.nyge = g.nyge;
    P.nys = g.nys;
    P.nye = g.nye;
    P.nproc = 1;
    P.delx = s->k.delx;
    P.delt = s->k.delt;
    P.c = s->k.c;
    for (int i = 0; i < g.nsp; ++i) {
        P.q[i] = s->k.q[i];
        P.r[i] = s->k.r[i];
    }
    return P;
}

int wm_sim_write_snapshot(wm_sim *s, const char *dir, const char *filename, int it)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    if (!dir || !filename) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    std::vector<int> cnt;
    int maxc;
    WM_TRY(sim_row_counts(s, cnt, maxc));
    if (maxc > g.np) return WM_ERR_OVERFLOW;
    WM_TRY(sim_pack_stage(s, maxc));
    const wmpio::Params P = sim_pio_params(s);
    wmpio::Writer w;
    WM_TRY(w.open(dir, filename));
    WM_TRY(wmpio::write_head(w, P, it, {{"nxs", g.nxgs}, {"nxe", g.nxgs + g.nxa - 1}}));
    WM_TRY(w.dataset("up", "f8", {6, g.np, g.ny, g.nsp, 1}, "particles"));
    WM_TRY(wmpio::write_rows_from_device(w, s->stage.p, sizeof(double) * 6 * maxc, sizeof(double) * 6 * g.np, g.nrows, s->st));
    WM_TRY(w.dataset("np2", "i4", {g.ny, g.nsp, 1}, "number of active particles"));
    WM_TRY(w.write(cnt.data(), sizeof(int) * g.nrows));
    const long long npts = (long long)g.nxw * g.nyw;
    WM_TRY(s->uf_aos.ensure(sizeof(double) * 6 * npts));
    WM_TRY(wm_launch_soa_to_aos(6, npts, s->f_uf.as<double>(), s->uf_aos.as<double>(), s->st));
    WM_TRY(w.dataset("uf", "f8", {6, g.nxw, g.nyw, 1}, "electromagnetic fields including ghost cells"));
    WM_TRY(wmpio::write_from_device(w, s->uf_aos.p, sizeof(double) * 6 * npts, s->st));
    return w.close();
}

int wm_sim_read_snapshot(wm_sim *s, const char *dir, const char *filename, int *it)
{
    if (!s || !dir || !filename || !it) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    wmpio::Reader rd;
    WM_TRY(rd.open(dir, filename));
    const wmpio::Params P = sim_pio_params(s);
    const char *names[8] = {"ndim", "np", "nxgs", "nxge", "nygs", "nyge", "nsp", "nproc"};
    const int want[8] = {6, P.np, P.nxgs, P.nxge, P.nygs, P.nyge, P.nsp, 1};
    for (int i = 0; i < 8; ++i) {
        int v;
        WM_TRY(rd.read_i4(names[i], v));
        if (v != want[i]) return WM_ERR_IO;  // paraio.f90:329-340
    }
    int nxs, nxe;
    WM_TRY(rd.read_i4("it", *it));
    WM_TRY(rd.read_i4("nxs", nxs));
    WM_TRY(rd.read_i4("nxe", nxe));
    if (nxs != g.nxgs || nxe > g.nxge || (nxe != g.nxge && g.bc != WM_BC_SHOCK) || nxe < g.nxgs + 3) return WM_ERR_UNSUPPORTED;
    s->g.nxa = nxe - g.nxgs + 1;  // the shock box's extent at the snapshot
    s->sync_inject_boundary();
    wmpio::Entry e_up, e_np2, e_uf;
    WM_TRY(rd.find("dataset", "up", e_up));
    WM_TRY(rd.find("dataset", "np2", e_np2));
    WM_TRY(rd.find("dataset", "uf", e_uf));
    if (e_up.shape != std::vector<long long>{6, g.np, g.ny, g.nsp, 1} || e_np2.shape != std::vector<long long>{g.ny, g.nsp, 1} ||
        e_uf.shape != std::vector<long long>{6, g.nxw, g.nyw, 1})
        return WM_ERR_IO;
    std::vector<int> np2_h(g.nrows);
    WM_TRY(rd.read(e_np2, np2_h.data(), sizeof(int) * g.nrows));
    int maxc = 1;
    for (int r = 0; r < g.nrows; ++r) {
        if (np2_h[r] < 0 || np2_h[r] > g.np) return WM_ERR_IO;
        maxc = std::max(maxc, np2_h[r]);
    }
    std::vector<double> uf_h((size_t)6 * g.nxw * g.nyw);
    WM_TRY(rd.read(e_uf, uf_h.data(), sizeof(double) * uf_h.size()));
    // only the active part of each row (the first maxc slots) is read, into page-locked memory
    const size_t row_bytes = sizeof(double) * 6 * (size_t)maxc;
    double *up_h = nullptr;
    WM_CUDA(cudaHostAlloc((void **)&up_h, row_bytes * g.nrows, cudaHostAllocPortable));
    int st = WM_OK;
    for (int r = 0; r < g.nrows && st == WM_OK; ++r) {
        wmpio::Entry row = e_up;
        row.offset = e_up.offset + (long long)r * sizeof(double) * 6 * g.np;
        st = rd.read(row, (char *)up_h + r * row_bytes, row_bytes);
    }
    if (st == WM_OK) st = sim_load_common(s, up_h, uf_h.data(), np2_h.data(), nullptr, maxc);
    cudaFreeHost(up_h);
    if (st == WM_OK) s->it = *it;
    return st;
}

int wm_sim_write_moments(wm_sim *s, const char *dir, int it)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    if (!dir) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    WM_TRY(sim_moments_device(s));
    const long long ncs = (long long)g.nx * g.ny * g.nsp, nc = (long long)g.nx * g.ny;
    WM_TRY(s->out_dev.ensure(sizeof(double) * (7 * ncs + 6 * nc)));
    WM_TRY(wm_launch_mom_file(g, s->mom_dev.as<double>(), s->uf(), s->out_dev.as<double>(), s->st));
    const wmpio::Params P = sim_pio_params(s);
    char name[32];
    snprintf(name, sizeof name, "%07d_mom", it);
    wmpio::Writer w;
    WM_TRY(w.open(dir, name));
    WM_TRY(wmpio::write_head(w, P, it, {}));
    const double *o = s->out_dev.as<double>();
    WM_TRY(w.dataset("den", "f8", {g.nx, g.ny, g.nsp}, "density"));
    WM_TRY(wmpio::write_from_device(w, o, sizeof(double) * ncs, s->st));
    WM_TRY(w.dataset("vel", "f8", {3, g.nx, g.ny, g.nsp}, "velocity"));
    WM_TRY(wmpio::write_from_device(w, o + ncs, sizeof(double) * 3 * ncs, s->st));
    WM_TRY(w.dataset("temp", "f8", {3, g.nx, g.ny, g.nsp}, "temperature"));
    WM_TRY(wmpio::write_from_device(w, o + 4 * ncs, sizeof(double) * 3 * ncs, s->st));
    WM_TRY(w.dataset("uf", "f8", {6, g.nx, g.ny}, "electromagnetic field"));
    WM_TRY(wmpio::write_from_device(w, o + 7 * ncs, sizeof(double) * 6 * nc, s->st));
    return w.close();
}

int wm_sim_write_particles(wm_sim *s, const char *dir, int it, int tracers_only)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    if (!dir) return WM_ERR_BAD_ARG;
    const WmGeom &g = s->g;
    const int mode = tracers_only ? 1 : 0;
    std::vector<int> cnt;
    int maxc;
    WM_TRY(sim_row_counts(s, cnt, maxc));
    WM_TRY(sim_pack_stage(s, maxc));
    // rows in file order (species, then j), compacted on the GPU with their slot order kept
    WM_TRY(s->out_cnt.ensure(sizeof(long long) * 2 * g.nrows));
    long long *dcnt = s->out_cnt.as<long long>(), *doff = dcnt + g.nrows;
    WM_TRY(wm_launch_row_count(g.nrows, s->stage.as<double>(), maxc, s->np2[s->cur].as<int>(), mode, dcnt, s->st));
    std::vector<long long> rc(g.nrows), off(g.nrows);
    WM_CUDA(cudaMemcpyAsync(rc.data(), dcnt, sizeof(long long) * g.nrows, cudaMemcpyDeviceToHost, s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    long long total = 0;
    std::vector<long long> nsp_count(g.nsp, 0);
    for (int r = 0; r < g.nrows; ++r) {
        off[r] = total;
        total += rc[r];
        nsp_count[r / g.ny] += rc[r];
    }
    const long long nc = (long long)g.nx * g.ny;
    WM_TRY(s->out_dev.ensure(sizeof(double) * (6 * std::max(total, 1LL) + 6 * nc)));
    double *parts = s->out_dev.as<double>(), *ufi = parts + 6 * std::max(total, 1LL);
    WM_CUDA(cudaMemcpyAsync(doff, off.data(), sizeof(long long) * g.nrows, cudaMemcpyHostToDevice, s->st));
    WM_TRY(wm_launch_row_compact(g.nrows, s->stage.as<double>(), maxc, s->np2[s->cur].as<int>(), mode, doff, parts, s->st));
    WM_TRY(wm_launch_uf_interior(g, s->uf(), ufi, s->st));
    const wmpio::Params P = sim_pio_params(s);
    char name[32];
    snprintf(name, sizeof name, "%07d%s", it, mode ? "_orb" : "_ptcl");
    wmpio::Writer w;
    WM_TRY(w.open(dir, name));
    WM_TRY(wmpio::write_head(w, P, it, {}));
    WM_TRY(w.dataset("uf", "f8", {6, g.nx, g.ny}, "electromagnetic field"));
    WM_TRY(wmpio::write_from_device(w, ufi, sizeof(double) * 6 * nc, s->st));
    long long done = 0;
    for (int isp = 0; isp < g.nsp; ++isp) {
        char ds[16], desc[64];
        snprintf(ds, sizeof ds, "up%02d", isp + 1);
        snprintf(desc, sizeof desc, "particle species #%02d", isp + 1);
        WM_TRY(w.dataset(ds, "f8", {6, nsp_count[isp]}, desc));
        WM_TRY(wmpio::write_from_device(w, parts + 6 * done, sizeof(double) * 6 * nsp_count[isp], s->st));
        done += nsp_count[isp];
    }
    return w.close();
}

int wm_sim_cg_iters(wm_sim *s, int *iters3)
{
    if (!s) return WM_ERR_BAD_ARG;
    for (int l = 0; l < 3; ++l) iters3[l] = s->iters[l];
    return WM_OK;
}

int wm_sim_kernel_times(wm_sim *s, const char **names, double *ms, int *n)
{
    if (!s || !n) return WM_ERR_BAD_ARG;
    const int cnt = (int)s->t_names.size();
    for (int i = 0; i < std::min(cnt, *n); ++i) {
        if (names) names[i] = s->t_names[i];
        if (ms) ms[i] = s->t_ms[i];
    }
    *n = cnt;
    return WM_OK;
}

int wm_sim_set_timing(wm_sim *s, int on)
{
    if (!s) return WM_ERR_BAD_ARG;
    s->timing = on != 0;
    return WM_OK;
}

int wm_sim_launches(wm_sim *s, int64_t *count)
{
    if (!s || !count) return WM_ERR_BAD_ARG;
    *count = s->launches;
    return WM_OK;
}

int wm_sim_info(wm_sim *s, int64_t *nparticles, int64_t *device_bytes)
{
    if (!s) return WM_ERR_BAD_ARG;
    if (nparticles && s->loaded && s->inject_on) {  // the count grows every step: read the rows
        std::vector<int> cnt;
        int maxc;
        WM_TRY(sim_row_counts(s, cnt, maxc));
        long long n = 0;
        for (int c : cnt) n += c;
        s->ntot = n;
    }
    if (nparticles) *nparticles = s->ntot;
    if (device_bytes) *device_bytes = (int64_t)s->device_bytes();
    return WM_OK;
}

int wm_sim_set_rebin(wm_sim *s, int mode)
{
    if (!s || (mode != WM_REBIN_PERMUTE && mode != WM_REBIN_MOVE)) return WM_ERR_BAD_ARG;
    if (mode == WM_REBIN_MOVE) WM_TRY(s->materialize());
    s->rebin_move = mode == WM_REBIN_MOVE;
    return WM_OK;
}

int wm_sim_sync(wm_sim *s)
{
    if (!s) return WM_ERR_BAD_ARG;
    WM_CUDA(cudaStreamSynchronize(s->st));
    return WM_OK;
}

int wm_sim_get_work(wm_sim *s, double *df, double *uj)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    const WmGeom &g = s->g;
    const long long npts = (long long)g.nxw * g.nyw;
    WM_TRY(s->uf_aos.ensure(sizeof(double) * 6 * npts));
    if (df) {
        WM_TRY(wm_launch_soa_to_aos(6, npts, s->f_df.as<double>(), s->uf_aos.as<double>(), s->st));
        WM_CUDA(cudaMemcpyAsync(df, s->uf_aos.p, sizeof(double) * 6 * npts, cudaMemcpyDeviceToHost, s->st));
        WM_CUDA(cudaStreamSynchronize(s->st));
    }
    if (uj) {
        WM_TRY(wm_launch_soa_to_aos(3, npts, s->f_uj.as<double>(), s->uf_aos.as<double>(), s->st));
        WM_CUDA(cudaMemcpyAsync(uj, s->uf_aos.p, sizeof(double) * 3 * npts, cudaMemcpyDeviceToHost, s->st));
        WM_CUDA(cudaStreamSynchronize(s->st));
    }
    return WM_OK;
}

int wm_sim_set_work(wm_sim *s, const double *df)
{
    if (!s || !s->loaded) return WM_ERR_NOT_INIT;
    const WmGeom &g = s->g;
    const long long npts = (long long)g.nxw * g.nyw;
    WM_TRY(s->uf_aos.ensure(sizeof(double) * 6 * npts));
    WM_CUDA(cudaMemcpyAsync(s->uf_aos.p, df, sizeof(double) * 6 * npts, cudaMemcpyHostToDevice, s->st));
    WM_TRY(wm_launch_aos_to_soa(6, npts, s->uf_aos.as<double>(), s->f_df.as<double>(), s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    return WM_OK;
}

int wm_sim_set_guess(wm_sim *s, const float *params, long long nparams)
{
    if (!s) return WM_ERR_BAD_ARG;
    if (!params) {
        s->guess_on = false;
        return WM_OK;
    }
    const WmGeom &g = s->g;
    if (nparams != (long long)wm_cnn_param_count() || g.nx % 16 != 0 || g.ny % 8 != 0) return WM_ERR_BAD_ARG;
    const size_t ncell = (size_t)g.nx * g.ny;
    WM_TRY(s->cnn_params.ensure(sizeof(float) * nparams));
    for (int l = 0; l < WM_CNN_LAYERS; ++l) {
        WM_TRY(s->cnn_wf[l].ensure(2 * 9 * (size_t)wm_cnn_cin[l] * wm_cnn_cout[l]));
        s->net.wf[l] = s->cnn_wf[l].p;
    }
    WM_TRY(s->cnn_x.ensure(2 * 16 * ncell));
    WM_TRY(s->cnn_a0.ensure(2 * 48 * ncell));
    WM_TRY(s->cnn_a1.ensure(2 * 48 * ncell));
    WM_TRY(s->cnn_pred.ensure(sizeof(float) * 8 * ncell));
    WM_TRY(s->cnn_partial.ensure(sizeof(double) * 3 * WM_CNN_RED_BLOCKS));
    WM_TRY(s->cnn_scale.ensure(sizeof(double) * 6));
    WM_TRY(s->guess_cand.ensure(sizeof(double) * 3 * ncell));
    WM_TRY(s->guess_stats.ensure(sizeof(double) * 12));
    WM_CUDA(cudaMemsetAsync(s->guess_stats.p, 0, sizeof(double) * 12, s->st));
    WM_CUDA(cudaMemcpyAsync(s->cnn_params.p, params, sizeof(float) * nparams, cudaMemcpyHostToDevice, s->st));
    s->net.params = s->cnn_params.as<float>();
    WM_TRY(wm_cnn_net_prepare(s->net, s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    s->gdesc = WmGuess{&wm_sim::guess_run, s, s->guess_cand.as<double>(), s->guess_stats.as<double>()};
    s->guess_on = true;
    return WM_OK;
}

int wm_sim_guess_stats(wm_sim *s, double *stats)
{
    if (!s || !stats) return WM_ERR_BAD_ARG;
    if (!s->guess_on) return WM_ERR_NOT_INIT;
    WM_CUDA(cudaMemcpyAsync(stats, s->guess_stats.p, sizeof(double) * 12, cudaMemcpyDeviceToHost, s->st));
    WM_CUDA(cudaStreamSynchronize(s->st));
    return WM_OK;
}

int wm_sim_step_timed(wm_sim *s, int nsteps, double *ms)
{
    if (!s || !s->loaded || !ms) return WM_ERR_BAD_ARG;
    cudaEvent_t e0, e1;
    WM_CUDA(cudaEventCreate(&e0));
    WM_CUDA(cudaEventCreate(&e1));
    WM_CUDA(cudaEventRecord(e0, s->st));
    const int st = wm_sim_step(s, nsteps);
    WM_CUDA(cudaEventRecord(e1, s->st));
    WM_CUDA(cudaEventSynchronize(e1));
    float f = 0.f;
    WM_CUDA(cudaEventElapsedTime(&f, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = f;
    return st;
}

int wm_set_device(int device)
{
    WM_CUDA(cudaSetDevice(device));
    return WM_OK;
}

int wm_host_register(void *ptr, size_t bytes)
{
    WM_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return WM_OK;
}

int wm_host_unregister(void *ptr)
{
    WM_CUDA(cudaHostUnregister(ptr));
    return WM_OK;
}

int wm_host_alloc(void **ptr, size_t bytes)
{
    if (!ptr) return WM_ERR_BAD_ARG;
    *ptr = nullptr;
    WM_CUDA(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocPortable | cudaHostAllocMapped));
    return WM_OK;
}

int wm_host_free(void *ptr)
{
    if (ptr) WM_CUDA(cudaFreeHost(ptr));
    return WM_OK;
}

}  // extern "C"
