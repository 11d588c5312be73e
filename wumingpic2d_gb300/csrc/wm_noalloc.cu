// wm_noalloc.cu -- the current deposit for callers that cannot allocate GPU memory.
//
// Some callers of this library cannot call cudaMalloc: a host application that hands the
// library GPU memory from its own pool and forbids any allocation after start-up (so that memory
// use is fixed and no implicit device synchronisation happens mid-run), or code that runs where an
// allocation is not allowed at all.  wm_deposit_current_noalloc serves them: the caller passes its
// own device buffers for inputs and output, and the per-cell partial currents the deposit needs as
// scratch come from a fixed array in this library's static device memory instead of cudaMalloc.
//
// Limits and rules:
//   * at most WM_NOALLOC_MAX_CELLS interior cells (nx*ny); larger grids are rejected with
//     WM_ERR_BAD_ARG before anything is launched;
//   * the scratch array (75 doubles per cell, 39.3 MB) and a status word are part of every
//     GPU's copy of the library and stay allocated until the process exits;
//   * every call uses the same scratch: calls that overlap on the GPU (different streams, or
//     different host threads on one device) race and give wrong currents; serialise them;
//   * the first call on each device looks up the scratch's device address with
//     cudaGetSymbolAddress (once per device, with that device current); under CUDA's default
//     lazy module loading that first call is also when the array is placed in device memory, so
//     make it at start-up, before any stream capture begins, and later calls allocate nothing;
//   * every call is synchronous: it reads the status word back and waits for the stream.
// The kernels are the ones of the allocating path (k_deposit_cells, k_deposit_fold and the
// current fold of boundary_periodic__curre); only the source of their scratch differs.
#include <mutex>

#include "wm_launch.cuh"

#define WM_NOALLOC_MAX_CELLS 65536

namespace {

// Per-cell 5x5x3 partial currents: the kernel writes all 75 values of every cell it covers, so
// nothing left from an earlier call is read.  The status word is cleared on every call.
static __device__ __align__(256) double g_noalloc_pj[75 * WM_NOALLOC_MAX_CELLS];
static __device__ __align__(256) unsigned g_noalloc_status;

constexpr int NOALLOC_MAX_DEVICES = 64;
double *g_pj_addr[NOALLOC_MAX_DEVICES];
unsigned *g_status_addr[NOALLOC_MAX_DEVICES];
bool g_ready[NOALLOC_MAX_DEVICES];
std::mutex g_setup_mutex;

// Host code cannot use the symbols above as device addresses: look the addresses up once per
// device, with that device current.
int noalloc_setup(int dev)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_ready[dev]) return WM_OK;
    void *pj = nullptr, *st = nullptr;
    WM_CUDA(cudaGetSymbolAddress(&pj, g_noalloc_pj));
    WM_CUDA(cudaGetSymbolAddress(&st, g_noalloc_status));
    g_pj_addr[dev] = static_cast<double *>(pj);
    g_status_addr[dev] = static_cast<unsigned *>(st);
    g_ready[dev] = true;
    return WM_OK;
}

}  // namespace

extern "C" int wm_deposit_current_noalloc(const double *up, const double *gp, const int *cumcnt, double *uj, int ndim, int np,
                                          int nsp, int nxgs, int nxge, int nygs, int nyge, double delx, double delt,
                                          double c, const double *q, void *stream)
{
    if (!up || !gp || !cumcnt || !uj || !q) return WM_ERR_BAD_ARG;
    if (ndim != 6 || nsp < 1 || nsp > WM_MAX_SP || np < 1 || !(c > 0) || !(delt > 0) || !(delx > 0)) return WM_ERR_BAD_ARG;
    const int nx = nxge - nxgs + 1, ny = nyge - nygs + 1;
    if (nx < 4 || ny < 4) return WM_ERR_BAD_ARG;
    if ((long long)nx * ny > WM_NOALLOC_MAX_CELLS) {
        fprintf(stderr, "wm_deposit_current_noalloc: %d x %d cells exceed the limit of %d cells\n", nx, ny,
                WM_NOALLOC_MAX_CELLS);
        return WM_ERR_BAD_ARG;
    }
    int dev = 0;
    WM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return WM_ERR_UNSUPPORTED;
    WM_TRY(noalloc_setup(dev));

    WmGeom g{};
    g.bc = WM_BC_PERIODIC;  // field__fdtd_i's current fold of the periodic module
    g.ndim = ndim;
    g.np = np;
    g.nsp = nsp;
    g.nxgs = nxgs;
    g.nxge = nxge;
    g.nygs = nygs;
    g.nyge = nyge;
    g.nys = nygs;
    g.nye = nyge;
    g.nx = nx;
    g.ny = ny;
    g.nrows = nsp * ny;
    g.nxw = nx + 4;
    g.nyw = ny + 4;
    g.nxa = nx;
    WmConst k{};
    k.delx = delx;
    k.delt = delt;
    k.c = c;
    for (int s = 0; s < WM_MAX_SP; ++s) {
        k.q[s] = s < nsp ? q[s] : 0.0;
        k.r[s] = 1.0;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned *status = g_status_addr[dev];
    WM_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
    AoSView vu{const_cast<double *>(up), np}, vg{const_cast<double *>(gp), np};
    FView<3, true> vj{uj, g.nxw, g.nyw};
    WM_TRY(wm_launch_deposit_cells(g, k, vu, vg, cumcnt, g_pj_addr[dev], status, st));
    WM_TRY(wm_launch_deposit_fold(g, vj, g_pj_addr[dev], st));
    WM_TRY(wm_launch_curre_bc(g, vj, st));
    unsigned h = 0;
    WM_CUDA(cudaMemcpyAsync(&h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    WM_CUDA(cudaStreamSynchronize(st));
    return h ? WM_ERR_CELL : WM_OK;
}
