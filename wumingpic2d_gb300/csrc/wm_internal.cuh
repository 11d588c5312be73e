// wm_internal.cuh -- shared definitions of the sm_103a kernels and the host layer.
//
// Index conventions (0-based on the device):
//   particle rows      row = isp*ny + (j - nys),  isp 0-based, j the Fortran row index
//   slots              s0 = ii - 1 within a row
//   ghosted field      ix = i - (nxgs-2) in [0, nx+4), iy = j - (nys-2) in [0, ny+4)
//   interior cell      (ci, cj) = (i - nxgs, j - nys), cell id = cj*nx + ci
//   global cell key    row*nx + ci   (species, row and cell in one int)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/wumingpic2d.h"

#define WM_MAX_SP 4

struct WmGeom {
    int ndim, np, nsp;
    int nxgs, nxge, nygs, nyge, nys, nye;
    int nx, ny, nrows;  // nrows = nsp * ny
    int nxw, nyw;       // ghosted extents nx+4, ny+4
    int bc;             // WM_BC_*: boundary module of the application (x direction; y is periodic in all three)
    int nxa;            // active cells in x, nxe - nxgs + 1: the particles' range, the field solve's extent and the
                        // place of the x boundaries; nx but while the shock application's box expands
};

struct WmConst {
    double delx, delt, c, gfac;
    double q[WM_MAX_SP], r[WM_MAX_SP];
    double cg_err;
    int cg_itemax;
    double u0;  // shock: upstream four-velocity of the injection boundary
};

// ------------------------------------------------------------------ particles
// Compact structure of arrays, rows stored back to back; rowbase[row] is the first index.
struct SoAView {
    double *x, *y, *ux, *uy, *uz;
    long long *pid;
    const long long *rowbase;
    __device__ __forceinline__ long long idx(int row, int s0) const { return rowbase[row] + s0; }
    __device__ __forceinline__ double &X(long long p) const { return x[p]; }
    __device__ __forceinline__ double &Y(long long p) const { return y[p]; }
    __device__ __forceinline__ double &UX(long long p) const { return ux[p]; }
    __device__ __forceinline__ double &UY(long long p) const { return uy[p]; }
    __device__ __forceinline__ double &UZ(long long p) const { return uz[p]; }
    __device__ __forceinline__ long long getpid(long long p) const { return pid[p]; }
    __device__ __forceinline__ void setpid(long long p, long long v) const { pid[p] = v; }
};

// The reference layout up(6, np, nys:nye, nsp): 6 doubles per slot, np slots per row.
struct AoSView {
    double *a;
    int np;
    __device__ __forceinline__ long long idx(int row, int s0) const { return (long long)row * np + s0; }
    __device__ __forceinline__ double &X(long long p) const { return a[6 * p + 0]; }
    __device__ __forceinline__ double &Y(long long p) const { return a[6 * p + 1]; }
    __device__ __forceinline__ double &UX(long long p) const { return a[6 * p + 2]; }
    __device__ __forceinline__ double &UY(long long p) const { return a[6 * p + 3]; }
    __device__ __forceinline__ double &UZ(long long p) const { return a[6 * p + 4]; }
    __device__ __forceinline__ long long getpid(long long p) const { return __double_as_longlong(a[6 * p + 5]); }
    __device__ __forceinline__ void setpid(long long p, long long v) const { a[6 * p + 5] = __longlong_as_double(v); }
};

// Mixed-precision particles: FP32 offsets (dx, dy) in [0, 1) inside the particle's cell, FP32
// momenta, i64 pid.  The cell itself is not stored: rows are cell-sorted and cumcnt gives it.
// (dx, dy, ux, uy) share one 16-byte record, so a particle moves with one vector access and one
// 4-byte access to the uz plane; the ids are a separate plane.
struct MixedView {
    float4 *xyuv;  // (dx, dy, ux, uy) per slot
    float *uz;
    long long *pid;
    const long long *rowbase;
    __device__ __forceinline__ long long idx(int row, int s0) const { return rowbase[row] + s0; }
    __device__ __forceinline__ float &X(long long p) const { return xyuv[p].x; }
    __device__ __forceinline__ float &Y(long long p) const { return xyuv[p].y; }
    __device__ __forceinline__ float &UX(long long p) const { return xyuv[p].z; }
    __device__ __forceinline__ float &UY(long long p) const { return xyuv[p].w; }
    __device__ __forceinline__ float &UZ(long long p) const { return uz[p]; }
    __device__ __forceinline__ float4 &XYUV(long long p) const { return xyuv[p]; }
    __device__ __forceinline__ long long getpid(long long p) const { return pid[p]; }
    __device__ __forceinline__ void setpid(long long p, long long v) const { pid[p] = v; }
};

template <class V>
__device__ __forceinline__ void copy_particle(const V &dst, long long pd, const V &src, long long ps)
{
    dst.X(pd) = src.X(ps);
    dst.Y(pd) = src.Y(ps);
    dst.UX(pd) = src.UX(ps);
    dst.UY(pd) = src.UY(ps);
    dst.UZ(pd) = src.UZ(ps);
    dst.setpid(pd, src.getpid(ps));
}
__device__ __forceinline__ void copy_particle(const MixedView &dst, long long pd, const MixedView &src, long long ps)
{
    dst.XYUV(pd) = src.XYUV(ps);
    dst.UZ(pd) = src.UZ(ps);
    dst.setpid(pd, src.getpid(ps));
}

// --------------------------------------------------------------------- fields
// NC components on the ghosted grid.  AOS = the reference layout (component fastest);
// otherwise one plane per component with x fastest.
template <int NC, bool AOS>
struct FView {
    double *b;
    int nxw, nyw;
    __device__ __forceinline__ double &operator()(int k, int ix, int iy) const
    {
        if (AOS) return b[k + NC * (ix + (long long)nxw * iy)];
        return b[((long long)k * nyw + iy) * nxw + ix];
    }
};

// ------------------------------------------------------------- device status
// Bits OR-ed into a device status word by kernels that detect bad input.
enum { WMDEV_CELL = 1, WMDEV_OVERFLOW = 2, WMDEV_ROWJUMP = 4, WMDEV_TIMEOUT = 8 };

// ------------------------------------------------------------------ host side
#define WM_CUDA(call)                                                                                       \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) {                                                                            \
            fprintf(stderr, "wumingpic2d: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                                              \
            return WM_ERR_CUDA;                                                                             \
        }                                                                                                   \
    } while (0)

#define WM_TRY(expr)              \
    do {                          \
        int s_ = (expr);          \
        if (s_ != WM_OK) return s_; \
    } while (0)

inline int wm_check_launch(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "wumingpic2d: launch of %s failed: %s\n", what, cudaGetErrorString(e));
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

static inline unsigned wm_div_up(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Device buffer that grows on demand.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    int ensure(size_t n)
    {
        if (n <= bytes) return WM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) return WM_OK;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            fprintf(stderr, "wumingpic2d: cudaMalloc(%zu) failed: %s\n", n, cudaGetErrorString(e));
            p = nullptr;
            return WM_ERR_CUDA;
        }
        bytes = n;
        return WM_OK;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const
    {
        return static_cast<T *>(p);
    }
};

// Rebin scratch shared by particle_y, the sort and the fused step.
struct WmRebinScratch {
    unsigned char *dir;   // [cap] 0 stay, 1 up, 2 down
    int *ord;             // [cap]
    int *P;               // [cap] 1-based slot after particle_y
    int *key;             // [cap] destination cell key
    int *holes;           // [cap] hole slots per row (indexed like particles)
    int *nup, *ndown;     // [nrows]
    int *cellcnt;         // [nrows*nx]
    unsigned long long *pairs;  // [cap]
    int *np2_new;         // [nrows]
    long long *rowbase_new;  // [nrows+1]
    unsigned *status;     // device status word
};
