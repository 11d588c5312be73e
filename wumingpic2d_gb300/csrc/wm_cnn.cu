// wm_cnn.cu -- the learned initial guess for the implicit field solve: a six-layer 3x3
// convolutional network (9 -> 48 -> 48 -> 48 -> 48 -> 48 -> 3 channels, GELU between layers) on
// the periodic cell grid, with BF16 tensor-core implicit-GEMM kernels for inference and training.
//
// The network maps (E, B at time n; J at n+1/2) to the magnetic-field increment dB that the CG of
// common/field.f90:319-461 solves for.  The reference has no such component: plain CG from the
// previous step's dB (field.f90:355) stays the fallback, and the solve still runs to the same
// residual tolerance whichever guess it starts from.
//
// Layout: activations NHWC (channels fastest) in BF16, one image per sample, periodic in both
// directions; layer weights [tap][cout][cin] in BF16 with tap = (dy+1)*3 + (dx+1), so that
//   out(y, x, co) = b(co) + sum_{tap, ci} W(tap, co, ci) * in((y+dy) mod H, (x+dx) mod W, ci).
// Channel counts are padded to the tensor-core tile: the 9 inputs to 16, the 3 outputs to 8 (16
// for the output gradient), with zero weights on the padding.
//
// The convolutions (forward and input gradient) and the weight gradient run on the 5th-generation
// tensor cores (tcgen05.mma, wm_cnn_tc.cu) when the image is a multiple of 16 x 8 pixels.  The
// kernels here use mma.sync.m16n8k16 BF16 with FP32 accumulation, operands staged in shared memory
// and read with ldmatrix: other shapes, and every convolution on request (WM_CNN_MMA_SYNC, the
// cross-check of the tcgen05 kernels).  A CTA computes an 8 x 16 pixel tile for all output channels; it keeps
// the layer's weights resident in shared memory and walks over tiles (persistent grid).
#include <algorithm>
#include <cmath>
#include <cstdint>

#include <cuda_bf16.h>

#include "wm_launch.cuh"

namespace {

constexpr int TH = 8, TWD = 16;  // output tile: 8 rows x 16 pixels

// Status word of the public entry points' tensor-core kernels (WMDEV_TIMEOUT when a bounded wait
// ran out); read and cleared by wm_cnn_status.
__device__ unsigned g_cnn_status;
unsigned *cnn_status_word()
{
    void *p = nullptr;
    return cudaGetSymbolAddress(&p, g_cnn_status) == cudaSuccess ? static_cast<unsigned *>(p) : nullptr;
}
constexpr int HALO_H = TH + 2, HALO_W = TWD + 2;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(smem_addr(p)));
}
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z)
{
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// Copy one 8 x 16 tile's (10 x 18)-pixel periodic halo of a [n][H][W][C] BF16 image into shared
// memory rows of C + 8 elements (the pad keeps ldmatrix rows on distinct banks).
template <int C>
__device__ __forceinline__ void load_halo(__nv_bfloat16 *dst, const __nv_bfloat16 *__restrict__ src, int n, int H, int W, int y0, int x0)
{
    constexpr int V = C / 8;  // 16-byte vectors per pixel
    for (int e = threadIdx.x; e < HALO_H * HALO_W * V; e += blockDim.x) {
        const int v = e % V, pix = e / V, hx = pix % HALO_W, hy = pix / HALO_W;
        int yy = y0 - 1 + hy, xx = x0 - 1 + hx;
        yy += (yy < 0) ? H : (yy >= H ? -H : 0);
        xx += (xx < 0) ? W : (xx >= W ? -W : 0);
        const uint4 val = *reinterpret_cast<const uint4 *>(src + (((long long)n * H + yy) * W + xx) * C + v * 8);
        *reinterpret_cast<uint4 *>(dst + pix * (C + 8) + v * 8) = val;
    }
}

enum { EPI_TRAIN = 0, EPI_INFER = 1, EPI_LINEAR = 2, EPI_BWD = 3 };

// Implicit-GEMM 3x3 convolution: M = 16 pixels of a tile row per warp tile, N = COUT, K = 9 taps x
// CIN.  Four warps, each two tile rows.  Epilogues: TRAIN (z = acc + b stored as BF16, a = GELU(z)
// as BF16), INFER (a only), LINEAR (acc + b as FP32), BWD (no bias; acc * GELU'(zprev) as BF16: the
// input gradient of the previous layer's pre-activation).
template <int CIN, int COUT, int EPI, bool GROUPED>
__global__ void __launch_bounds__(128) k_conv3x3(const __nv_bfloat16 *__restrict__ in, const __nv_bfloat16 *__restrict__ wk,
                                                 const float *__restrict__ bias, int nimg, int H, int W, void *out,
                                                 __nv_bfloat16 *__restrict__ zout, const __nv_bfloat16 *__restrict__ zprev)
{
    constexpr int CP = CIN + 8, NT = COUT / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16 *w_s = reinterpret_cast<__nv_bfloat16 *>(smem_raw);  // [9][COUT][CP]
    __nv_bfloat16 *x_s = w_s + 9 * COUT * CP;                          // [HALO_H][HALO_W][CP]
    for (int e = threadIdx.x; e < 9 * COUT * (CIN / 8); e += blockDim.x) {
        const int v = e % (CIN / 8), row = e / (CIN / 8);
        *reinterpret_cast<uint4 *>(w_s + row * CP + v * 8) = *reinterpret_cast<const uint4 *>(wk + (long long)row * CIN + v * 8);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int ntx = W / TWD, nty = H / TH;
    const long long ntiles = (long long)nimg * nty * ntx;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int n = (int)(tile / ((long long)nty * ntx));
        const int rem = (int)(tile % ((long long)nty * ntx));
        const int y0 = (rem / ntx) * TH, x0 = (rem % ntx) * TWD;
        __syncthreads();  // previous tile's reads of x_s are done (and the weights are in)
        load_halo<CIN>(x_s, in, n, H, W, y0, x0);
        __syncthreads();
        float acc[2][NT][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int j = 0; j < NT; ++j)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[mt][j][q] = 0.f;
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
                uint32_t a[2][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
                    ldsm_x4(a[mt], x_s + ((2 * warp + mt + dy + 1) * HALO_W + (lane & 15) + dx + 1) * CP + kc * 16 + (lane >> 4) * 8);
                if constexpr (NT == 1) {
                    uint32_t b[2];
                    ldsm_x2(b, w_s + (tap * COUT + (lane & 7)) * CP + kc * 16 + ((lane >> 3) & 1) * 8);
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) mma_bf16(acc[mt][0], a[mt], b[0], b[1]);
                } else {
#pragma unroll
                    for (int jp = 0; jp < NT / 2; ++jp) {
                        if (GROUPED && jp != kc) continue;  // block-diagonal: output group jp reads input group jp only
                        uint32_t b[4];
                        ldsm_x4(b, w_s + (tap * COUT + 16 * jp + (lane >> 4) * 8 + (lane & 7)) * CP + kc * 16 + ((lane >> 3) & 1) * 8);
#pragma unroll
                        for (int mt = 0; mt < 2; ++mt) {
                            mma_bf16(acc[mt][2 * jp], a[mt], b[0], b[1]);
                            mma_bf16(acc[mt][2 * jp + 1], a[mt], b[2], b[3]);
                        }
                    }
                }
            }
        }
        // epilogue: acc[mt][j][0..1] = pixel (row 2*warp+mt, x g), channels 8j+2t, +1; [2..3] = x g+8
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const long long p = ((long long)n * H + y0 + 2 * warp + mt) * W + x0 + g + 8 * h;
#pragma unroll
                for (int j = 0; j < NT; ++j) {
                    const int co = 8 * j + 2 * t;
                    float v0 = acc[mt][j][2 * h], v1 = acc[mt][j][2 * h + 1];
                    if constexpr (EPI == EPI_BWD) {
                        const __nv_bfloat162 zz = *reinterpret_cast<const __nv_bfloat162 *>(zprev + p * COUT + co);
                        v0 *= gelu_grad(__bfloat162float(zz.x));
                        v1 *= gelu_grad(__bfloat162float(zz.y));
                        *reinterpret_cast<__nv_bfloat162 *>(static_cast<__nv_bfloat16 *>(out) + p * COUT + co) = __floats2bfloat162_rn(v0, v1);
                    } else {
                        v0 += bias[co];
                        v1 += bias[co + 1];
                        if constexpr (EPI == EPI_LINEAR) {
                            *reinterpret_cast<float2 *>(static_cast<float *>(out) + p * COUT + co) = make_float2(v0, v1);
                        } else {
                            if constexpr (EPI == EPI_TRAIN)
                                *reinterpret_cast<__nv_bfloat162 *>(zout + p * COUT + co) = __floats2bfloat162_rn(v0, v1);
                            *reinterpret_cast<__nv_bfloat162 *>(static_cast<__nv_bfloat16 *>(out) + p * COUT + co) =
                                __floats2bfloat162_rn(gelu(v0), gelu(v1));
                        }
                    }
                }
            }
    }
}

// Weight gradient dW(tap, co, ci) = sum_p dz(p, co) * x(p + d_tap, ci) and bias gradient
// db(co) = sum_p dz(p, co), per CTA over its tiles (nine warps, one per tap), written as per-CTA
// partials that k_reduce_partials sums in CTA order.
template <int CIN, int COUTP, bool GROUPED>
__global__ void __launch_bounds__(288) k_conv3x3_wgrad(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ dz, int nimg,
                                                       int H, int W, float *__restrict__ part)
{
    constexpr int CP = CIN + 8, DP = COUTP + 8, MT = COUTP / 16, NT = CIN / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16 *x_s = reinterpret_cast<__nv_bfloat16 *>(smem_raw);  // [HALO_H][HALO_W][CP]
    __nv_bfloat16 *d_s = x_s + HALO_H * HALO_W * CP;                   // [TH*TWD][DP]
    const int lane = threadIdx.x & 31, tap = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3, q = lane >> 3;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int ntx = W / TWD, nty = H / TH;
    const long long ntiles = (long long)nimg * nty * ntx;
    float acc[MT][NT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[mt][j][k] = 0.f;
    float dbias = 0.f;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int n = (int)(tile / ((long long)nty * ntx));
        const int rem = (int)(tile % ((long long)nty * ntx));
        const int y0 = (rem / ntx) * TH, x0 = (rem % ntx) * TWD;
        __syncthreads();
        load_halo<CIN>(x_s, x, n, H, W, y0, x0);
        for (int e = threadIdx.x; e < TH * TWD * (COUTP / 8); e += blockDim.x) {
            const int v = e % (COUTP / 8), pix = e / (COUTP / 8), py = pix / TWD, px = pix % TWD;
            *reinterpret_cast<uint4 *>(d_s + pix * DP + v * 8) =
                *reinterpret_cast<const uint4 *>(dz + (((long long)n * H + y0 + py) * W + x0 + px) * COUTP + v * 8);
        }
        __syncthreads();
        if (threadIdx.x < COUTP)
            for (int pix = 0; pix < TH * TWD; ++pix) dbias += __bfloat162float(d_s[pix * DP + threadIdx.x]);
#pragma unroll 1
        for (int r = 0; r < TH; ++r) {  // k-step: the 16 pixels of tile row r
            uint32_t a[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) ldsm_x4_t(a[mt], d_s + (r * TWD + (q >> 1) * 8 + (lane & 7)) * DP + mt * 16 + (q & 1) * 8);
#pragma unroll
            for (int jp = 0; jp < NT / 2; ++jp) {
                uint32_t b[4];
                ldsm_x4_t(b, x_s + ((r + dy + 1) * HALO_W + (q & 1) * 8 + (lane & 7) + dx + 1) * CP + 8 * (2 * jp + (q >> 1)));
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) {
                    if (GROUPED && mt != jp) continue;  // off-block gradients stay zero
                    mma_bf16(acc[mt][2 * jp], a[mt], b[0], b[1]);
                    mma_bf16(acc[mt][2 * jp + 1], a[mt], b[2], b[3]);
                }
            }
        }
    }
    // partial layout [cta][9][COUTP][CIN] then [COUTP] bias
    float *pw = part + (long long)blockIdx.x * (9 * COUTP * CIN + COUTP);
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int co = mt * 16 + g + 8 * h, ci = 8 * j + 2 * t;
                *reinterpret_cast<float2 *>(pw + (tap * COUTP + co) * CIN + ci) = make_float2(acc[mt][j][2 * h], acc[mt][j][2 * h + 1]);
            }
    if (threadIdx.x < COUTP) pw[9 * COUTP * CIN + threadIdx.x] = dbias;
}

// dW(tap, co, ci) for co < cout (and db(co)) = sum over CTAs, in CTA order.
__global__ void k_reduce_wgrad(const float *__restrict__ part, int nparts, int cin, int coutp, int cout, float *__restrict__ dw,
                               float *__restrict__ db)
{
    const int per = 9 * coutp * cin + coutp;
    const int nw = 9 * cout * cin;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nw + cout; e += gridDim.x * blockDim.x) {
        int src;
        if (e < nw) {
            const int ci = e % cin, co = (e / cin) % cout, tap = e / (cin * cout);
            src = (tap * coutp + co) * cin + ci;
        } else {
            src = 9 * coutp * cin + (e - nw);
        }
        float s = 0.f;
        for (int k = 0; k < nparts; ++k) s += part[(long long)k * per + src];
        if (e < nw) dw[e] = s;
        else db[e - nw] = s;
    }
}

// Loss 0.5/count * sum (pred - target)^2 over the three real output channels; dz = dL/dpred as
// BF16 [p][16] (zeros on the padding).  Per-block partial sums, then one block adds them in order.
// border > 0: the pixels within `border` of an image edge ([.][H][W] images) are left out of the
// loss and get dz = 0 (crops of a larger field, whose periodic padding is not the field's).
__global__ void k_mse(const float *__restrict__ pred, const float *__restrict__ target, long long npix, int H, int W, int border, float scale,
                      __nv_bfloat16 *__restrict__ dz, double *__restrict__ partial)
{
    __shared__ double red[256];
    double s = 0.0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        bool in = true;
        if (border > 0) {
            const int x = (int)(p % W), y = (int)((p / W) % H);
            in = x >= border && x < W - border && y >= border && y < H - border;
        }
        float e[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            e[c] = in ? pred[p * 8 + c] - target[p * 3 + c] : 0.f;
            s += (double)e[c] * e[c];
        }
        const __nv_bfloat162 e01 = __floats2bfloat162_rn(scale * e[0], scale * e[1]);
        const __nv_bfloat162 e2 = __floats2bfloat162_rn(scale * e[2], 0.f);
        uint4 *d = reinterpret_cast<uint4 *>(dz + p * 16);
        d[0] = make_uint4(*reinterpret_cast<const unsigned *>(&e01), *reinterpret_cast<const unsigned *>(&e2), 0u, 0u);
        d[1] = make_uint4(0u, 0u, 0u, 0u);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_sum_in_order(const double *__restrict__ partial, int n, double scale, double *__restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += partial[k];
        *out = scale * s;
    }
}

// Adam on the FP32 master parameters (bias-corrected step size precomputed on the host).
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ gr, const float *__restrict__ mask, float *__restrict__ m,
                       float *__restrict__ v, long long n, float lr_t, float b1, float b2, float eps)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float gg = mask ? gr[e] * mask[e] : gr[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        p[e] -= lr_t * mm / (sqrtf(vv) + eps);
    }
}

// Layer weights from the FP32 master: forward [tap][cout][cin] in BF16 and, for the input
// gradient, the flipped transpose Wt(tap', ci, co) = W(8 - tap', co, ci) with co padded to coutb.
__global__ void k_prep_weights(const float *__restrict__ w, int cin, int cout, int coutb, __nv_bfloat16 *__restrict__ wf,
                               __nv_bfloat16 *__restrict__ wt)
{
    const int nf = 9 * cout * cin, nt = wt ? 9 * cin * coutb : 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nf + nt; e += gridDim.x * blockDim.x) {
        if (e < nf) {
            wf[e] = __float2bfloat16(w[e]);
        } else {
            const int k = e - nf;
            const int co = k % coutb, ci = (k / coutb) % cin, tp = k / (coutb * cin);
            wt[k] = __float2bfloat16(co < cout ? w[((8 - tp) * cout + co) * cin + ci] : 0.f);
        }
    }
}

template <int CIN, int COUT, int EPI, bool GROUPED = false>
int launch_conv(const void *in, const void *wk, const float *bias, int nimg, int H, int W, void *out, void *zout, const void *zprev,
                cudaStream_t st)
{
    constexpr int CP = CIN + 8;
    const size_t smem = sizeof(__nv_bfloat16) * (9 * COUT * CP + HALO_H * HALO_W * CP);
    WM_CUDA(cudaFuncSetAttribute(k_conv3x3<CIN, COUT, EPI, GROUPED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long ntiles = (long long)nimg * (H / TH) * (W / TWD);
    const int grid = (int)std::min<long long>(ntiles, 152LL * 3);
    k_conv3x3<CIN, COUT, EPI, GROUPED><<<grid, 128, smem, st>>>(static_cast<const __nv_bfloat16 *>(in), static_cast<const __nv_bfloat16 *>(wk), bias,
                                                        nimg, H, W, out, static_cast<__nv_bfloat16 *>(zout),
                                                        static_cast<const __nv_bfloat16 *>(zprev));
    return wm_check_launch("k_conv3x3");
}

template <int CIN, int COUTP, bool GROUPED = false>
int launch_wgrad(const void *x, const void *dz, int nimg, int H, int W, int cout, float *dw, float *db, float *scratch,
                 long long scratch_floats, cudaStream_t st)
{
    constexpr int CP = CIN + 8, DP = COUTP + 8;
    const size_t smem = sizeof(__nv_bfloat16) * (HALO_H * HALO_W * CP + TH * TWD * DP);
    const long long ntiles = (long long)nimg * (H / TH) * (W / TWD);
    const long long per = 9LL * COUTP * CIN + COUTP;
    int grid = (int)std::min<long long>(ntiles, 152LL * 2);
    grid = (int)std::min<long long>(grid, scratch_floats / per);
    if (grid < 1) return WM_ERR_BAD_ARG;
    k_conv3x3_wgrad<CIN, COUTP, GROUPED><<<grid, 288, smem, st>>>(static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(dz), nimg,
                                                         H, W, scratch);
    WM_TRY(wm_check_launch("k_conv3x3_wgrad"));
    const int nout = 9 * cout * CIN + cout;
    k_reduce_wgrad<<<(nout + 255) / 256, 256, 0, st>>>(scratch, grid, CIN, COUTP, cout, dw, db);
    return wm_check_launch("k_reduce_wgrad");
}

bool shape_ok(int nimg, int H, int W) { return nimg > 0 && H >= TH && W >= TWD && H % TH == 0 && W % TWD == 0; }

// ---------------------------------------------------------------- inference inside the solve
// The CG unknowns decouple: dBx depends on (Bx, Ez, Jz) only, dBy on (By, Ez, Jz), dBz on (Bz, Ex,
// Ey, Jx, Jy) (the right-hand side of field.f90:125-146 and a diagonal operator per component).
// Input channels, each group divided by its own root mean square s_k over the grid:
//   0-2 (Bx, Ez, Jz)/s_x, 3-5 (By, Ez, Jz)/s_y, 6-10 (Bz, Ex, Ey, Jx, Jy)/s_z, 11-15 zero,
// read at each cell's stored Yee index (i+2, j+2).  The network's weights are block-diagonal over
// the three groups, so the guess is (s_x, s_y, s_z) * net(input), exact in scale per component.
constexpr int GUESS_NIN = 11;
__device__ __forceinline__ double raw_input(const FView<6, false> &uf, const FView<3, false> &uj, int c, int ix, int iy)
{
    // c: 0-2 Ex, Ey, Ez; 3-5 Bx, By, Bz; 6-8 Jx, Jy, Jz
    if (c < 3) return uf(3 + c, ix, iy);
    if (c < 6) return uf(c - 3, ix, iy);
    return uj(c - 6, ix, iy);
}
__device__ __forceinline__ int packed_source(int k)
{
    constexpr int src[GUESS_NIN] = {3, 2, 8, 4, 2, 8, 5, 0, 1, 6, 7};
    return src[k];
}
__device__ __forceinline__ int packed_group(int k) { return k < 3 ? 0 : (k < 6 ? 1 : 2); }

__global__ void k_guess_sumsq(WmGeom g, FView<6, false> uf, FView<3, false> uj, double *__restrict__ partial)
{
    __shared__ double red[3][256];
    const long long ncell = (long long)g.nx * g.ny;
    double s[3] = {0.0, 0.0, 0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncell; e += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(e % g.nx) + 2, iy = (int)(e / g.nx) + 2;
#pragma unroll
        for (int k = 0; k < GUESS_NIN; ++k) {
            const double v = raw_input(uf, uj, packed_source(k), ix, iy);
            s[packed_group(k)] += v * v;
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) red[q][threadIdx.x] = s[q];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
#pragma unroll
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3) partial[3 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

// scale[k] = s_k (root mean square of group k), scale[3+k] = 1/s_k (0 for an all-zero group)
__global__ void k_guess_scale(const double *__restrict__ partial, int n, long long ncell, double *__restrict__ scale)
{
    if (blockIdx.x == 0 && threadIdx.x < 3) {
        const int q = threadIdx.x;
        double t = 0.0;
        for (int k = 0; k < n; ++k) t += partial[3 * k + q];
        const double s = sqrt(t / ((q == 2 ? 5.0 : 3.0) * (double)ncell));
        scale[q] = s;
        scale[3 + q] = s > 0.0 ? 1.0 / s : 0.0;
    }
}

__global__ void k_guess_pack(WmGeom g, FView<6, false> uf, FView<3, false> uj, const double *__restrict__ scale,
                             __nv_bfloat16 *__restrict__ x)
{
    const long long ncell = (long long)g.nx * g.ny;
    const double inv[3] = {scale[3], scale[4], scale[5]};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncell; e += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(e % g.nx) + 2, iy = (int)(e / g.nx) + 2;
        unsigned w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int c0 = 2 * k, c1 = 2 * k + 1;
            const float lo = c0 < GUESS_NIN ? (float)(raw_input(uf, uj, packed_source(c0), ix, iy) * inv[packed_group(c0)]) : 0.f;
            const float hi = c1 < GUESS_NIN ? (float)(raw_input(uf, uj, packed_source(c1), ix, iy) * inv[packed_group(c1)]) : 0.f;
            const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
            w[k] = *reinterpret_cast<const unsigned *>(&v);
        }
        uint4 *d = reinterpret_cast<uint4 *>(x + e * 16);
        d[0] = make_uint4(w[0], w[1], w[2], w[3]);
        d[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// cand[l][j*nx + i] = s_l * pred(j, i, l), l = dBx, dBy, dBz
__global__ void k_guess_unpack(WmGeom g, const float *__restrict__ pred, const double *__restrict__ scale, double *__restrict__ cand)
{
    const long long ncell = (long long)g.nx * g.ny;
    const double s[3] = {scale[0], scale[1], scale[2]};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncell; e += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int l = 0; l < 3; ++l) cand[l * ncell + e] = s[l] * (double)pred[e * 8 + l];
    }
}

}  // namespace

size_t wm_cnn_param_count()
{
    size_t n = 0;
    for (int l = 0; l < WM_CNN_LAYERS; ++l) n += 9 * (size_t)wm_cnn_cin[l] * wm_cnn_cout[l] + wm_cnn_cout[l];
    return n;
}

int wm_cnn_net_prepare(WmCnnNet &net, cudaStream_t st)
{
    size_t off = 0;
    for (int l = 0; l < WM_CNN_LAYERS; ++l) {
        const int cin = wm_cnn_cin[l], cout = wm_cnn_cout[l];
        WM_TRY(wm_cnn_prep_weights(net.params + off, cin, cout, cout, net.wf[l], nullptr, st));
        net.bias[l] = net.params + off + 9 * (size_t)cin * cout;
        off += 9 * (size_t)cin * cout + cout;
    }
    return WM_OK;
}

int wm_cnn_infer_guess(const WmGeom &g, const WmCnnNet &net, FView<6, false> uf, FView<3, false> uj, const WmCnnWork &w, double *cand,
                       cudaStream_t st, unsigned *status)
{
    if (!shape_ok(1, g.ny, g.nx)) return WM_ERR_BAD_ARG;
    const long long ncell = (long long)g.nx * g.ny;
    const int blocks = (int)std::min<long long>((ncell + 255) / 256, WM_CNN_RED_BLOCKS);
    k_guess_sumsq<<<blocks, 256, 0, st>>>(g, uf, uj, w.partial);
    WM_TRY(wm_check_launch("k_guess_sumsq"));
    k_guess_scale<<<1, 32, 0, st>>>(w.partial, blocks, ncell, w.scale);
    WM_TRY(wm_check_launch("k_guess_scale"));
    k_guess_pack<<<blocks, 256, 0, st>>>(g, uf, uj, w.scale, static_cast<__nv_bfloat16 *>(w.x));
    WM_TRY(wm_check_launch("k_guess_pack"));
    const void *in = w.x;
    void *bufs[2] = {w.a0, w.a1};
    for (int l = 0; l < WM_CNN_LAYERS - 1; ++l) {
        if (wm_cnn_tc_shape_ok(1, g.ny, g.nx)) {  // tensor cores (tcgen05)
            WM_TRY(wm_cnn_conv3x3_tc(in, net.wf[l], net.bias[l], wm_cnn_cin[l], wm_cnn_cout[l], WM_CNN_FWD_INFER, 1, g.ny, g.nx, bufs[l & 1],
                                     nullptr, nullptr, status, st));
        } else {
            const int grp = (wm_cnn_cin[l] == 48 && wm_cnn_cout[l] == 48) ? WM_CNN_GROUPED : 0;
            WM_TRY(wm_cnn_conv3x3(in, net.wf[l], net.bias[l], wm_cnn_cin[l], wm_cnn_cout[l], WM_CNN_FWD_INFER | grp | WM_CNN_MMA_SYNC, 1,
                                  g.ny, g.nx, bufs[l & 1], nullptr, nullptr, st));
        }
        in = bufs[l & 1];
    }
    const int L = WM_CNN_LAYERS - 1;
    if (wm_cnn_tc_shape_ok(1, g.ny, g.nx))
        WM_TRY(wm_cnn_conv3x3_tc(in, net.wf[L], net.bias[L], wm_cnn_cin[L], wm_cnn_cout[L], WM_CNN_FWD_LINEAR, 1, g.ny, g.nx, w.pred, nullptr,
                                 nullptr, status, st));
    else
        WM_TRY(wm_cnn_conv3x3(in, net.wf[L], net.bias[L], wm_cnn_cin[L], wm_cnn_cout[L], WM_CNN_FWD_LINEAR | WM_CNN_MMA_SYNC, 1, g.ny, g.nx,
                              w.pred, nullptr, nullptr, st));
    k_guess_unpack<<<blocks, 256, 0, st>>>(g, w.pred, w.scale, cand);
    return wm_check_launch("k_guess_unpack");
}

extern "C" {

int wm_cnn_conv3x3(const void *in, const void *w, const float *bias, int cin, int cout, int mode, int nimg, int h, int wd, void *out,
                   void *zout, const void *zprev, void *stream)
{
    if (!in || !w || !out || !shape_ok(nimg, h, wd)) return WM_ERR_BAD_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool grouped = (mode & WM_CNN_GROUPED) != 0, legacy = (mode & WM_CNN_MMA_SYNC) != 0;
    mode &= ~(WM_CNN_GROUPED | WM_CNN_MMA_SYNC);
    const bool tc = (cout == 48 && (cin == 16 || cin == 48) && (mode == WM_CNN_FWD_TRAIN || mode == WM_CNN_FWD_INFER || mode == WM_CNN_BWD)) ||
                    (cout == 8 && cin == 48 && mode == WM_CNN_FWD_LINEAR);
    if (!legacy && tc && wm_cnn_tc_shape_ok(nimg, h, wd)) {
        unsigned *status = cnn_status_word();
        if (!status) return WM_ERR_CUDA;
        return wm_cnn_conv3x3_tc(in, w, bias, cin, cout, mode, nimg, h, wd, out, zout, zprev, status, st);
    }
    if (mode != WM_CNN_BWD && !bias) return WM_ERR_BAD_ARG;
    if (mode == WM_CNN_FWD_TRAIN && !zout) return WM_ERR_BAD_ARG;
    if (mode == WM_CNN_BWD && !zprev) return WM_ERR_BAD_ARG;
    if (cin == 16 && cout == 48) {
        if (mode == WM_CNN_FWD_TRAIN) return launch_conv<16, 48, EPI_TRAIN>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
        if (mode == WM_CNN_FWD_INFER) return launch_conv<16, 48, EPI_INFER>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
        if (mode == WM_CNN_BWD) return launch_conv<16, 48, EPI_BWD>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
    } else if (cin == 48 && cout == 48 && grouped) {
        if (mode == WM_CNN_FWD_TRAIN) return launch_conv<48, 48, EPI_TRAIN, true>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
        if (mode == WM_CNN_FWD_INFER) return launch_conv<48, 48, EPI_INFER, true>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
        if (mode == WM_CNN_BWD) return launch_conv<48, 48, EPI_BWD, true>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
    } else if (cin == 48 && cout == 48) {
        if (mode == WM_CNN_FWD_TRAIN) return launch_conv<48, 48, EPI_TRAIN>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
        if (mode == WM_CNN_FWD_INFER) return launch_conv<48, 48, EPI_INFER>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
        if (mode == WM_CNN_BWD) return launch_conv<48, 48, EPI_BWD>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
    } else if (cin == 48 && cout == 8) {
        if (mode == WM_CNN_FWD_LINEAR) return launch_conv<48, 8, EPI_LINEAR>(in, w, bias, nimg, h, wd, out, zout, zprev, st);
    }
    return WM_ERR_UNSUPPORTED;
}

int wm_cnn_status(int clear)
{
    unsigned v = 0;
    WM_CUDA(cudaMemcpyFromSymbol(&v, g_cnn_status, sizeof v));
    if (clear) {
        const unsigned z = 0;
        WM_CUDA(cudaMemcpyToSymbol(g_cnn_status, &z, sizeof z));
    }
    return (v & WMDEV_TIMEOUT) ? WM_ERR_CUDA : WM_OK;
}

int wm_cnn_conv3x3_wgrad(const void *x, const void *dz, int cin, int coutp, int cout, int nimg, int h, int wd, int flags, float *dw,
                         float *db, float *scratch, long long scratch_floats, void *stream)
{
    if (!x || !dz || !dw || !db || !scratch || !shape_ok(nimg, h, wd) || cout < 1 || cout > coutp) return WM_ERR_BAD_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool shape_tc = (cin == 16 && coutp == 48) || (cin == 48 && (coutp == 48 || coutp == 16));
    if (!(flags & WM_CNN_MMA_SYNC) && shape_tc && wm_cnn_tc_shape_ok(nimg, h, wd)) {  // tensor cores (tcgen05)
        unsigned *status = cnn_status_word();
        if (!status) return WM_ERR_CUDA;
        int nparts = 0;
        WM_TRY(wm_cnn_wgrad_tc(x, dz, cin, coutp, (flags & WM_CNN_GROUPED) != 0, nimg, h, wd, scratch, scratch_floats, &nparts, status, st));
        const int nout = 9 * cout * cin + cout;
        k_reduce_wgrad<<<(nout + 255) / 256, 256, 0, st>>>(scratch, nparts, cin, coutp, cout, dw, db);
        return wm_check_launch("k_reduce_wgrad");
    }
    if ((flags & WM_CNN_GROUPED) && cin == 48 && coutp == 48)
        return launch_wgrad<48, 48, true>(x, dz, nimg, h, wd, cout, dw, db, scratch, scratch_floats, st);
    if (cin == 16 && coutp == 48) return launch_wgrad<16, 48>(x, dz, nimg, h, wd, cout, dw, db, scratch, scratch_floats, st);
    if (cin == 48 && coutp == 48) return launch_wgrad<48, 48>(x, dz, nimg, h, wd, cout, dw, db, scratch, scratch_floats, st);
    if (cin == 48 && coutp == 16) return launch_wgrad<48, 16>(x, dz, nimg, h, wd, cout, dw, db, scratch, scratch_floats, st);
    return WM_ERR_UNSUPPORTED;
}

int wm_cnn_mse(const float *pred, const float *target, long long npix, void *dz, double *partial, int nblocks, double *loss, void *stream)
{
    if (!pred || !target || !dz || !partial || !loss || npix <= 0 || nblocks < 1) return WM_ERR_BAD_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const double count = 3.0 * (double)npix;
    k_mse<<<nblocks, 256, 0, st>>>(pred, target, npix, 1, 1, 0, (float)(1.0 / count), static_cast<__nv_bfloat16 *>(dz), partial);
    WM_TRY(wm_check_launch("k_mse"));
    k_sum_in_order<<<1, 32, 0, st>>>(partial, nblocks, 0.5 / count, loss);
    return wm_check_launch("k_sum_in_order");
}

int wm_cnn_mse_interior(const float *pred, const float *target, int nimg, int h, int wd, int border, void *dz, double *partial, int nblocks,
                        double *loss, void *stream)
{
    if (!pred || !target || !dz || !partial || !loss || nimg < 1 || border < 0 || h <= 2 * border || wd <= 2 * border || nblocks < 1)
        return WM_ERR_BAD_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long npix = (long long)nimg * h * wd;
    const double count = 3.0 * (double)nimg * (h - 2 * border) * (wd - 2 * border);
    k_mse<<<nblocks, 256, 0, st>>>(pred, target, npix, h, wd, border, (float)(1.0 / count), static_cast<__nv_bfloat16 *>(dz), partial);
    WM_TRY(wm_check_launch("k_mse"));
    k_sum_in_order<<<1, 32, 0, st>>>(partial, nblocks, 0.5 / count, loss);
    return wm_check_launch("k_sum_in_order");
}

int wm_cnn_adam(float *p, const float *grad, const float *mask, float *m, float *v, long long n, float lr, float beta1, float beta2,
                float eps, int step, void *stream)
{
    if (!p || !grad || !m || !v || n <= 0 || step < 1) return WM_ERR_BAD_ARG;
    const double bc1 = 1.0 - std::pow((double)beta1, step), bc2 = 1.0 - std::pow((double)beta2, step);
    const float lr_t = (float)(lr * std::sqrt(bc2) / bc1);
    const float eps_t = (float)(eps * std::sqrt(bc2));
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 8);
    k_adam<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(p, grad, mask, m, v, n, lr_t, beta1, beta2, eps_t);
    return wm_check_launch("k_adam");
}

int wm_cnn_prep_weights(const float *w, int cin, int cout, int coutb, void *wf, void *wt, void *stream)
{
    if (!w || !wf || cin < 1 || cout < 1 || (wt && coutb < cout)) return WM_ERR_BAD_ARG;
    const int n = 9 * cout * cin + (wt ? 9 * cin * coutb : 0);
    k_prep_weights<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(w, cin, cout, coutb, static_cast<__nv_bfloat16 *>(wf),
                                                                                     static_cast<__nv_bfloat16 *>(wt));
    return wm_check_launch("k_prep_weights");
}

}  // extern "C"
