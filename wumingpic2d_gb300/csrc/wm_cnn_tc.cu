// wm_cnn_tc.cu -- the 3x3 convolutions of the learned CG guess on the 5th-generation tensor cores:
// tcgen05.mma with both operands in shared memory and the FP32 accumulator in tensor memory (TMEM),
// read back with tcgen05.ld for the epilogue (bias + GELU, or GELU' for the input gradient of
// training).  The forward and input-gradient convolutions are described here; the weight gradient
// (k_conv3x3_wgrad_tc) further down.
//
// Implicit GEMM per CTA tile of 16 rows x 8 pixels: M = 128 pixels, N = 48 output channels,
// K = 9 taps x cin, one tcgen05.mma (M128 N48 K16) per tap and 16 input channels.  The tile's
// periodic halo (18 x 10 pixels) is stored in shared memory as 16-byte core-matrix rows,
// [channel group of 8][halo pixel][8 channels]: eight consecutive pixels of a halo row form one
// 8 x 16-byte core matrix, the next tile row is one halo row (160 bytes) further on and the next
// channel group one plane further on.  So the A operand of every tap is the same no-swizzle
// K-major layout with its start address moved by (dy, dx) -- no data is copied per tap.  The
// weights are stored [tap][channel group][cout][8 channels], the B operand of the same form.
// One thread issues the 27 (cin 48) or 9 (cin 16) MMAs of a tile and commits them to an mbarrier;
// the four warps then read their 32 TMEM lanes (pixels) and write the activations.
//
// The network and its arithmetic are those of wm_cnn.cu (BF16 operands, FP32 accumulation); block
// diagonal (grouped) weights are multiplied as they are, zeros included, which gives the grouped
// result exactly.  Waits on the mbarrier are bounded: on a timeout the kernel records
// WMDEV_TIMEOUT in its status word, waits (bounded) once more, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "wm_launch.cuh"

namespace {

constexpr int TC_TH = 16, TC_TW = 8;                  // output tile: 16 rows x 8 pixels (M = 128)
constexpr int TC_HW = TC_TW + 2, TC_HPIX = (TC_TH + 2) * TC_HW;  // halo 18 x 10 pixels
constexpr int TC_XP = 184;  // pixels per channel-group plane: 180 used, 2944 bytes keeps planes 128-byte aligned for TMA
constexpr uint32_t TC_SPIN = 1u << 22;                // mbarrier polls before giving up

// no-swizzle shared-memory matrix descriptor: start address, leading (K-direction) and stride
// (M/N-direction) byte offsets between 8 x 16-byte core matrices, descriptor version 1.  The same
// fields serve K-major operands (a core-matrix row = 8 K elements) and MN-major ones (a row = 8 M
// or N elements, the instruction descriptor's transpose bits set).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
           (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N and M = 128
constexpr uint32_t tc_idesc(int n) { return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24); }

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t i = 0; i < TC_SPIN; ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
                   "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu_tc(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
// d GELU / dz = Phi(z) + z phi(z)
__device__ __forceinline__ float gelu_grad_tc(float z)
{
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ void tma_halo(uint32_t dst, const CUtensorMap *tmap, int c0, int c1, int c2, int c3, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
                 : "memory");
}

// EPI: 0 = TRAIN (out = GELU(z), zout = z), 1 = INFER (out = GELU(z)); z = conv + bias, BF16,
// 48 channels.  2 = LINEAR: out = conv + bias in FP32 [.][COUT] with COUT = 8 real channels, the
// MMA's N padded to 16 with zero weights.  3 = BWD (the input gradient of training): out = conv *
// GELU'(zprev) in BF16, no bias.
// A CTA holds one copy of the layer's weights and runs TC_GROUPS independent groups of four warps,
// each with its own tiles, two halo buffers, mbarriers, TMEM accumulator and named barrier.  In a
// group, while a tile's MMAs and epilogue run, the next tile's halo arrives by TMA (tmap: the input
// [nimg][H][W][CIN] with boxes of 8 channels x 10 x 18 pixels) when it lies inside the image;
// tiles whose halo wraps around the periodic edges load it with plain loads.
constexpr int TC_GROUPS = 2;
template <int CIN, int NOUT, int COUT, int EPI>
__global__ void __launch_bounds__(128 * TC_GROUPS, 2) k_conv3x3_tc(const __grid_constant__ CUtensorMap tmap, const __nv_bfloat16 *__restrict__ in,
                                                                   const __nv_bfloat16 *__restrict__ wk, const float *__restrict__ bias,
                                                                   int nimg, int H, int W, void *__restrict__ out,
                                                                   __nv_bfloat16 *__restrict__ zout, const __nv_bfloat16 *__restrict__ zprev,
                                                                   unsigned *status)
{
    constexpr int KG = CIN / 8;                          // channel groups of 8 (16 bytes)
    constexpr uint32_t TMEM_COLS = NOUT > 32 ? 64 : 32;  // FP32 accumulator columns of a group (power of 2 >= N, >= 32)
    constexpr uint32_t IDESC = tc_idesc(NOUT);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __nv_bfloat16 *w_s = reinterpret_cast<__nv_bfloat16 *>(smem_raw);        // [9][KG][NOUT][8]
    __nv_bfloat16 *x_all = w_s + 9 * KG * NOUT * 8;                           // [group][2][KG][TC_XP][8]
    uint64_t *bar_all = reinterpret_cast<uint64_t *>(x_all + TC_GROUPS * 2 * KG * TC_XP * 8);  // [group][halo 0, halo 1, MMA 0, MMA 1]
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar_all + 4 * TC_GROUPS);
    __shared__ int give_up[TC_GROUPS];
    __shared__ float bias_s[NOUT];  // the layer's biases, read by every epilogue from shared memory
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = tid >> 7, gtid = tid & 127, gwarp = warp & 3;  // group, thread and warp in the group
    if constexpr (EPI != 3)
        for (int e = tid; e < NOUT; e += blockDim.x) bias_s[e] = e < COUT ? bias[e] : 0.f;

    for (int e = tid; e < 9 * NOUT * KG; e += blockDim.x) {  // [9][COUT][CIN] -> core-matrix rows, zero rows past COUT
        const int kg = e % KG, co = (e / KG) % NOUT, tap = e / (KG * NOUT);
        *reinterpret_cast<uint4 *>(w_s + ((tap * KG + kg) * NOUT + co) * 8) =
            co < COUT ? *reinterpret_cast<const uint4 *>(wk + ((long long)tap * COUT + co) * CIN + kg * 8) : make_uint4(0u, 0u, 0u, 0u);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)), "r"(TC_GROUPS * 2 * TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 4 * TC_GROUPS; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar_all + b)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        for (int g2 = 0; g2 < TC_GROUPS; ++g2) give_up[g2] = 0;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the weights, seen by the tensor core
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot + (uint32_t)(grp * 2 * TMEM_COLS);  // this group's two accumulators
    uint64_t *bars = bar_all + 4 * grp;                                  // [halo 0, halo 1, MMA 0, MMA 1]
    __nv_bfloat16 *x_s = x_all + grp * 2 * KG * TC_XP * 8;
    const uint32_t ws_a = saddr(w_s);
    auto xs = [&](int buf) { return saddr(x_s + buf * KG * TC_XP * 8); };
    auto gsync = [&]() { asm volatile("bar.sync %0, 128;\n" ::"r"(1 + grp) : "memory"); };

    const int ntx = W / TC_TW, nty = H / TC_TH;
    const long long ntiles = (long long)nimg * nty * ntx;
    const long long tstride = (long long)gridDim.x * TC_GROUPS, tfirst = (long long)blockIdx.x * TC_GROUPS + grp;
    auto coords = [&](long long t, int &n, int &y0, int &x0) {
        n = (int)(t / ((long long)nty * ntx));
        const int rem = (int)(t % ((long long)nty * ntx));
        y0 = (rem / ntx) * TC_TH;
        x0 = (rem % ntx) * TC_TW;
    };
    auto inside = [&](int y0, int x0) { return y0 >= 1 && y0 + TC_TH + 1 <= H && x0 >= 1 && x0 + TC_TW + 1 <= W; };
    // bit b: a TMA halo copy in flight into buffer b, its barrier's phase; MMAs committed to MMA
    // barrier b and not yet waited for, that barrier's phase
    uint32_t pending = 0u, hph = 0u, mma_out = 0u, mph = 0u;
    auto issue = [&](int buf, long long t) {  // all threads: the TMA copy of tile t's halo (one thread issues it)
        int n, y0, x0;
        coords(t, n, y0, x0);
        if (!inside(y0, x0)) return;  // periodic halo across the image edges: plain loads later
        if (gtid == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(bars + buf)), "r"((uint32_t)(KG * TC_HPIX * 16))
                         : "memory");
#pragma unroll
            for (int kg = 0; kg < KG; ++kg) tma_halo(xs(buf) + (uint32_t)(kg * TC_XP * 16), &tmap, kg * 8, x0 - 1, y0 - 1, n, saddr(bars + buf));
        }
        pending |= 1u << buf;
    };
    auto halo_ready = [&](int buf, long long t) -> bool {  // all threads: tile t's halo in buffer buf
        if (pending & (1u << buf)) {  // it came by TMA
            const bool ok = mbar_wait(saddr(bars + buf), (hph >> buf) & 1u);
            hph ^= 1u << buf;
            pending &= ~(1u << buf);
            return ok;
        }
        int n, y0, x0;
        coords(t, n, y0, x0);
        __nv_bfloat16 *xb = x_s + buf * KG * TC_XP * 8;
        for (int e = gtid; e < TC_HPIX * KG; e += 128) {
            const int kg = e % KG, pix = e / KG, hy = pix / TC_HW, hx = pix % TC_HW;
            int yy = y0 - 1 + hy, xx = x0 - 1 + hx;
            yy += (yy < 0) ? H : (yy >= H ? -H : 0);
            xx += (xx < 0) ? W : (xx >= W ? -W : 0);
            *reinterpret_cast<uint4 *>(xb + (kg * TC_XP + pix) * 8) =
                *reinterpret_cast<const uint4 *>(in + (((long long)n * H + yy) * W + xx) * CIN + kg * 8);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the halo stores, seen by the tensor core
        return true;
    };
    auto issue_mma = [&](int buf) {  // tile in halo buffer buf -> accumulator buf, committed to MMA barrier buf
        if (gtid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t xa = xs(buf), acc = tmem + (uint32_t)(buf * TMEM_COLS);
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
                const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
                for (int ks = 0; ks < KG / 2; ++ks) {
                    const uint64_t ad = smem_desc(xa + (uint32_t)((2 * ks * TC_XP + (dy + 1) * TC_HW + dx + 1) * 16), TC_XP * 16, TC_HW * 16);
                    const uint64_t bd = smem_desc(ws_a + (uint32_t)(((tap * KG + 2 * ks) * NOUT) * 16), NOUT * 16, 8 * 16);
                    mma_f16(acc, ad, bd, IDESC, (tap | ks) != 0 ? 1u : 0u);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bars + 2 + buf))
                         : "memory");
        }
        mma_out |= 1u << buf;
    };
    // Tile i of the group: halo buffer and accumulator i & 1.  Tile i+1's MMAs are issued before
    // tile i's epilogue, so they run while it reads the other accumulator; tile i+2's halo copy
    // starts once tile i's MMAs are done with its buffer.
    if (tfirst < ntiles) {
        issue(0, tfirst);
        if (tfirst + tstride < ntiles) issue(1, tfirst + tstride);
        if (!halo_ready(0, tfirst)) give_up[grp] = 1;
        gsync();
        if (!give_up[grp]) issue_mma(0);
    }
    int i = 0;
    for (long long tile = tfirst; tile < ntiles && !give_up[grp]; tile += tstride, ++i) {
        const int b = i & 1;
        int n, y0, x0;
        coords(tile, n, y0, x0);
        const long long nt = tile + tstride;
        if (nt < ntiles) {  // the next tile's MMAs into the other accumulator (its epilogue of tile i-1 ended at the last barrier)
            if (!halo_ready(b ^ 1, nt)) give_up[grp] = 1;
            gsync();
            if (give_up[grp]) break;
            issue_mma(b ^ 1);
        }
        if (!mbar_wait(saddr(bars + 2 + b), (mph >> b) & 1u)) give_up[grp] = 1;
        mph ^= 1u << b;
        mma_out &= ~(1u << b);
        if (tile + 2 * tstride < ntiles) issue(b, tile + 2 * tstride);  // buffer b is free: tile i's MMAs are done
        gsync();
        if (give_up[grp]) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // epilogue, 16 columns at a time: warp w of the group holds TMEM lanes 32w..32w+31 = MMA
        // rows m = 8 r + c
        const uint32_t acc = tmem + (uint32_t)(b * TMEM_COLS);
        const int m = 32 * gwarp + lane, r = m >> 3, c = m & 7;
        const long long p = ((long long)n * H + y0 + r) * W + x0 + c;
#pragma unroll
        for (int q = 0; q < NOUT / 16; ++q) {
            float v[16];
            tmem_ld16(acc + ((uint32_t)(32 * gwarp) << 16) + (uint32_t)(16 * q), v);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if constexpr (EPI == 3) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int co = 16 * q + 8 * h;
                    const uint4 zz = *reinterpret_cast<const uint4 *>(zprev + p * NOUT + co);
                    const uint32_t zw[4] = {zz.x, zz.y, zz.z, zz.w};
                    uint32_t ga[4];
#pragma unroll
                    for (int i2 = 0; i2 < 4; ++i2) {
                        const __nv_bfloat162 zp = *reinterpret_cast<const __nv_bfloat162 *>(&zw[i2]);
                        const __nv_bfloat162 gg = __floats2bfloat162_rn(v[8 * h + 2 * i2] * gelu_grad_tc(__bfloat162float(zp.x)),
                                                                        v[8 * h + 2 * i2 + 1] * gelu_grad_tc(__bfloat162float(zp.y)));
                        ga[i2] = *reinterpret_cast<const uint32_t *>(&gg);
                    }
                    *reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(out) + p * NOUT + co) = make_uint4(ga[0], ga[1], ga[2], ga[3]);
                }
            } else if constexpr (EPI == 2) {
                float *o = static_cast<float *>(out) + p * COUT;
#pragma unroll
                for (int h = 0; h < COUT / 4; ++h)
                    *reinterpret_cast<float4 *>(o + 4 * h) = make_float4(v[4 * h] + bias_s[4 * h], v[4 * h + 1] + bias_s[4 * h + 1],
                                                                         v[4 * h + 2] + bias_s[4 * h + 2], v[4 * h + 3] + bias_s[4 * h + 3]);
            } else {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int co = 16 * q + 8 * h;
                    uint32_t za[4], ga[4];
#pragma unroll
                    for (int i2 = 0; i2 < 4; ++i2) {
                        const float z0 = v[8 * h + 2 * i2] + bias_s[co + 2 * i2], z1 = v[8 * h + 2 * i2 + 1] + bias_s[co + 2 * i2 + 1];
                        const __nv_bfloat162 zz = __floats2bfloat162_rn(z0, z1), gg = __floats2bfloat162_rn(gelu_tc(z0), gelu_tc(z1));
                        za[i2] = *reinterpret_cast<const uint32_t *>(&zz);
                        ga[i2] = *reinterpret_cast<const uint32_t *>(&gg);
                    }
                    if constexpr (EPI == 0) *reinterpret_cast<uint4 *>(zout + p * NOUT + co) = make_uint4(za[0], za[1], za[2], za[3]);
                    *reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(out) + p * NOUT + co) = make_uint4(ga[0], ga[1], ga[2], ga[3]);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        gsync();  // accumulator b read before the MMAs of tile i+2 go into it
    }
    if (give_up[grp]) {  // the copies and MMAs still in flight, if any (bounded), before the TMEM goes
        if (gtid == 0) atomicOr(status, (unsigned)WMDEV_TIMEOUT);
        for (int b = 0; b < 2; ++b) {
            if (pending & (1u << b)) mbar_wait(saddr(bars + b), (hph >> b) & 1u);
            if (mma_out & (1u << b)) mbar_wait(saddr(bars + 2 + b), (mph >> b) & 1u);
        }
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(*tslot), "r"(TC_GROUPS * 2 * TMEM_COLS) : "memory");
}

template <int CIN, int NOUT, int COUT, int EPI>
int launch_tc(const void *in, const void *wk, const float *bias, int nimg, int H, int W, void *out, void *zout, const void *zprev,
              unsigned *status, cudaStream_t st)
{
    constexpr int KG = CIN / 8;
    CUtensorMap tmap;
    const unsigned long long gdim[4] = {(unsigned long long)CIN, (unsigned long long)W, (unsigned long long)H, (unsigned long long)nimg};
    const unsigned long long gstride[3] = {(unsigned long long)CIN * 2, (unsigned long long)W * CIN * 2, (unsigned long long)H * W * CIN * 2};
    const unsigned box[4] = {8, TC_HW, TC_TH + 2, 1};
    WM_TRY(wm_tensor_map(&tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, in, gdim, gstride, box));
    const size_t smem = 16 * (size_t)(9 * KG * NOUT + TC_GROUPS * 2 * KG * TC_XP) + 8 * 4 * TC_GROUPS + 16;
    WM_CUDA(cudaFuncSetAttribute(k_conv3x3_tc<CIN, NOUT, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long ntiles = (long long)nimg * (H / TC_TH) * (W / TC_TW);
    // resident CTAs per SM: at most 2 (registers; 2 x 2 groups x 2 accumulators x 64 TMEM columns = all 512), within the shared memory
    const int per_sm = std::max(1, std::min(2, (int)(233472 / (smem + 2048))));  // 228 KB per SM, 2 KB per CTA for the static part and the system
    const int grid = (int)std::min<long long>((ntiles + TC_GROUPS - 1) / TC_GROUPS, 152LL * per_sm);
    k_conv3x3_tc<CIN, NOUT, COUT, EPI><<<grid, 128 * TC_GROUPS, smem, st>>>(tmap, static_cast<const __nv_bfloat16 *>(in),
                                                                            static_cast<const __nv_bfloat16 *>(wk), bias, nimg, H, W, out,
                                                                            static_cast<__nv_bfloat16 *>(zout),
                                                                            static_cast<const __nv_bfloat16 *>(zprev), status);
    return wm_check_launch("k_conv3x3_tc");
}

// Weight gradient of training on tcgen05: dW(tap, co, ci) = sum_p dz(p, co) x(p + d_tap, ci) and
// db(co) = sum_p dz(p, co), p over every pixel of every image.  A GEMM per tap with K = pixels:
// D[co][ci] += A[co][k] B[ci][k] with A = dz^T and B = the shifted input x^T, both taken from
// shared memory in the MN-major layout (8 channels of one pixel form a 16-byte core-matrix row,
// 8 pixels = one tile row form the 8 K rows of a core matrix), so the NHWC data is staged as it
// lies, without a transpose:
//   dz of the tile's 128 pixels as [channel group][pixel][8]: the M (co) direction steps one
//     channel group (2048 bytes), the K direction one tile row (128 bytes);
//   the input halo as [halo row][channel group][halo column][8]: the N direction (ci) steps one
//     channel group (160 bytes), and since a halo row holds every channel group, the next tap
//     row (dy + 1) is the next N block at the same stride, so one MMA covers the three taps of a
//     column dx (N = 3 cin); the K direction steps one halo row.
// The shift of tap (dy, dx) is a start address moved by whole 16-byte rows.  M = 128 rows of
// co: rows past coutp read whatever the shared memory holds beyond the staged channels, and their
// accumulator lanes are never read (every D row depends on its own A row only).  Three FP32
// accumulators in tensor memory (dx = -1, 0, 1; 3 cin columns each) sum the CTA's tiles; the
// next two tiles are copied in (cp.async, three buffers) while the current tile's 24 MMAs (8 K
// steps of 16 pixels x 3 dx) run.  Per-CTA partials [cta][9][coutp][cin] + [coutp] as k_conv3x3_wgrad writes
// them; k_reduce_wgrad sums them in CTA order.  Waits are bounded (WMDEV_TIMEOUT, TMEM freed).
constexpr uint32_t WG_MARGIN = 32768;  // shared memory past the buffers: the M = 128 rows of the A operand stay inside it
constexpr int WG_NB = 3;               // staging buffers: a tile in use, two being copied in
template <int CIN, int COUTP, bool GROUPED>
__global__ void __launch_bounds__(128, 1) k_conv3x3_wgrad_tc(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ dz, int nimg,
                                                             int H, int W, float *__restrict__ part, unsigned *status)
{
    constexpr int KG = CIN / 8, DG = COUTP / 8;
    constexpr int N3 = 3 * CIN;                         // one accumulator: taps dy = -1, 0, 1 x cin, for one dx
    constexpr uint32_t TCOLS = 9 * CIN > 256 ? 512 : 256;  // TMEM columns (a power of 2 >= 9 cin)
    constexpr uint32_t ROW = KG * TC_HW * 16;           // bytes per halo row
    constexpr uint32_t XB = (TC_TH + 2) * ROW;          // one halo buffer
    constexpr uint32_t DB = DG * 2048;                  // one dz buffer: DG groups x 128 pixels x 16 bytes
    // kind::f16: FP32 D, BF16 A and B, both MN-major (bits 15, 16), N = 3 cin, M = 128
    constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((uint32_t)(N3 >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);
    static_assert(N3 % 16 == 0 && N3 <= 256, "N of an M = 128 MMA");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *dz_s = smem_raw;                                   // [WG_NB][DG][128][8] BF16
    unsigned char *x_s = smem_raw + WG_NB * DB;                       // [WG_NB][18][KG][10][8] BF16
    uint64_t *bars = reinterpret_cast<uint64_t *>(x_s + WG_NB * XB);  // MMA completion of each buffer's tile
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + WG_NB);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)), "r"(TCOLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < WG_NB; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bars + b)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;

    const int ntx = W / TC_TW, nty = H / TC_TH;
    const long long ntiles = (long long)nimg * nty * ntx;
    auto cp16 = [](void *dst, const void *src) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr(dst)), "l"(src) : "memory");
    };
    auto commit = []() { asm volatile("cp.async.commit_group;\n" ::: "memory"); };
    auto stage = [&](long long t, int b) {  // tile t into buffer b by asynchronous 16-byte copies
        const int n = (int)(t / ((long long)nty * ntx));
        const int rem = (int)(t % ((long long)nty * ntx));
        const int y0 = (rem / ntx) * TC_TH, x0 = (rem % ntx) * TC_TW;
        unsigned char *xb = x_s + b * XB;
        for (int e = tid; e < TC_HPIX * KG; e += 128) {  // periodic halo, [halo row][group][column][8]
            const int kg = e % KG, pix = e / KG, hy = pix / TC_HW, hx = pix % TC_HW;
            int yy = y0 - 1 + hy, xx = x0 - 1 + hx;
            yy += (yy < 0) ? H : (yy >= H ? -H : 0);
            xx += (xx < 0) ? W : (xx >= W ? -W : 0);
            cp16(xb + hy * ROW + kg * (TC_HW * 16) + hx * 16, x + (((long long)n * H + yy) * W + xx) * CIN + kg * 8);
        }
        unsigned char *db = dz_s + b * DB;
        for (int e = tid; e < 128 * DG; e += 128) {  // the tile's pixels p = 8 r + c, [group][p][8]
            const int g = e % DG, p = e / DG;
            cp16(db + g * 2048 + p * 16, dz + (((long long)n * H + y0 + (p >> 3)) * W + x0 + (p & 7)) * COUTP + g * 8);
        }
    };
    float dbias = 0.f;
    auto bias_sum = [&](int b) {  // db(co) over the tile's pixels: four interleaved partial sums, added in a fixed order
        if (tid < COUTP) {
            const __nv_bfloat16 *d = reinterpret_cast<const __nv_bfloat16 *>(dz_s + b * DB + (tid >> 3) * 2048) + (tid & 7);
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll 8
            for (int p = 0; p < 128; p += 4) {
                s0 += __bfloat162float(d[p * 8]);
                s1 += __bfloat162float(d[(p + 1) * 8]);
                s2 += __bfloat162float(d[(p + 2) * 8]);
                s3 += __bfloat162float(d[(p + 3) * 8]);
            }
            dbias += (s0 + s1) + (s2 + s3);
        }
    };

    // Tile it of the CTA lives in buffer it % WG_NB; tiles it+1 and it+2 are being copied in
    // meanwhile.  The MMAs of tile it commit to barrier it % WG_NB; buffer (it+2) % WG_NB is
    // refilled once the MMAs of tile it-1, its last reader, are done.
    uint32_t ph = 0u;  // bit b: phase of MMA barrier b
    long long tile = blockIdx.x;
    int it = 0;
    int ncommit = 0;                  // tiles whose MMAs were issued (one commit each)
    bool fail = false, stop = false;  // this thread's wait gave up; some thread's did (block-uniform)
    for (int k = 0; k < 2; ++k) {
        const long long t = tile + (long long)k * gridDim.x;
        if (t < ntiles) stage(t, k);
        commit();
    }
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const int b = it % WG_NB;
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");          // this tile's copies are in
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // and visible to the tensor core
        __syncthreads();
        bias_sum(b);
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t da = saddr(dz_s + b * DB), xa = saddr(x_s + b * XB);
#pragma unroll
            for (int s = 0; s < TC_TH / 2; ++s) {  // K step s: tile rows 2s, 2s+1 (16 pixels)
                const uint64_t ad = smem_desc(da + (uint32_t)(s * 256), 128, 2048);
#pragma unroll
                for (int dxi = 0; dxi < 3; ++dxi) {
                    const uint64_t bd = smem_desc(xa + (uint32_t)(2 * s * ROW + dxi * 16), ROW, TC_HW * 16);
                    mma_f16(tmem + (uint32_t)(dxi * N3), ad, bd, IDESC, (it | s) != 0 ? 1u : 0u);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bars + b)) : "memory");
        }
        ncommit = it + 1;
        if (it >= 1) {  // tile it-1's MMAs: the last readers of the buffer refilled next
            const int pb = (it - 1) % WG_NB;
            fail = !mbar_wait(saddr(bars + pb), (ph >> pb) & 1u);
            ph ^= 1u << pb;
        }
        const long long t2 = tile + 2LL * gridDim.x;
        if (!fail && t2 < ntiles) stage(t2, (it + 2) % WG_NB);
        commit();  // (empty groups keep the count that the wait above relies on)
        stop = __syncthreads_or(fail) != 0;
        if (stop) break;
    }
    const int last = (ncommit - 1) % WG_NB;  // the last commit covers every MMA issued before it
    if (!stop && ncommit > 0) stop = __syncthreads_or(!mbar_wait(saddr(bars + last), (ph >> last) & 1u)) != 0;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (stop) {  // the MMAs still in flight (bounded) before the TMEM goes; the partials are not written
        if (tid == 0) atomicOr(status, (unsigned)WMDEV_TIMEOUT);
        if (ncommit > 0) mbar_wait(saddr(bars + last), (ph >> last) & 1u);
    }
    const bool ok = !stop;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    float *pw = part + (long long)blockIdx.x * (9 * COUTP * CIN + COUTP);
    if (ok && warp * 32 < COUTP) {  // warp w reads TMEM lanes (co) 32w .. 32w+31
        const int co = warp * 32 + lane;
#pragma unroll 1
        for (int q = 0; q < 9 * CIN / 16; ++q) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(16 * q), v);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const int col = 16 * q, dxi = col / N3, dyi = (col % N3) / CIN, ci0 = col % CIN;
            const int tap = dyi * 3 + dxi;
            if (co < COUTP) {
                float *o = pw + ((long long)tap * COUTP + co) * CIN + ci0;
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    float4 w4 = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                    if (GROUPED && (co >> 4) != ((ci0 + i) >> 4)) w4 = make_float4(0.f, 0.f, 0.f, 0.f);  // off-block: zero
                    *reinterpret_cast<float4 *>(o + i) = w4;
                }
            }
        }
    }
    if (tid < COUTP) pw[9 * COUTP * CIN + tid] = dbias;
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS) : "memory");
}

template <int CIN, int COUTP, bool GROUPED>
int launch_wgrad_tc(const void *x, const void *dz, int nimg, int H, int W, float *part, long long part_floats, int *nparts, unsigned *status,
                    cudaStream_t st)
{
    constexpr uint32_t DB = (COUTP / 8) * 2048, XB = (TC_TH + 2) * (CIN / 8) * TC_HW * 16;
    const size_t smem = WG_NB * ((size_t)DB + XB) + 64 + WG_MARGIN;
    WM_CUDA(cudaFuncSetAttribute(k_conv3x3_wgrad_tc<CIN, COUTP, GROUPED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        WM_CUDA(cudaGetDevice(&dev));
        WM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    const long long ntiles = (long long)nimg * (H / TC_TH) * (W / TC_TW);
    const long long per = 9LL * COUTP * CIN + COUTP;
    const int grid = (int)std::min<long long>(std::min<long long>(ntiles, nsm), part_floats / per);
    if (grid < 1) return WM_ERR_BAD_ARG;
    k_conv3x3_wgrad_tc<CIN, COUTP, GROUPED><<<grid, 128, smem, st>>>(static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(dz),
                                                                     nimg, H, W, part, status);
    *nparts = grid;
    return wm_check_launch("k_conv3x3_wgrad_tc");
}

}  // namespace

int wm_cnn_wgrad_tc(const void *x, const void *dz, int cin, int coutp, bool grouped, int nimg, int h, int wd, float *part, long long part_floats,
                    int *nparts, unsigned *status, cudaStream_t st)
{
    if (!wm_cnn_tc_shape_ok(nimg, h, wd) || !status || !nparts) return WM_ERR_BAD_ARG;
    if (grouped && cin == 48 && coutp == 48) return launch_wgrad_tc<48, 48, true>(x, dz, nimg, h, wd, part, part_floats, nparts, status, st);
    if (cin == 16 && coutp == 48) return launch_wgrad_tc<16, 48, false>(x, dz, nimg, h, wd, part, part_floats, nparts, status, st);
    if (cin == 48 && coutp == 48) return launch_wgrad_tc<48, 48, false>(x, dz, nimg, h, wd, part, part_floats, nparts, status, st);
    if (cin == 48 && coutp == 16) return launch_wgrad_tc<48, 16, false>(x, dz, nimg, h, wd, part, part_floats, nparts, status, st);
    return WM_ERR_UNSUPPORTED;
}

int wm_tensor_map(CUtensorMap *map, CUtensorMapDataType type, int rank, const void *base, const unsigned long long *dims,
                  const unsigned long long *strides, const unsigned *box)
{
    static PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    if (!enc) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return WM_ERR_CUDA;
        enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], es[5];
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (i + 1 < rank) st[i] = strides[i];
    }
    return enc(map, type, (cuuint32_t)rank, const_cast<void *>(base), d, st, b, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
               ? WM_OK
               : WM_ERR_BAD_ARG;
}

bool wm_cnn_tc_shape_ok(int nimg, int H, int W) { return nimg > 0 && H >= TC_TH && W >= TC_TW && H % TC_TH == 0 && W % TC_TW == 0; }

int wm_cnn_conv3x3_tc(const void *in, const void *w, const float *bias, int cin, int cout, int mode, int nimg, int h, int wd, void *out,
                      void *zout, const void *zprev, unsigned *status, cudaStream_t st)
{
    if (!wm_cnn_tc_shape_ok(nimg, h, wd) || !status || (mode == 0 && !zout) || (mode == 3 && !zprev) || (mode != 3 && !bias))
        return WM_ERR_BAD_ARG;
    if (cout == 48 && (cin == 16 || cin == 48)) {
        if (mode == 0) return cin == 16 ? launch_tc<16, 48, 48, 0>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st)
                                        : launch_tc<48, 48, 48, 0>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st);
        if (mode == 1) return cin == 16 ? launch_tc<16, 48, 48, 1>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st)
                                        : launch_tc<48, 48, 48, 1>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st);
        if (mode == 3) return cin == 16 ? launch_tc<16, 48, 48, 3>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st)
                                        : launch_tc<48, 48, 48, 3>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st);
    }
    if (cout == 8 && cin == 48 && mode == 2) return launch_tc<48, 16, 8, 2>(in, w, bias, nimg, h, wd, out, zout, zprev, status, st);
    return WM_ERR_BAD_ARG;
}
