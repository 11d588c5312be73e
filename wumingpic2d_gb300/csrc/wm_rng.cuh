// wm_rng.cuh -- counter-based random numbers for the initial conditions and the injection.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11): ten rounds of two 32x32->64 multiplications with the key bumped by the Weyl constants
// between rounds.  A draw is a pure function of (counter, key), so every particle's numbers are
// independent of the launch shape and the same on the host and the device.
//
// Counter layout used here: (index low, index high, call, tag): index = the particle's place in
// its species' rows, call = which draw of that particle, tag = which generator.  Key = the seed.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define WM_HD __host__ __device__ __forceinline__
#else
#define WM_HD inline
#endif

struct WmPhilox {
    uint32_t v[4];
};

WM_HD WmPhilox wm_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    WmPhilox o;
    o.v[0] = c0;
    o.v[1] = c1;
    o.v[2] = c2;
    o.v[3] = c3;
    return o;
}

// [0, 1) with 53 random bits: (a >> 5) * 2^26 + (b >> 6), times 2^-53 (exact in FP64).
WM_HD double wm_uniform53(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

enum { WM_RNG_WEIBEL = 1, WM_RNG_HARRIS = 2, WM_RNG_SHOCK = 3, WM_RNG_INJECT = 4, WM_RNG_INJECT_COUNT = 5, WM_RNG_EXPAND = 6 };

// Draw `call` of particle `idx`: two uniforms in [0, 1).
WM_HD void wm_rng_uniform2(uint64_t seed, long long idx, uint32_t call, uint32_t tag, double &u1, double &u2)
{
    const WmPhilox r = wm_philox4x32_10((uint32_t)idx, (uint32_t)((unsigned long long)idx >> 32), call, tag, (uint32_t)seed,
                                        (uint32_t)(seed >> 32));
    u1 = wm_uniform53(r.v[0], r.v[1]);
    u2 = wm_uniform53(r.v[2], r.v[3]);
}

#if defined(__CUDACC__)
// Two standard normals by the Box-Muller transform of one draw: r = sqrt(-2 ln(1 - u1)),
// (r cos 2 pi u2, r sin 2 pi u2).
__device__ __forceinline__ void wm_rng_normal2(uint64_t seed, long long idx, uint32_t call, uint32_t tag, double &n1, double &n2)
{
    double u1, u2, s, c;
    wm_rng_uniform2(seed, idx, call, tag, u1, u2);
    const double r = sqrt(-2.0 * log(1.0 - u1));
    sincospi(2.0 * u2, &s, &c);
    n1 = r * c;
    n2 = r * s;
}
#endif
