// gpda_device.cuh — device-side random numbers, FP32 elementary functions and
// samplers of the photon-burst Monte-Carlo PDA kernels (sm_103a).
//
// Everything here is deterministic FP32/INT32 arithmetic with a fixed
// operation order. The kernels are compiled with -fmad=false, so no multiply-
// add is contracted unless written as fmaf(); together with IEEE division and
// square root this makes every sampling decision reproducible on the host.
//
// Random numbers: Philox4x32-10 (Salmon et al., SC'11) kept in registers. A
// unit (parameter-set word, burst, sample) owns the counter space
// (block, sample, burst, pword) under key = seed; this replaces the
// reference's per-thread curandStateScrambledSobol64 + rk_state arrays in HBM
// (src/gen_rand.cuh:7-25, src/mc.cu:366-454).
#pragma once
#include <cstdint>

namespace gpda {

constexpr int kMaxStates = 8;
constexpr int kMaxSeg = 65536;      // segments per unit before the trajectory is cut
constexpr int kMaxRestart = 256;    // rejection restarts before the sampler gives up
// 1: Rng::align_now generates its block inline (the photon step's one block
// per segment), every other draw site calls the out-of-line generator; 0:
// all go out of line. Inline measured 0.664 -> 0.659 ms on the photon kernel
// (e2e 0.796 -> 0.781 ms per gpda_run_host call), the same bits either way.
#ifndef GPDA_ALIGN_INLINE
#define GPDA_ALIGN_INLINE 1
#endif

// ---------------------------------------------------------------- Philox
// One Philox4x32-10 block for counter (c0, c1, c2, c3) under key (k0, k1).
__device__ __forceinline__ uint4 philox_block_inline(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3,
                                                     uint32_t a, uint32_t b) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * x0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ x1 ^ a;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ x3 ^ b;
        x1 = (uint32_t)p1;
        x3 = (uint32_t)p0;
        x0 = n0;
        x2 = n2;
        a += 0x9E3779B9u;
        b += 0xBB67AE85u;
    }
    return make_uint4(x0, x1, x2, x3);
}

// The same block behind one out-of-line copy: the draw sites of the samplers
// call it instead of carrying their own inlined rounds, which keeps the
// instruction footprint of the simulation loop small.
static __device__ __noinline__ uint4 philox_block(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3,
                                           uint32_t a, uint32_t b) {
    return philox_block_inline(x0, x1, x2, x3, a, b);
}

struct Rng {
    uint32_t k0, k1, c1, c2, c3, blk;
    uint32_t w0, w1, w2, w3;
    int idx;

    __device__ __forceinline__ void init(uint64_t seed, uint32_t pword, uint32_t b, uint32_t s) {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
        c1 = s; c2 = b; c3 = pword;
        blk = 0u;
        idx = 4;
    }
    __device__ __forceinline__ void take(uint4 v) {
        w0 = v.x; w1 = v.y; w2 = v.z; w3 = v.w;
        blk += 1u;
        idx = 0;
    }
    __device__ __forceinline__ uint32_t next() {
        if (idx == 4) take(philox_block(blk, c1, c2, c3, k0, k1));
        uint32_t r = (idx == 0) ? w0 : (idx == 1) ? w1 : (idx == 2) ? w2 : w3;
        ++idx;
        return r;
    }
    // The next draw starts a fresh block (the rest of the current one is
    // discarded): keeps block generation at the same program point for all
    // lanes of a warp.
    __device__ __forceinline__ void align() { idx = 4; }
    // The next draw starts at counter block `b` (a stream position that does
    // not depend on how many draws came before).
    __device__ __forceinline__ void seek(uint32_t b) { blk = b; idx = 4; }
    // align() + generate that block now, inline; only where at least one
    // draw follows before the next align (same words as align()).
    __device__ __forceinline__ void align_now() {
#if GPDA_ALIGN_INLINE
        take(philox_block_inline(blk, c1, c2, c3, k0, k1));
#else
        idx = 4;
#endif
    }
    // uniform on (0,1]: ((x >> 8) + 1) * 2^-24, exact
    __device__ __forceinline__ float u01() { return u01_of(next()); }
    __device__ __forceinline__ static float u01_of(uint32_t x) {
        return (float)((x >> 8) + 1u) * 5.9604644775390625e-08f;
    }
    // the next block, generated out of line, for a caller that takes its four
    // words itself (the same words as four next() calls from a fresh block)
    __device__ __forceinline__ uint4 block() {
        const uint4 v = philox_block(blk, c1, c2, c3, k0, k1);
        blk += 1u;
        idx = 4;
        return v;
    }
};

// Unsigned division by an invariant divisor (Granlund & Montgomery, "Division
// by invariant integers using multiplication", PLDI 1994, fig. 4.1): for
// 1 <= d < 2^31, l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1 give
// n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0), t = umulhi(m, n),
// for every 32-bit n. The kernels divide by the samples per burst (unit ->
// burst, sample), by a burst's photon count (its bin) and by the bin count.
struct Divisor {
    uint32_t m, l;
};

__device__ __forceinline__ Divisor divisor_of(uint32_t d) {
    const uint32_t l = (d > 1u) ? 32u - (uint32_t)__clz((int)(d - 1u)) : 0u;
    const uint64_t num = (uint64_t)((1ull << l) - d) << 32;
    return Divisor{(uint32_t)(num / d + 1ull), l};
}

__device__ __forceinline__ uint32_t div_by(uint32_t n, uint32_t m, uint32_t l) {
    const uint32_t t = __umulhi(m, n);
    const uint32_t sh1 = l > 0u ? 1u : 0u;
    const uint32_t sh2 = l > 0u ? l - 1u : 0u;
    return (t + ((n - t) >> sh1)) >> sh2;
}

// ---------------------------------------------------------------- FP32 math
// Written from the mathematics: log by 2*atanh((m-1)/(m+1)) series, exp by
// Taylor series after k*ln2 reduction, cos(2*pi*u) by the sine series.
constexpr float kLn2Hi = 0x1.62e430p-1f;
constexpr float kLn2Lo = -0x1.05c610p-29f;
constexpr float kLog2e = 0x1.715476p+0f;
constexpr float kSqrt2 = 0x1.6a09e6p+0f;
constexpr float kInf = __builtin_huge_valf();

__device__ __forceinline__ float logf_(float x) {
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return -kInf;
    if (x == kInf) return x;
    uint32_t bits = __float_as_uint(x);
    int e = 0;
    if ((bits >> 23) == 0u) {
        x = x * 0x1p24f;
        bits = __float_as_uint(x);
        e = -24;
    }
    e += (int)(bits >> 23) - 127;
    float m = __uint_as_float((bits & 0x007FFFFFu) | 0x3F800000u);
    if (m > kSqrt2) { m = m * 0.5f; e += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float poly = fmaf(z, fmaf(z, fmaf(z, 0x1.c71c72p-3f, 0x1.24924ap-2f), 0x1.99999ap-2f), 0x1.555556p-1f);
    float lm = fmaf(s * z, poly, 2.0f * s);
    float ef = (float)e;
    return fmaf(ef, kLn2Hi, fmaf(ef, kLn2Lo, lm));
}

__device__ __forceinline__ float expf_(float x) {
    if (x != x) return x;
    if (x > 88.72284f) return kInf;
    if (x < -103.97208f) return 0.0f;
    float kf = rintf(x * kLog2e);
    float r = fmaf(-kf, kLn2Hi, x);
    r = fmaf(-kf, kLn2Lo, r);
    float p = 0x1.a01a02p-13f;
    p = fmaf(p, r, 0x1.6c16c2p-10f);
    p = fmaf(p, r, 0x1.111112p-7f);
    p = fmaf(p, r, 0x1.555556p-5f);
    p = fmaf(p, r, 0x1.555556p-3f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int k = (int)kf;
    if (k >= -126 && k <= 127) return p * __uint_as_float((uint32_t)(k + 127) << 23);
    int k1 = k / 2, k2 = k - k1;
    return (p * __uint_as_float((uint32_t)(k1 + 127) << 23)) * __uint_as_float((uint32_t)(k2 + 127) << 23);
}

__device__ __forceinline__ float cos2pif_(float u) {
    float w = (u > 0.5f) ? 1.0f - u : u;
    float rr = 0.25f - w;
    float th = rr * 0x1.921fb6p+2f;
    float t2 = th * th;
    float p = 0x1.612462p-33f;
    p = fmaf(p, t2, -0x1.ae6456p-26f);
    p = fmaf(p, t2, 0x1.71de3ap-19f);
    p = fmaf(p, t2, -0x1.a01a02p-13f);
    p = fmaf(p, t2, 0x1.111112p-7f);
    p = fmaf(p, t2, -0x1.555556p-3f);
    p = fmaf(p, t2, 1.0f);
    return th * p;
}

// logf_ for finite normal x > 0 (the uniforms of u01() are in [2^-24, 1]):
// the same operations without the special cases, so the same bits.
__device__ __forceinline__ float logf_pos(float x) {
    uint32_t bits = __float_as_uint(x);
    int e = (int)(bits >> 23) - 127;
    float m = __uint_as_float((bits & 0x007FFFFFu) | 0x3F800000u);
    if (m > kSqrt2) { m = m * 0.5f; e += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float poly = fmaf(z, fmaf(z, fmaf(z, 0x1.c71c72p-3f, 0x1.24924ap-2f), 0x1.99999ap-2f), 0x1.555556p-1f);
    float lm = fmaf(s * z, poly, 2.0f * s);
    float ef = (float)e;
    return fmaf(ef, kLn2Hi, fmaf(ef, kLn2Lo, lm));
}

// expf_ for -87 <= x <= 0 (so 2^k with -126 <= k <= 0 is a normal float):
// the same operations without the range checks, so the same bits.
__device__ __forceinline__ float expf_neg(float x) {
    float kf = rintf(x * kLog2e);
    float r = fmaf(-kf, kLn2Hi, x);
    r = fmaf(-kf, kLn2Lo, r);
    float p = 0x1.a01a02p-13f;
    p = fmaf(p, r, 0x1.6c16c2p-10f);
    p = fmaf(p, r, 0x1.111112p-7f);
    p = fmaf(p, r, 0x1.555556p-5f);
    p = fmaf(p, r, 0x1.555556p-3f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return p * __uint_as_float((uint32_t)((int)kf + 127) << 23);
}

// Stirling correction fc(k) = ln k! - ((k+1/2) ln(k+1) - (k+1) + ln(2 pi)/2), k < 10
__device__ __forceinline__ float fc_tab(int k) {
    switch (k) {
    case 0: return 8.106146680e-02f; case 1: return 4.134069596e-02f;
    case 2: return 2.767792568e-02f; case 3: return 2.079067210e-02f;
    case 4: return 1.664469119e-02f; case 5: return 1.387612882e-02f;
    case 6: return 1.189670995e-02f; case 7: return 1.041126526e-02f;
    case 8: return 9.255462183e-03f; default: return 8.330563433e-03f;
    }
}
__device__ __forceinline__ float lf_tab(int k) {
    switch (k) {
    case 0: return 0.0f; case 1: return 0.0f; case 2: return 0.693147182f;
    case 3: return 1.791759491f; case 4: return 3.178053856f; case 5: return 4.787491798f;
    case 6: return 6.579251289f; case 7: return 8.525161743f; case 8: return 10.60460281f;
    default: return 12.80182743f;
    }
}
__device__ __forceinline__ float fc(float k) {
    if (k < 10.0f) return fc_tab((int)k);
    float kp = k + 1.0f;
    float k2 = kp * kp;
    return (0.083333333333333333f - (0.0027777777777777778f - 0.00079365079365079365f / k2) / k2) / kp;
}

// ---------------------------------------------------------------- samplers
// The sequential-search loops multiply by a table of reciprocals
// inv[k] = 1.0f / k (k < 64, filled per CTA in shared memory) instead of
// dividing: the search bounds keep k <= 51.
constexpr int kInvTable = 64;

// Binomial by sequential-search inversion (Kachitvichyanukul & Schmeiser
// 1988); p <= 1/2, n p < 10; logq = log(1-p) and rr = p/(1-p) as computed here.
__device__ __forceinline__ int binv_pre(Rng &r, int n, float p, float logq, float rr, int &lim,
                                        const float *inv) {
    float q = 1.0f - p;
    float nf = (float)n;
    float qn = expf_(nf * logq);
    float g = rr * (nf + 1.0f);
    float np = nf * p;
    // bound = min(n, np + 10 sqrt(np q + 1)) >= min(n, 10): evaluated only
    // once the search passes min(n, 10)
    const int x10 = n < 10 ? n : 10;
    int bound = -1;
    for (int it = 0; it < kMaxRestart; ++it) {
        int x = 0;
        float f = qn;
        float u = r.u01();
        bool over = false;
        while (u > f) {
            u = u - f;
            x += 1;
            if (x > x10) {
                if (bound < 0) {
                    float bf = np + 10.0f * sqrtf(np * q + 1.0f);
                    bound = (bf < nf) ? (int)bf : n;
                }
                if (x > bound) { over = true; break; }
            }
            f = f * (g * inv[x] - rr);
        }
        if (!over) return x;
    }
    lim += 1;
    return (int)np;
}

__device__ __forceinline__ int binv(Rng &r, int n, float p, int &lim, const float *inv) {
    float q = 1.0f - p;
    return binv_pre(r, n, p, logf_(q), p / q, lim, inv);
}

// Binomial by transformed rejection with decomposition (Hoermann 1993,
// BTRD); p <= 1/2, n p >= 10. LAZY: the constants of the rejection steps are
// set on the first draw that needs them, else on every such draw (the same
// values either way). Measured: lazy is 2.9 % faster on the occupancy kernel,
// whose split is mostly BTRD; the photon step, where BTRD is a rare fallback,
// keeps the eager form (the lazy one's state costs it a spilled register).
template <bool LAZY>
__device__ __forceinline__ int btrd(Rng &r, int n, float p, int &lim) {
    float nf = (float)n;
    float q = 1.0f - p;
    float npq = nf * p * q;
    float snpq = sqrtf(npq);
    float b = 1.15f + 2.53f * snpq;
    float a = -0.0873f + 0.0248f * b + 0.01f * p;
    float c = nf * p + 0.5f;
    float vr = 0.92f - 4.2f / b;
    float urvr = 0.86f * vr;
    // constants of the rejection steps only (two of them divisions): set on
    // the first draw that fails the quick acceptance, by the same operations
    float rr = 0.0f, nr = 0.0f, m = 0.0f, alpha = 0.0f;
    bool slow = false;
    for (int it = 0; it < kMaxRestart; ++it) {
        float v = r.u01();
        float u;
        if (v <= urvr) {
            u = v / vr - 0.43f;
            float kf = floorf((2.0f * a / (0.5f - fabsf(u)) + b) * u + c);
            if (kf >= 0.0f && kf <= nf) return (int)kf;
            continue;
        }
        if (!LAZY || !slow) {
            rr = p / q;
            nr = (nf + 1.0f) * rr;
            m = floorf((nf + 1.0f) * p);
            alpha = (2.83f + 5.1f / b) * snpq;
            slow = true;
        }
        if (v >= vr) {
            u = r.u01() - 0.5f;
        } else {
            u = v / vr - 0.93f;
            u = copysignf(0.5f, u) - u;
            v = r.u01() * vr;
        }
        float us = 0.5f - fabsf(u);
        if (!(us > 0.0f)) continue;
        float kf = floorf((2.0f * a / us + b) * u + c);
        if (!(kf >= 0.0f && kf <= nf)) continue;
        v = v * alpha / (a / (us * us) + b);
        float km = fabsf(kf - m);
        if (km <= 15.0f) {
            // step 3.1: v <= prod (nr/i - rr) over i in (m, k], or v prod
            // over (k, m] <= 1, with each factor written (nr - rr i) / i and
            // numerator and denominator scaled by 1/m (both products stay
            // near 1): two products and one comparison, no division per
            // factor
            int k = (int)kf, mi = (int)m;
            int lo = mi < k ? mi : k, hi = mi < k ? k : mi;
            float im = 1.0f / m;
            float num = 1.0f, den = 1.0f;
            for (int i = lo + 1; i <= hi; ++i) {
                float fi = (float)i;
                num = num * ((nr - rr * fi) * im);
                den = den * (fi * im);
            }
            if ((mi < k) ? (v * den <= num) : (v * num <= den)) return k;
            continue;
        }
        v = logf_(v);
        float rho = (km / npq) * (((km / 3.0f + 0.625f) * km + 0.16666666666666667f) / npq + 0.5f);
        float t = -km * km / (2.0f * npq);
        if (v < t - rho) return (int)kf;
        if (v > t + rho) continue;
        float nm = nf - m + 1.0f;
        float h = (m + 0.5f) * logf_((m + 1.0f) / (rr * nm)) + fc(m) + fc(nf - m);
        float nk = nf - kf + 1.0f;
        float bound = h + (nf + 1.0f) * logf_(nm / nk) + (kf + 0.5f) * logf_(nk * rr / (kf + 1.0f))
                      - fc(kf) - fc(nf - kf);
        if (v <= bound) return (int)kf;
    }
    lim += 1;
    return (int)floorf((nf + 1.0f) * p);
}

template <bool LAZY = true>
__device__ __forceinline__ int binom(Rng &r, int n, float p, int &lim, const float *inv) {
    if (n <= 0 || !(p > 0.0f)) return 0;
    if (p >= 1.0f) return n;
    bool flip = p > 0.5f;
    float pp = flip ? 1.0f - p : p;
    int x = ((float)n * pp < 10.0f) ? binv(r, n, pp, lim, inv) : btrd<LAZY>(r, n, pp, lim);
    return flip ? n - x : x;
}

// Same draw as binom(r, n, p) with the p-only constants precomputed on the
// host per state (pp = min(p,1-p), logq = logf_(1-pp), rr = pp/(1-pp)).
__device__ __forceinline__ int binom_pre(Rng &r, int n, float p, float pp, float logq, float rr,
                                         int &lim, const float *inv) {
    if (n <= 0 || !(p > 0.0f)) return 0;
    if (p >= 1.0f) return n;
    bool flip = p > 0.5f;
    int x = ((float)n * pp < 10.0f) ? binv_pre(r, n, pp, logq, rr, lim, inv) : btrd<false>(r, n, pp, lim);
    return flip ? n - x : x;
}

#ifndef GPDA_PINV_UNROLL
#define GPDA_PINV_UNROLL 10
#endif
static_assert(GPDA_PINV_UNROLL >= 1 && GPDA_PINV_UNROLL <= 10, "the inversion's unrolled head");

// Poisson by sequential-search inversion, lam < 10. RES: also the residual
// of the accepted uniform inside the drawn count's interval,
// res = (u - F(k-1)) / P(k), uniform on (0, 1] given k.
template <bool RES>
__device__ __forceinline__ int pinv_t(Rng &r, float lam, int &lim, const float *inv, float &res) {
    float L = expf_neg(-lam);        // 0 < lam < 10
    // bound = lam + 10 sqrt(lam) + 10 >= 10: evaluated only once k passes 10
    int bound = -1;
    for (int it = 0; it < kMaxRestart; ++it) {
        int k = 0;
        float f = L;
        float u = r.u01();
        // k = 1..GPDA_PINV_UNROLL (<= 10) unrolled with immediate
        // reciprocals (the same values as inv[k]); the bound is >= 10, so it
        // cannot stop the search before k = 11
        bool more = u > f;
#pragma unroll
        for (int j = 1; j <= GPDA_PINV_UNROLL; ++j) {
            if (more) {
                u = u - f;
                k = j;
                f = (f * lam) * (1.0f / (float)j);
                more = u > f;
            }
        }
        bool over = false;
        if (more) {
            while (u > f) {
                u = u - f;
                k += 1;
                if (bound < 0) bound = (int)(lam + 10.0f * sqrtf(lam) + 10.0f);
                if (k > bound) { over = true; break; }
                f = (f * lam) * inv[k];
            }
        }
        if (!over) {
            if (RES) res = u / f;
            return k;
        }
    }
    lim += 1;
    if (RES) res = 0.5f;
    return (int)lam;
}

__device__ __forceinline__ int pinv(Rng &r, float lam, int &lim, const float *inv) {
    float unused;
    return pinv_t<false>(r, lam, lim, inv, unused);
}

__device__ __forceinline__ float logfact(float k) {
    if (k < 10.0f) return lf_tab((int)k);
    return (k + 0.5f) * logf_(k + 1.0f) - (k + 1.0f) + 0.91893853320467274f + fc(k);
}

// Poisson by transformed rejection with squeeze (Hoermann 1993, PTRS), lam >= 10.
__device__ __forceinline__ int ptrs(Rng &r, float lam, int &lim) {
    float slam = sqrtf(lam);
    float loglam = logf_(lam);
    float b = 0.931f + 2.53f * slam;
    float a = -0.059f + 0.02483f * b;
    float invalpha = 1.1239f + 1.1328f / (b - 3.4f);
    float vr = 0.9277f - 3.6224f / (b - 2.0f);
    float lia = logf_(invalpha);
    for (int it = 0; it < kMaxRestart; ++it) {
        float U = r.u01() - 0.5f;
        float V = r.u01();
        float us = 0.5f - fabsf(U);
        if (!(us > 0.0f)) continue;
        float kf = floorf((2.0f * a / us + b) * U + lam + 0.43f);
        if (us >= 0.07f && V <= vr) {
            if (kf >= 0.0f && kf < 2.0e9f) return (int)kf;
            continue;
        }
        if (!(kf >= 0.0f && kf < 2.0e9f)) continue;
        if (us < 0.013f && V > us) continue;
        float lhs = logf_(V) + lia - logf_(a / (us * us) + b);
        float rhs = -lam + kf * loglam - logfact(kf);
        if (lhs <= rhs) return (int)kf;
    }
    lim += 1;
    return (int)lam;
}

__device__ __forceinline__ int poisson(Rng &r, float lam, int &lim, const float *inv) {
    if (!(lam > 0.0f)) return 0;
    return (lam < 10.0f) ? pinv(r, lam, lim, inv) : ptrs(r, lam, lim);
}

__device__ __forceinline__ float normal(Rng &r) {
    float u1 = r.u01();
    float u2 = r.u01();
    return sqrtf(-2.0f * logf_(u1)) * cos2pif_(u2);
}

__device__ __forceinline__ float root6(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? 0.0f : __int_as_float(0x7fc00000);
    return expf_(logf_(x) * 0.16666666666666667f);
}

// drawE (src/gen_rand.cuh:63-68): distance-broadened efficiency
__device__ __forceinline__ float broaden(Rng &r, float e, float r0, float v) {
    float z = normal(r);
    float rd = z * v + r0 * root6(1.0f / e - 1.0f);
    float t = rd / r0;
    float t2 = t * t;
    float t6 = (t2 * t2) * t2;
    return 1.0f / (1.0f + t6);
}

__device__ __forceinline__ float eps_of(float e, float g, float ct) {
    float om = 1.0f - e;
    float num = g * e + ct * om;
    return num / (num + om);
}

// ---------------------------------------------------------------- model draws
// Categorical draw over a cumulative table; jump to a state other than `from`.
__device__ __forceinline__ int cat_draw(const float *cdf, int n, float u) {
    for (int i = 0; i < n; ++i)
        if (u <= cdf[i]) return i;
    return n - 1;
}

__device__ __forceinline__ int jump_draw(const float *row, int n, int from, float u) {
    int last = from;
    for (int i = 0; i < n; ++i) {
        if (i == from) continue;
        last = i;
        if (u <= row[i]) return i;
    }
    return last;
}

// Background of one window (Poisson, clipped as draw_P_B_Tr does,
// src/gen_rand.cuh:92-107), acceptor channel first; returns the acceptor
// background, writes the remaining signal photons to *sig.
__device__ __forceinline__ int background(Rng &r, int navail, float lam_a, float lam_d, int *sig,
                                          int &lim, const float *inv) {
    int B[2];
    int avail = navail;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        int x = poisson(r, c == 0 ? lam_a : lam_d, lim, inv);
        if (x > avail) x = (int)floorf((float)avail * r.u01());
        B[c] = x;
        avail -= x;
    }
    *sig = avail;
    return B[0];
}

// background() through out-of-line Poisson samplers (the same draws): the
// occupancy split, which runs once per unit, measured 3-5 % faster with it;
// the photon step keeps them inline (out of line costs it 40 %).
static __device__ __noinline__ int pinv_ool(Rng &r, float lam, int &lim, const float *inv) {
    return pinv(r, lam, lim, inv);
}
static __device__ __noinline__ int ptrs_ool(Rng &r, float lam, int &lim) { return ptrs(r, lam, lim); }

__device__ __forceinline__ int background_occ(Rng &r, int navail, float lam_a, float lam_d, int *sig,
                                              int &lim, const float *inv) {
    int B[2];
    int avail = navail;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const float lam = c == 0 ? lam_a : lam_d;
        int x = !(lam > 0.0f) ? 0 : (lam < 10.0f) ? pinv_ool(r, lam, lim, inv) : ptrs_ool(r, lam, lim);
        if (x > avail) x = (int)floorf((float)avail * r.u01());
        B[c] = x;
        avail -= x;
    }
    *sig = avail;
    return B[0];
}

// Background of one photon-mode segment as a pair: T = A + D ~ Poisson(lam),
// lam = (bg_a + bg_d) dt, split by A ~ Binomial(T, pa), pa = bg_a / (bg_a +
// bg_d), which has the law of independent Poisson(bg_a dt) and
// Poisson(bg_d dt). For lam < 10, T comes from one uniform by inversion and
// the split from T Bernoulli trials on that uniform's residual (uniform on
// (0, 1] given T), rescaled after each trial: one random word in all for the
// pair. bgc = {bg_a + bg_d, pa, 1 / pa, 1 / (1 - pa)}. Clipping to the
// segment's photons as background().
__device__ __forceinline__ int background_pair(Rng &r, int navail, float dt, const float *bgc, int *sig,
                                               int &lim, const float *inv) {
    const float lam = bgc[0] * dt;
    int T = 0, A = 0;
    if (lam > 0.0f) {
        if (lam < 10.0f) {
            const float pa = bgc[1], ipa = bgc[2], iqa = bgc[3];
            float res;
            T = pinv_t<true>(r, lam, lim, inv, res);
            for (int i = 0; i < T; ++i) {
                if (res <= pa) { A += 1; res = res * ipa; }
                else res = (res - pa) * iqa;
            }
        } else {
            T = ptrs(r, lam, lim);
            A = binom<false>(r, T, bgc[1], lim, inv);
        }
    }
    int D = T - A;
    int avail = navail;
    if (A > avail) A = (int)floorf((float)avail * r.u01());
    avail -= A;
    if (D > avail) D = (int)floorf((float)avail * r.u01());
    avail -= D;
    *sig = avail;
    return A;
}

}  // namespace gpda
