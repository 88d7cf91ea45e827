// gpda_expected.cu — differentiable expected-histogram PDA (occupancy model)
// and its adjoint, sm_103a.
//
// Per unit (parameter set p, burst b, dwell sample s) the state skeleton is
// the sampled occupancy model's, drawn from the same Philox counters
// (seed, pword = p, b, s) in the same order (traj_occ in gpda_kernels.cu); it
// comes from the anchor theta0 and carries the likelihood-ratio weight W (see
// ExpParams). The background counts are drawn as in the occupancy split but from counter
// block 2^31 on, so that they do not depend on the trajectory's length. With
//   E_eff = sum_k dt_k E[s_k] / T,  dt_k = -ln(u_k) / k_exit(s_k; theta)
//   p     = eps(E_eff) = (g E + ct (1-E)) / (g E + (1+ct)(1-E))
// the unit adds W * P(X = x), X ~ Binomial(sig, p), to the bin of the
// proximity ratio (ba + x) / N for every x; sig and ba are the signal photons
// and acceptor background left by the background draw.
//
// Binomial masses: the mode's probability by Loader's saddle-point form
// (C. Loader, "Fast and accurate computation of binomial probabilities",
// 2000), then the ratio recurrence P(x+1)/P(x) = (sig-x) p / ((x+1) q) in both
// directions until a mass drops below 2^-24 of the mode's (the neglected tail
// is below FP32 resolution of the unit's total).
//
// Kernels (one parameter set per blockIdx.y, units strided over blockIdx.x):
//   exp_fwd_kernel   per-thread FP32 bin rows in shared memory, reduced in a
//                    fixed order into per-block FP64 partials
//   exp_chi2_kernel  partials -> expected counts, reduced chi-square (FP64,
//                    sequential over bins as chi2_kernel) and d chi2 / d count
//   exp_adj_kernel   re-walks each unit's trajectory: G = sum g_bin P(bin),
//                    H = d G / d p from the mass tape the forward wrote (or by
//                    walking the binomial again without one), and the pathwise
//                    (dwells, E) plus score (skeleton) terms
//   exp_grad_kernel  per-block partials -> gradient, times the upstream d chi2
// All sums have a fixed order, so results do not depend on scheduling.
#include <algorithm>

#include "gpda_device.cuh"
#include "gpda_internal.h"

namespace gpda {

namespace {

constexpr int kExpThreads = 256;
// 1: the adjoint keeps its per-unit statistics and gradient sums in the
// thread's shared-memory columns (see exp_walk); 0: in registers
#ifndef GPDA_ADJ_SMEM
#define GPDA_ADJ_SMEM 1
#endif
// 1: the unit's background draws through the out-of-line Poisson samplers
// (background_occ: the same draws, a smaller kernel body; the 4-state adjoint
// then needs 48 registers instead of 62). fit_4state gradient step 9.48 ->
// 9.40 ms; Loader's pmf out of line as well measured 9.52 ms.
#ifndef GPDA_EXP_BG_OOL
#define GPDA_EXP_BG_OOL 1
#endif
// the trajectory's segments in pairs from one Philox block (see exp_walk):
// 0 off, 1 with the out-of-line block generator, 2 with it inline
#ifndef GPDA_EXP_PAIRS
#define GPDA_EXP_PAIRS 2
#endif
constexpr float kMassCut = 0x1p-24f;
constexpr uint32_t kExpBgBlock = 0x80000000u;   // above any trajectory block (< 2^15)

// ln(1 - x) for 0 <= x < 1 without forming 1 - x when x is small
__device__ __forceinline__ float log1m_(float x) {
    if (x < 0.01f) {
        float x2 = x * x;
        return -(x + x2 * (0.5f + x * (0.333333343f + x * (0.25f + x * 0.2f))));
    }
    return logf_(1.0f - x);
}

// 1/(2j+1), j = 1..15, for the bd0 series
__device__ __forceinline__ float inv_odd(int j) {
    switch (j) {
    case 1: return 0x1.555556p-2f;  case 2: return 0x1.99999ap-3f;  case 3: return 0x1.24924ap-3f;
    case 4: return 0x1.c71c72p-4f;  case 5: return 0x1.745d18p-4f;  case 6: return 0x1.3b13b2p-4f;
    case 7: return 0x1.111112p-4f;  case 8: return 0x1.e1e1e2p-5f;  case 9: return 0x1.af286cp-5f;
    case 10: return 0x1.861862p-5f; case 11: return 0x1.642c86p-5f; case 12: return 0x1.47ae14p-5f;
    case 13: return 0x1.2f684cp-5f; case 14: return 0x1.1a7b96p-5f; default: return 0x1.084210p-5f;
    }
}

// Loader's deviance term bd0(x, np) = x ln(x / np) + np - x, by its series
// sum_j 2 x v^(2j+1) / (2j+1), v = (x - np)/(x + np), when x is close to np.
__device__ __forceinline__ float bd0(float x, float np) {
    float d = x - np;
    if (fabsf(d) < 0.1f * (x + np)) {
        float v = d / (x + np);
        float s = d * v;
        float ej = 2.0f * x * v;
        float v2 = v * v;
        for (int j = 1; j < 16; ++j) {
            ej = ej * v2;
            float s1 = fmaf(ej, inv_odd(j), s);
            if (s1 == s) return s1;
            s = s1;
        }
        return s;
    }
    return x * logf_(x / np) + np - x;
}

// stirlerr(k) = ln k! - (k + 1/2) ln k + k - ln(2 pi)/2, k >= 1: exact values
// for k <= 15, the asymptotic series 1/12k - 1/360k^3 + 1/1260k^5 - 1/1680k^7
// beyond (truncation below 1e-13)
__device__ __forceinline__ float stirlerr(int k) {
    switch (k) {
    case 1: return 0x1.4c071cp-4f;  case 2: return 0x1.52a9bap-5f;  case 3: return 0x1.c579a2p-6f;
    case 4: return 0x1.54a266p-6f;  case 5: return 0x1.10b4e6p-6f;  case 6: return 0x1.c6b168p-7f;
    case 7: return 0x1.85d4d6p-7f;  case 8: return 0x1.552806p-7f;  case 9: return 0x1.2f4872p-7f;
    case 10: return 0x1.10f9d4p-7f; case 11: return 0x1.f05930p-8f; case 12: return 0x1.c70188p-8f;
    case 13: return 0x1.a40514p-8f; case 14: return 0x1.86076cp-8f; case 15: return 0x1.6c08f6p-8f;
    default: {
        float r = 1.0f / (float)k;
        float r2 = r * r;
        return r * (0.0833333358f - r2 * (0.00277777785f - r2 * (0.000793650805f - r2 * 0.000595238095f)));
    }
    }
}

// P(X = m) for X ~ Binomial(n, p), 0 < p < 1, q = 1 - p (Loader's form)
__device__ __forceinline__ float binom_pmf(int n, int m, float p, float q) {
    if (m == 0) return expf_((float)n * log1m_(p));
    if (m == n) return expf_((float)n * log1m_(q));
    float fn = (float)n;
    float lc = stirlerr(n) - stirlerr(m) - stirlerr(n - m) - bd0((float)m, fn * p) -
               bd0((float)(n - m), fn * q);
    const float inv2pi = 0.159154943091895336f;
    return expf_(lc) * sqrtf(fn * inv2pi / ((float)m * (float)(n - m)));
}

// first acceptor count a with floor(a * nbins / N) >= b. The store holds
// N <= 2^21 photons per burst and this path nbins <= 64, so every product
// below stays under 2^27: 32-bit unsigned division is exact.
__device__ __forceinline__ int bin_start(int b, int N, int nbins, Divisor dn) {
    return (int)div_by((unsigned)b * (unsigned)N + (unsigned)(nbins - 1), dn.m, dn.l);
}

__device__ __forceinline__ int bin_of(int a, int N, int nbins) {
    int b = (int)(((unsigned)a * (unsigned)nbins) / (unsigned)N);
    return b < nbins - 1 ? b : nbins - 1;
}

template <int NS>
struct ExpUnit {
    float acc;          // sum dt E
    float lw;           // log weight
    float dtl;          // duration of the last segment
    int s0, sm;         // first and last state
    float D[NS];        // time in each state over the segments before the last
    int cnt[NS][NS];    // jumps from -> to
};

// Where the adjoint's trajectory statistics live: STATS_REG in U.D / U.cnt
// (registers), STATS_SMEM in the thread's own columns of shared arrays,
// scnt[(i * NS + j) * kExpThreads] (jumps i -> j) and sD[i * kExpThreads]
// (time in state i): one shared-memory update per segment instead of NS * NS
// predicated register updates, and the registers freed for occupancy. The
// same integer counts and the same FP32 sums in the same order either way.
constexpr int STATS_NONE = 0, STATS_REG = 1, STATS_SMEM = 2;

// The trajectory of one unit under (skeleton theta0, dwells theta), then the
// background; returns false when the burst has no photons.
template <int NS, int STATS>
__device__ __forceinline__ bool exp_walk(const ExpParams &P, Rng &r, int Nb, float Tb, float bga,
                                         float bgd, ExpUnit<NS> &U, int &sig, int &ba, int &lim,
                                         const float *sinv, int *scnt = nullptr, float *sD = nullptr) {
    U.acc = 0.0f;
    U.lw = 0.0f;
    U.dtl = 0.0f;
    if (STATS == STATS_REG) {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            U.D[i] = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; ++j) U.cnt[i][j] = 0;
        }
    }
    if (STATS == STATS_SMEM) {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            sD[i * kExpThreads] = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; ++j) scnt[(i * NS + j) * kExpThreads] = 0;
        }
    }
    float t = 0.0f;
    int st = 0;
#if GPDA_EXP_PAIRS
    // Every segment draws two words (state, dwell), so a Philox block covers
    // two segments: the words are taken in place, the same draws in the same
    // order as one next() per draw. Returns true when the trajectory ends.
    auto step = [&](int seg, uint32_t xs, uint32_t xu) -> bool {
        const float us = Rng::u01_of(xs);
        int ns;
        if (seg == 0) {
            ns = cat_draw(P.init_cdf, NS, us);
            U.s0 = ns;
            U.lw += P.lw_init[ns];
        } else {
            ns = jump_draw(P.jump_cdf + st * 4, NS, st, us);
            U.lw += P.lw_jump[st * 4 + ns];
            if (STATS == STATS_REG) {
#pragma unroll
                for (int i = 0; i < NS; ++i)
#pragma unroll
                    for (int j = 0; j < NS; ++j)
                        if (i == st && j == ns) U.cnt[i][j] += 1;
            }
            if (STATS == STATS_SMEM) scnt[(st * NS + ns) * kExpThreads] += 1;
        }
        st = ns;
        if (!(Tb > 0.0f)) return true;
        const float u = Rng::u01_of(xu);
        float tau = (P.kexit[st] > 0.0f) ? (-logf_pos(u)) * P.inv_kexit[st] : kInf;
        float tn = t + tau;
        bool cut = seg == kMaxSeg - 1;
        bool last = !(tn < Tb) || cut;
        if (cut && tn < Tb) lim += 1;
        float dt = last ? Tb - t : tn - t;
        U.acc = fmaf(dt, P.E[st], U.acc);
        if (last) {
            U.dtl = dt;
            return true;
        }
        if (STATS == STATS_REG) {
#pragma unroll
            for (int i = 0; i < NS; ++i)
                if (i == st) U.D[i] += dt;
        }
        if (STATS == STATS_SMEM) sD[st * kExpThreads] += dt;
        t = tn;
        return false;
    };
    for (int seg = 0; seg < kMaxSeg; seg += 2) {
#if GPDA_EXP_PAIRS == 2
        const uint4 w = philox_block_inline(r.blk, r.c1, r.c2, r.c3, r.k0, r.k1);
        r.blk += 1u;
#else
        const uint4 w = r.block();
#endif
        if (step(seg, w.x, w.y) || step(seg + 1, w.z, w.w)) break;
    }
    if (false)
#endif
    for (int seg = 0; seg < kMaxSeg; ++seg) {
        const float us = r.u01();
        int ns;
        if (seg == 0) {
            ns = cat_draw(P.init_cdf, NS, us);
            U.s0 = ns;
            U.lw += P.lw_init[ns];
        } else {
            ns = jump_draw(P.jump_cdf + st * 4, NS, st, us);
            U.lw += P.lw_jump[st * 4 + ns];
            if (STATS == STATS_REG) {
#pragma unroll
                for (int i = 0; i < NS; ++i)
#pragma unroll
                    for (int j = 0; j < NS; ++j)
                        if (i == st && j == ns) U.cnt[i][j] += 1;
            }
            if (STATS == STATS_SMEM) scnt[(st * NS + ns) * kExpThreads] += 1;
        }
        st = ns;
        if (!(Tb > 0.0f)) break;
        float u = r.u01();
        float tau = (P.kexit[st] > 0.0f) ? (-logf_pos(u)) * P.inv_kexit[st] : kInf;
        float tn = t + tau;
        bool cut = seg == kMaxSeg - 1;
        bool last = !(tn < Tb) || cut;
        if (cut && tn < Tb) lim += 1;
        float dt = last ? Tb - t : tn - t;
        U.acc = fmaf(dt, P.E[st], U.acc);
        if (last) {
            U.dtl = dt;
            break;
        }
        if (STATS == STATS_REG) {
#pragma unroll
            for (int i = 0; i < NS; ++i)
                if (i == st) U.D[i] += dt;
        }
        if (STATS == STATS_SMEM) sD[st * kExpThreads] += dt;
        t = tn;
    }
    U.sm = st;
    // the background comes from a fixed block, so that its counts do not
    // change when a dwell crosses the end of the burst
    r.seek(kExpBgBlock);
    ba = GPDA_EXP_BG_OOL ? background_occ(r, Nb, bga * Tb, bgd * Tb, &sig, lim, sinv)
                         : background(r, Nb, bga * Tb, bgd * Tb, &sig, lim, sinv);
    return Nb > 0;
}

__device__ __forceinline__ float eps_p(float e, float g, float ct) { return eps_of(e, g, ct); }

// d eps / d E
__device__ __forceinline__ float eps_dp(float e, float g, float ct) {
    float om = 1.0f - e;
    float num = g * e + ct * om;
    float den = num + om;
    return ((g - ct) * om + num) / (den * den);
}

// Walks the masses of (ba + X) / N, X ~ Binomial(sig, p), one bin at a
// time, outward from the mode: F(bin, mass, sum of x * mass) is called
// exactly once for every bin the masses touch (the bin holding the mode is
// reached from both sides; the downward part of it is held back and joined to
// the upward part). Inside a bin the number of terms is known, so the term
// loop carries no bin test; the mass cut is tested every 4 terms.
template <bool WANT_X, class F>
__device__ __forceinline__ void binom_bins(int Nb, int sig, int ba, float p, int nbins, Divisor dn,
                                           const float *inv, F &&flush) {
    if (sig <= 0 || !(p > 0.0f)) {
        flush(bin_of(ba, Nb, nbins), 1.0f, 0.0f);
        return;
    }
    if (p >= 1.0f) {
        flush(bin_of(ba + sig, Nb, nbins), 1.0f, (float)sig);
        return;
    }
    const float q = 1.0f - p;
    int m = (int)((float)(sig + 1) * p);
    if (m > sig) m = sig;
    const float w0 = binom_pmf(sig, m, p, q);
    const float cut = w0 * kMassCut;
    const float rho = p / q, irho = q / p;
    const bool tab = sig + 1 < kExpInvN;
    const int bm = bin_of(ba + m, Nb, nbins);        // the mode's bin
    float hold = 0.0f, holdx = 0.0f;                // downward mass inside bin bm
    // downward: x = m-1 .. 0, ratio P(x-1)/P(x) = x / ((sig - x + 1) rho)
    if (m > 0) {
        int x = m - 1;
        float w = w0 * ((float)m * irho) * (tab ? __ldg(inv + sig - m + 1) : 1.0f / (float)(sig - m + 1));
        if (w >= cut) {
            float fx = (float)x;
            int b = bin_of(ba + x, Nb, nbins);
            bool more = true;
            while (more) {
                int first = bin_start(b, Nb, nbins, dn) - ba;
                if (first < 0) first = 0;
                int cnt = x - first + 1;
                float run = 0.0f, runx = 0.0f;
                while (cnt > 0) {
                    int k = cnt < 4 ? cnt : 4;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (j < k) {
                            run += w;
                            if (WANT_X) runx = fmaf(fx, w, runx);
                            float iv = tab ? __ldg(inv + sig - x + 1) : 1.0f / (float)(sig - x + 1);
                            w = w * (fx * irho) * iv;
                            fx -= 1.0f;
                            x -= 1;
                        }
                    }
                    cnt -= k;
                    if (w < cut) { more = false; break; }
                }
                if (b == bm) { hold = run; holdx = runx; }
                else flush(b, run, runx);
                if (x < 0) more = false;
                --b;
            }
        }
    }
    // upward: x = m .. sig, ratio P(x+1)/P(x) = (sig - x) rho / (x + 1)
    {
        int x = m;
        float w = w0;
        float fs = (float)(sig - m);
        float fx = (float)m;
        int b = bm;
        bool more = true;
        while (more) {
            int last = (b < nbins - 1) ? bin_start(b + 1, Nb, nbins, dn) - 1 - ba : sig;
            if (last > sig) last = sig;
            int cnt = last - x + 1;
            float run = 0.0f, runx = 0.0f;
            while (cnt > 0) {
                int k = cnt < 4 ? cnt : 4;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (j < k) {
                        run += w;
                        if (WANT_X) runx = fmaf(fx, w, runx);
                        float iv = tab ? __ldg(inv + x + 1) : 1.0f / (float)(x + 1);
                        w = w * (fs * rho) * iv;
                        fs -= 1.0f;
                        fx += 1.0f;
                        x += 1;
                    }
                }
                cnt -= k;
                if (w < cut) { more = false; break; }
            }
            if (b == bm) { run += hold; runx += holdx; }
            flush(b, run, runx);
            if (x > sig) more = false;
            ++b;
        }
    }
}

// sum of v[t * stride] over the block's threads in a fixed order, FP64;
// warp w of the block reduces the values it is given
__device__ __forceinline__ double warp_sum_fixed(const float *col, int lane) {
    double v = 0.0;
    for (int t = lane; t < kExpThreads; t += 32) v += (double)col[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int NS, bool TAPE>
__global__ void __launch_bounds__(kExpThreads) exp_fwd_kernel(const ExpArgs a) {
    extern __shared__ float sh_rows[];          // [nbins][kExpThreads]
    __shared__ float s_inv[kInvTable];
    __shared__ ExpParams sP;
    const int tid = threadIdx.x;
    const int p = blockIdx.y;
    if (tid < kInvTable) s_inv[tid] = tid > 0 ? 1.0f / (float)tid : 0.0f;
    if (tid < 128) reinterpret_cast<float *>(&sP)[tid] = reinterpret_cast<const float *>(a.params + p)[tid];
    for (int i = tid; i < a.nbins * kExpThreads; i += kExpThreads) sh_rows[i] = 0.0f;
    __syncthreads();
    const int64_t units = a.B * (int64_t)a.S;
    const int64_t stride = (int64_t)a.nblk * kExpThreads;
    const bool narrow = units + stride <= (int64_t)0xffffffffu;
    int lim = 0;
    float *row = sh_rows + tid;
    const int nb2 = 2 * a.nbins;
    const Divisor dn = divisor_of((uint32_t)a.nbins), dS = divisor_of((uint32_t)a.S);
    for (int64_t u = (int64_t)blockIdx.x * kExpThreads + tid; u < units; u += stride) {
        // (32-bit division by the invariant S whenever the unit count allows)
        const int b = narrow ? (int)div_by((uint32_t)u, dS.m, dS.l) : (int)(u / a.S);
        const int s = (int)(u - (int64_t)b * a.S);
        const int Nb = __ldg(a.N + b);
        const float Tb = __ldg(a.T + b);
        Rng r;
        r.init(a.seed, (uint32_t)p, (uint32_t)b, (uint32_t)s);
        ExpUnit<NS> U;
        int sig, ba;
        if (!exp_walk<NS, STATS_NONE>(sP, r, Nb, Tb, a.bg_a, a.bg_d, U, sig, ba, lim, s_inv)) continue;
        const float eeff = (Tb > 0.0f) ? U.acc / Tb : sP.E[U.sm];
        const float W = expf_(U.lw);
        const float pe = eps_p(eeff, a.gamma, a.ct);
        // the unit's tape slots: every touched bin written once (they form one
        // contiguous range), zeros around them
        float *t = TAPE ? a.tape + (size_t)p * nb2 * a.units_p + u : nullptr;
        int bmin = a.nbins, bmax = -1;
        binom_bins<TAPE>(Nb, sig, ba, pe, a.nbins, dn, a.inv, [&](int bin, float m, float mx) {
            row[bin * kExpThreads] += W * m;
            if (TAPE) {
                __stcs(t + (size_t)bin * a.units_p, m);
                __stcs(t + (size_t)(a.nbins + bin) * a.units_p, mx);
                bmin = bin < bmin ? bin : bmin;
                bmax = bin > bmax ? bin : bmax;
            }
        });
        if (TAPE)
            for (int f = 0; f < a.nbins; ++f)
                if (f < bmin || f > bmax) {
                    __stcs(t + (size_t)f * a.units_p, 0.0f);
                    __stcs(t + (size_t)(a.nbins + f) * a.units_p, 0.0f);
                }
    }
    if (lim) atomicAdd(a.limit_hits, (unsigned long long)lim);
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    double *out = a.part + ((size_t)p * a.nblk + blockIdx.x) * a.nbins;
    for (int bin = warp; bin < a.nbins; bin += kExpThreads / 32) {
        double v = warp_sum_fixed(sh_rows + bin * kExpThreads, lane);
        if (lane == 0) out[bin] = v;
    }
}

// sum over k < count of src[k * stride] in a fixed order: lane l adds
// k = l, l + 32, ... in turn, then a fixed shuffle tree; the result is in lane 0
__device__ __forceinline__ double warp_sum_strided(const double *src, int count, size_t stride,
                                                   int lane) {
    double v = 0.0;
    // (unrolled: the loads go out together, the additions keep their order)
#pragma unroll 16
    for (int k = lane; k < count; k += 32) v += src[(size_t)k * stride];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// One block of 1024 threads per parameter set: a warp per bin sums the
// per-block partials (32 bins at a time: the sums are latency bound), then
// the chi-square (sequential over bins, FP64, as chi2_kernel) and
// d chi2 / d count for each bin.
constexpr int kExpChi2Threads = 1024;
__global__ void __launch_bounds__(kExpChi2Threads) exp_chi2_kernel(const ExpArgs a) {
    __shared__ double sM[kExpMaxBins];
    __shared__ double s_den;
    const int p = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int bin = warp; bin < a.nbins; bin += kExpChi2Threads / 32) {
        double v = warp_sum_strided(a.part + (size_t)p * a.nblk * a.nbins + bin, a.nblk,
                                    (size_t)a.nbins, lane);
        if (lane == 0) {
            sM[bin] = v;
            a.hist[(size_t)p * a.nbins + bin] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int effN = a.nbins - a.left_pad;
        double chi = 0.0;
        for (int i = a.left_pad; i < a.nbins; ++i) {
            if (sM[i] > 0.0) {
                double mi = sM[i] / (double)a.S;
                double d = (double)a.obs[i] - mi;
                chi = chi + d * d / mi;
            } else {
                effN -= 1;
            }
        }
        const double den = (double)(effN - a.n * (a.n + 1));
        a.chi2[p] = chi / den;
        s_den = den;
    }
    __syncthreads();
    const int i = threadIdx.x;
    if (i < a.nbins) {
        double gi = 0.0;
        if (i >= a.left_pad && sM[i] > 0.0) {
            double mi = sM[i] / (double)a.S;
            double o = (double)a.obs[i];
            gi = (1.0 - (o * o) / (mi * mi)) / ((double)a.S * s_den);
        }
        a.g[(size_t)p * a.nbins + i] = (float)gi;
    }
}

template <int NS, bool TAPE>
__global__ void __launch_bounds__(kExpThreads) exp_adj_kernel(const ExpArgs a) {
    constexpr int NG = NS + NS * (NS - 1);
    constexpr bool kSm = GPDA_ADJ_SMEM != 0;
    __shared__ float s_inv[kInvTable];
    __shared__ float s_g[kExpMaxBins];
    __shared__ float s_red[NG][kExpThreads];
    __shared__ int s_cnt[kSm ? NS * NS : 1][kSm ? kExpThreads : 1];
    __shared__ float s_D[kSm ? NS : 1][kSm ? kExpThreads : 1];
    __shared__ ExpParams sP;
    const int tid = threadIdx.x;
    const int p = blockIdx.y;
    if (tid < kInvTable) s_inv[tid] = tid > 0 ? 1.0f / (float)tid : 0.0f;
    if (tid < 128) reinterpret_cast<float *>(&sP)[tid] = reinterpret_cast<const float *>(a.params + p)[tid];
    if (tid < a.nbins) s_g[tid] = a.g[(size_t)p * a.nbins + tid];
    __syncthreads();
    // the gradient sums: registers, or (kSm) the thread's column of s_red
    float gacc[kSm ? 1 : NG];
#pragma unroll
    for (int k = 0; k < NG; ++k) {
        if (kSm) s_red[k][tid] = 0.0f;
        else gacc[k] = 0.0f;
    }
    auto gadd = [&](int k, float v) -> float & { return kSm ? s_red[k][tid] : gacc[kSm ? 0 : k]; };
    int *const cnt_col = kSm ? &s_cnt[0][tid] : nullptr;
    float *const d_col = kSm ? &s_D[0][tid] : nullptr;
    const int64_t units = a.B * (int64_t)a.S;
    const int64_t stride = (int64_t)a.nblk_adj * kExpThreads;
    const bool narrow = units + stride <= (int64_t)0xffffffffu;
    int lim = 0;
    const Divisor dn = divisor_of((uint32_t)a.nbins), dS = divisor_of((uint32_t)a.S);
    for (int64_t u = (int64_t)blockIdx.x * kExpThreads + tid; u < units; u += stride) {
        // (32-bit division by the invariant S whenever the unit count allows)
        const int b = narrow ? (int)div_by((uint32_t)u, dS.m, dS.l) : (int)(u / a.S);
        const int s = (int)(u - (int64_t)b * a.S);
        const int Nb = __ldg(a.N + b);
        const float Tb = __ldg(a.T + b);
        Rng r;
        r.init(a.seed, (uint32_t)p, (uint32_t)b, (uint32_t)s);
        ExpUnit<NS> U;
        int sig, ba;
        if (!exp_walk<NS, kSm ? STATS_SMEM : STATS_REG>(sP, r, Nb, Tb, a.bg_a, a.bg_d, U, sig, ba, lim,
                                                        s_inv, cnt_col, d_col))
            continue;
        const bool timed = Tb > 0.0f;
        const float eeff = timed ? U.acc / Tb : sP.E[U.sm];
        const float W = expf_(U.lw);
        const float pe = eps_p(eeff, a.gamma, a.ct);
        float G = 0.0f, GX = 0.0f;
        if (TAPE) {
            const float *t = a.tape + (size_t)p * 2 * a.nbins * a.units_p + u;
            for (int bin = 0; bin < a.nbins; ++bin) {
                const float gb = s_g[bin];
                G = fmaf(gb, __ldcs(t + (size_t)bin * a.units_p), G);
                GX = fmaf(gb, __ldcs(t + (size_t)(a.nbins + bin) * a.units_p), GX);
            }
        } else {
            binom_bins<true>(Nb, sig, ba, pe, a.nbins, dn, a.inv, [&](int bin, float m, float mx) {
                const float gb = s_g[bin];
                G = fmaf(gb, m, G);
                GX = fmaf(gb, mx, GX);
            });
        }
        // H = sum g P'(x) = (sum g x P - sig p sum g P) / (p q); zero at p in {0, 1}
        float H = 0.0f;
        if (sig > 0 && pe > 0.0f && pe < 1.0f) H = (GX - (float)sig * pe * G) / (pe * (1.0f - pe));
        const float HE = W * H * eps_dp(eeff, a.gamma, a.ct);
        const float WG = W * G;
        // d / d E_s: occupancy fraction of state s
        const float invT = timed ? 1.0f / Tb : 0.0f;
        auto Dof = [&](int i) -> float { return kSm ? d_col[i * kExpThreads] : U.D[kSm ? 0 : i]; };
        auto cntof = [&](int i, int j) -> int {
            return kSm ? cnt_col[(i * NS + j) * kExpThreads] : U.cnt[kSm ? 0 : i][kSm ? 0 : j];
        };
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            float occ;
            if (timed) occ = (Dof(i) + (i == U.sm ? U.dtl : 0.0f)) * invT;
            else occ = (i == U.sm) ? 1.0f : 0.0f;
            float &g = gadd(i, 0.0f);
            g = fmaf(HE, occ, g);
        }
        // d / d ln K(l, i), rate i -> l: skeleton score and dwell pathwise term
        const float Esm = sP.E[U.sm];
#pragma unroll
        for (int l = 0; l < NS; ++l) {
#pragma unroll
            for (int i = 0; i < NS; ++i) {
                if (i == l) continue;
                const int idx = l * (NS - 1) + (i < l ? i : i - 1);
                int nout = 0;
#pragma unroll
                for (int j = 0; j < NS; ++j) nout += cntof(i, j);
                const float pj = sP.pj[i * 4 + l];
                float score = sP.dlnpi[U.s0 * 12 + idx] + (float)cntof(i, l) - (float)nout * pj;
                float path = -pj * Dof(i) * (sP.E[i] - Esm) * invT;
                float &g = gadd(NS + idx, 0.0f);
                g = fmaf(WG, score, fmaf(HE, path, g));
            }
        }
    }
    if (lim) atomicAdd(a.limit_hits, (unsigned long long)lim);
    if (!kSm) {
#pragma unroll
        for (int k = 0; k < NG; ++k) s_red[k][tid] = gacc[kSm ? 0 : k];
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    double *out = a.gpart + ((size_t)p * a.nblk_adj + blockIdx.x) * kExpGrad;
    for (int k = warp; k < NG; k += kExpThreads / 32) {
        double v = warp_sum_fixed(&s_red[k][0], lane);
        if (lane == 0) out[k] = v;
    }
}

// One block of kExpGrad warps per parameter set: warp k sums component k of
// the per-block partials in a fixed order and scales it by the upstream
// gradient.
__global__ void __launch_bounds__(32 * kExpGrad) exp_grad_kernel(const ExpArgs a) {
    const int p = blockIdx.x;
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ng = a.n + a.n * (a.n - 1);
    if (k >= ng) return;
    double v = warp_sum_strided(a.gpart + (size_t)p * a.nblk_adj * kExpGrad + k, a.nblk_adj,
                                (size_t)kExpGrad, lane);
    if (lane == 0) {
        const double up = a.dchi2 ? a.dchi2[p] : 1.0;
        a.grad[(size_t)p * kExpGrad + k] = v * up;
    }
}

__global__ void inv_table_kernel(float *inv) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < kExpInvN) inv[k] = k > 0 ? 1.0f / (float)k : 0.0f;
}

template <int NS, bool TAPE>
size_t fwd_smem(int nbins) { return sizeof(float) * (size_t)nbins * kExpThreads; }

template <int NS, bool TAPE>
cudaError_t fwd_t(const ExpArgs &a, cudaStream_t st) {
    const size_t dyn = fwd_smem<NS, TAPE>(a.nbins);
    cudaError_t e = cudaFuncSetAttribute(exp_fwd_kernel<NS, TAPE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    exp_fwd_kernel<NS, TAPE><<<dim3(a.nblk, a.P), kExpThreads, dyn, st>>>(a);
    return cudaGetLastError();
}

template <int NS>
cudaError_t fwd_n(const ExpArgs &a, cudaStream_t st) {
    return a.tape ? fwd_t<NS, true>(a, st) : fwd_t<NS, false>(a, st);
}

template <int NS>
cudaError_t adj_n(const ExpArgs &a, cudaStream_t st) {
    if (a.tape) exp_adj_kernel<NS, true><<<dim3(a.nblk_adj, a.P), kExpThreads, 0, st>>>(a);
    else exp_adj_kernel<NS, false><<<dim3(a.nblk_adj, a.P), kExpThreads, 0, st>>>(a);
    return cudaGetLastError();
}

template <int NS, bool TAPE>
cudaError_t occ_t(int nbins, int *fwd, int *adj) {
    const size_t dyn = fwd_smem<NS, TAPE>(nbins);
    cudaError_t e = cudaFuncSetAttribute(exp_fwd_kernel<NS, TAPE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(fwd, exp_fwd_kernel<NS, TAPE>, kExpThreads, dyn);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(adj, exp_adj_kernel<NS, TAPE>, kExpThreads, 0);
}

template <int NS>
cudaError_t occ_n(int nbins, bool tape, int *fwd, int *adj) {
    return tape ? occ_t<NS, true>(nbins, fwd, adj) : occ_t<NS, false>(nbins, fwd, adj);
}

}  // namespace

cudaError_t launch_exp_forward(const ExpArgs &a, cudaStream_t st) {
    cudaError_t e;
    switch (a.n) {
    case 1: e = fwd_n<1>(a, st); break;
    case 2: e = fwd_n<2>(a, st); break;
    case 3: e = fwd_n<3>(a, st); break;
    case 4: e = fwd_n<4>(a, st); break;
    default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    exp_chi2_kernel<<<a.P, kExpChi2Threads, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_exp_adjoint(const ExpArgs &a, cudaStream_t st) {
    cudaError_t e;
    switch (a.n) {
    case 1: e = adj_n<1>(a, st); break;
    case 2: e = adj_n<2>(a, st); break;
    case 3: e = adj_n<3>(a, st); break;
    case 4: e = adj_n<4>(a, st); break;
    default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    exp_grad_kernel<<<a.P, 32 * kExpGrad, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_exp_inv_table(float *inv, cudaStream_t st) {
    inv_table_kernel<<<(kExpInvN + 255) / 256, 256, 0, st>>>(inv);
    return cudaGetLastError();
}

// Blocks per parameter set for each kernel: one wave of the device over all
// parameter sets (the units are strided over the blocks of a set), and no
// more blocks than the units need.
cudaError_t exp_grid(int n, int nbins, int P, int64_t units, int num_sms, bool tape, int *nblk_fwd,
                     int *nblk_adj) {
    int of = 1, oa = 1;
    cudaError_t e;
    switch (n) {
    case 1: e = occ_n<1>(nbins, tape, &of, &oa); break;
    case 2: e = occ_n<2>(nbins, tape, &of, &oa); break;
    case 3: e = occ_n<3>(nbins, tape, &of, &oa); break;
    case 4: e = occ_n<4>(nbins, tape, &of, &oa); break;
    default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    const int64_t need = (units + kExpThreads - 1) / kExpThreads;
    auto per = [&](int occ) {
        int64_t want = (int64_t)num_sms * std::max(1, occ) / std::max(1, P);
        return (int)std::max<int64_t>(1, std::min(want, need));
    };
    *nblk_fwd = per(of);
    *nblk_adj = per(oa);
    return cudaSuccess;
}

}  // namespace gpda
