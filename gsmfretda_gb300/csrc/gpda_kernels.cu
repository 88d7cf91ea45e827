// gpda_kernels.cu — sm_103a kernels of the photon-burst Monte-Carlo PDA path.
//
//   pda_kernel<MODE>   persistent CTAs pull (parameter set, burst tile) work
//                      items from an atomic counter; the tile's photon counts,
//                      durations and (photon mode) arrival offsets are staged
//                      in shared memory with 16-byte vector loads; each thread
//                      simulates (burst, sample) units and bins the proximity
//                      ratio into a shared-memory histogram with warp-
//                      aggregated atomics; the histogram is flushed once per
//                      work item; the last CTA to finish computes the reduced
//                      chi-square (src/streamWorker.cpp:197-206) in FP64.
//                      MODE 0: occupancy-weighted E; rounds of one unit per
//                      thread: trajectories, then the background + binomial
//                      splits regrouped by sampler across the CTA. MODE 1: photon-by-photon
//                      state assignment, one binomial per dwell segment,
//                      drawn from tabulated CDFs (one 16-byte guide entry).
//                      MODE 2: MODE 1 whose CTAs stage their tiles from the
//                      caller's page-locked host arrays and write them
//                      through to the burst store (gpda_run_host).
//   binom_table_kernel the photon-mode CDF rows, one warp per row.
//   chi2_kernel        reduced chi-square per parameter set, for callers that
//                      launch without an observed histogram in the context.
//   rc_kernel          mc_kernel's semantics (src/mc.cu:83-197), one thread
//                      per (burst, sample), fused with the reference's
//                      histogram binning (src/streamWorker.cpp:33-38).
//   validate_kernel    burst-store checks, one warp per burst.
//
// No tensor cores: nothing here is a contraction. The work is INT32 (Philox)
// and FP32 ALU bound; HBM traffic is the burst store read once per item.
#include <algorithm>

#include "gpda_device.cuh"
#include "gpda_internal.h"

namespace gpda {

// direct reads: host-memory loads each thread keeps in flight while staging
constexpr int kStageBatch = 4;

// occupancy mode: the same order (1); 64 population sets with untuned tiles
// 13.66 -> 13.49 ms, the same bits
#ifndef GPDA_LPT_OCC
#define GPDA_LPT_OCC 1
#endif
// photon mode: each tile's bursts taken longest first (1). Measured on
// photon_3state: MC kernel with its tables 0.640 -> 0.617 ms, gpda_run_host
// 0.736 -> 0.704 ms per call, the same bits.
#ifndef GPDA_LPT
#define GPDA_LPT 1
#endif

// occupancy mode: units per thread per round (trajectories and background of
// all of them, then one barrier and the regrouped binomial splits)
#ifndef GPDA_OCC_ROUND
#define GPDA_OCC_ROUND 1
#endif
constexpr int kOccRound = GPDA_OCC_ROUND;
// with one unit per thread per round: a CTA barrier between the
// trajectories and the background draws (1)
#ifndef GPDA_OCC_MIDSYNC
#define GPDA_OCC_MIDSYNC 1
#endif
constexpr int kOccEntries = kOccRound * kThreads;

// a divisor kept in shared memory, read at each use (so that it does not hold
// two registers across the simulation loop)
__device__ __forceinline__ Divisor sdiv(const uint32_t &m, const uint32_t &l) {
    return Divisor{*(const volatile uint32_t *)&m, *(const volatile uint32_t *)&l};
}

// The proximity-ratio bin min(A nbins / N, nbins - 1) of A acceptor photons
// out of N (0 <= A <= N <= 2^21, nbins <= 1024), exact. x = A nbins < 2^31;
// the float quotient (x rounded to float, then the approximate division,
// relative error below 2^-21 in all) is within 5e-4 of x / N <= 1024, so its
// truncation v is floor(x / N) or one off, and one integer comparison each
// way corrects it (v N <= 1025 * 2^21 < 2^32).
#ifndef GPDA_PR_BIN
#define GPDA_PR_BIN 1
#endif
__device__ __forceinline__ int pr_bin(int A, int N, int nbins) {
    const uint32_t x = (uint32_t)A * (uint32_t)nbins;
    const uint32_t n = (uint32_t)N;
    uint32_t v = __float2uint_rz(__fdividef((float)x, (float)N));
    const uint32_t vn = v * n;
    if (vn > x) v -= 1u;
    else if (x - vn >= n) v += 1u;
    return v >= (uint32_t)nbins ? nbins - 1 : (int)v;
}

// number of offsets < x in the sorted range a[lo, hi)
__device__ __forceinline__ int lower_bound(const float *a, int lo, int hi, float x) {
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// One (burst, sample) unit in flight on a lane. The trajectory advances one
// dwell segment per step so that a lane whose unit is finished can take the
// next unit at once instead of idling until the slowest lane of its warp is
// done (trajectory lengths vary from 1 to tens of segments).
struct Unit {
    Rng r;
    float t, acc, Tb;
    int st, lo, A, seg, Nb;
    int lb, s;          // tile-local burst, sample
    int obase;          // staged: offset of the burst in shared memory
    bool done;
};

__device__ __forceinline__ void unit_begin(Unit &U, int u, int S, Divisor dS, int64_t tb0,
                                           const int32_t *sN, const float *sT, uint64_t seed,
                                           uint32_t pw, const uint8_t *order = nullptr) {
    const int k = (int)div_by((uint32_t)u, dS.m, dS.l);
    U.s = u - k * S;
    U.lb = order ? (int)order[k] : k;
    U.Nb = sN[U.lb];
    U.Tb = sT[U.lb];
    U.r.init(seed, pw, (uint32_t)(tb0 + U.lb), (uint32_t)U.s);
    U.t = 0.0f;
    U.acc = 0.0f;
    U.lo = 0;
    U.A = 0;
    U.seg = 0;
    U.st = 0;
    U.done = U.Nb <= 0;
    if (U.done) U.A = -1;
}

// State of segment U.seg: the stationary draw for the first segment, the jump
// from the previous state afterwards (one word, the first of the step).
__device__ __forceinline__ int next_state(const Unit &U, const DevParams &P, float us) {
    return (U.seg == 0) ? cat_draw(P.init_cdf, P.n, us)
                        : jump_draw(P.jump_cdf + U.st * 8, P.n, U.st, us);
}

// Binomial(n, eps) of a photon-mode segment (eps = eps_state, V_state = 0):
// same early returns as binom(); for n <= kTableN one uniform inverts the
// tabulated CDF of Binomial(n, min(eps, 1-eps)): the smallest k with
// u <= cdf[k] (cdf[n] = 1); larger n fall back to BINV/BTRD.
__device__ __forceinline__ int binom_table(Rng &r, int n, const DevParams &P, int st,
                                           const float *cdf_p, const GuideEntry *guide_p, int &lim,
                                           const float *inv) {
    const float p = P.eps[st];
    if (n <= 0 || !(p > 0.0f)) return 0;
    if (p >= 1.0f) return n;
    if (n > kTableN) return binom_pre(r, n, p, P.bpp[st], P.blogq[st], P.brr[st], lim, inv);
    const bool flip = p > 0.5f;
    const int row = st * kTableRows + n * (n + 1) / 2;
    const float *cdf = cdf_p + row;
    const float u = r.u01();
    int j = (int)(u * (float)(n + 1));
    if (j > n) j = n;
    const GuideEntry e = __ldg(guide_p + row + j);
    int k = (int)e.x;
    if (u <= __uint_as_float(e.w)) {                 // rounding of j: below the start
        k -= 1;
        while (k > 0 && u <= __ldg(cdf + k - 1)) --k;
    } else if (u > __uint_as_float(e.y)) {
        k += 1;
        if (u > __uint_as_float(e.z)) {
            k += 1;
            while (k < n && u > __ldg(cdf + k)) ++k;
        }
    }
    return flip ? n - k : k;
}

// Photon mode: one dwell segment. Draw order per step: a fresh Philox block
// [state, dwell, background pair, binomial] (a rare extra draw of the
// background or the samplers continues in the following blocks). Photons
// whose arrival offset falls in the segment take its state; the Poisson
// background pair (background_pair, bgc its constants), then
// Binomial(signal, eps_state).
__device__ __forceinline__ bool step_pho(Unit &U, const DevParams &P, const float *offs, float g,
                                         float ct, float r0, const float *bgc, int &lim,
                                         const float *inv, const float *cdf_p,
                                         const GuideEntry *guide_p) {
    U.r.align_now();   // the state draw follows at once
    const int st = next_state(U, P, U.r.u01());
    U.st = st;
    float u = U.r.u01();
    float tau = (P.kexit[st] > 0.0f) ? (-logf_pos(u)) * P.inv_kexit[st] : kInf;
    float tn = U.t + tau;
    bool cut = U.seg == kMaxSeg - 1;
    bool last = !(tn < U.Tb) || cut;
    if (cut && tn < U.Tb) lim += 1;
    int hi;
    float dt;
    if (last) { hi = U.Nb; dt = U.Tb - U.t; }
    else { hi = lower_bound(offs, U.lo, U.Nb, tn); dt = tn - U.t; }
    int nk = hi - U.lo;
    if (nk > 0) {
        int sig;
        int ba = background_pair(U.r, nk, dt, bgc, &sig, lim, inv);
        if (P.V[st] > 0.0f) {
            float ek = eps_of(broaden(U.r, P.E[st], r0, P.V[st]), g, ct);
            U.A += binom<false>(U.r, sig, ek, lim, inv) + ba;
        } else {
            U.A += binom_table(U.r, sig, P, st, cdf_p, guide_p, lim, inv) + ba;
        }
    }
    U.lo = hi;
    if (last) return true;
    U.t = tn;
    U.seg += 1;
    return false;
}

// Occupancy mode: one dwell segment per step, draws [state, dwell]; returns
// true once the trajectory has reached the end of the burst (U.acc then holds
// the occupancy-weighted efficiency times T). Then a fresh block for the
// background and the single binomial split with the occupancy-weighted
// efficiency (pda_kernel<0>).
__device__ __forceinline__ bool traj_occ(Unit &U, const DevParams &P, float r0, int &lim) {
    const int st = next_state(U, P, U.r.u01());
    U.st = st;
    if (!(U.Tb > 0.0f)) return true;
    float u = U.r.u01();
    float tau = (P.kexit[st] > 0.0f) ? (-logf_pos(u)) * P.inv_kexit[st] : kInf;
    float tn = U.t + tau;
    bool cut = U.seg == kMaxSeg - 1;
    bool last = !(tn < U.Tb) || cut;
    if (cut && tn < U.Tb) lim += 1;
    float dt = last ? U.Tb - U.t : tn - U.t;
    float es = P.E[st];
    if (P.V[st] > 0.0f) es = broaden(U.r, es, r0, P.V[st]);
    U.acc = fmaf(dt, es, U.acc);
    if (last) return true;
    U.t = tn;
    U.seg += 1;
    return false;
}

// traj_occ for parameter sets without distance broadening (every segment
// draws exactly two words, state and dwell), with the segment's two words
// given: the caller takes them from one Philox block per pair of segments,
// the same draws in the same order as traj_occ's two u01() calls.
__device__ __forceinline__ bool traj_occ_words(Unit &U, const DevParams &P, int &lim, uint32_t xs,
                                               uint32_t xu) {
    const int st = next_state(U, P, Rng::u01_of(xs));
    U.st = st;
    if (!(U.Tb > 0.0f)) return true;
    float u = Rng::u01_of(xu);
    float tau = (P.kexit[st] > 0.0f) ? (-logf_pos(u)) * P.inv_kexit[st] : kInf;
    float tn = U.t + tau;
    bool cut = U.seg == kMaxSeg - 1;
    bool last = !(tn < U.Tb) || cut;
    if (cut && tn < U.Tb) lim += 1;
    float dt = last ? U.Tb - U.t : tn - U.t;
    U.acc = fmaf(dt, P.E[st], U.acc);
    if (last) return true;
    U.t = tn;
    U.seg += 1;
    return false;
}

// 1: occupancy trajectories without broadening take their segments in pairs
// from one block (traj_occ_words)
#ifndef GPDA_OCC_PAIRS
#define GPDA_OCC_PAIRS 1
#endif


// warp-aggregated shared-memory histogram increment; all 32 lanes call it
// (bin < 0: no count)
__device__ __forceinline__ void hist_add_warp(unsigned int *sh, int bin) {
    unsigned peers = __match_any_sync(0xffffffffu, bin);
    int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader && bin >= 0) atomicAdd(&sh[bin], (unsigned)__popc(peers));
}

// warp-aggregated shared-memory histogram increment from divergent code
__device__ __forceinline__ void hist_add(unsigned int *sh, int bin) {
    unsigned mask = __activemask();
    unsigned peers = __match_any_sync(mask, bin);
    int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader && bin >= 0) atomicAdd(&sh[bin], (unsigned)__popc(peers));
}

// Reduced chi-square of parameter set p (src/streamWorker.cpp:197-206), FP64,
// sequential over bins; the counts are read past L1 (__ldcg), since other
// CTAs wrote them with atomics.
__device__ __forceinline__ double chi2_of(const unsigned long long *h, const float *obs, int nbins,
                                          int left_pad, int S, int n_states) {
    int effN = nbins - left_pad;
    double chi = 0.0;
    for (int i = left_pad; i < nbins; ++i) {
        const unsigned long long c = __ldcg(h + i);
        if (c > 0ull) {
            double mi = (double)c / (double)S;
            double d = (double)obs[i] - mi;
            chi = chi + d * d / mi;
        } else {
            effN -= 1;
        }
    }
    return chi / (double)(effN - n_states * (n_states + 1));
}

// the last CTA to finish computes every parameter set's chi-square (no CTA
// waits: each counts itself once, after its own atomics); out of line so that
// the simulation loop's registers are not shaped by it
static __device__ __noinline__ void last_cta_chi2(const PdaArgs &a) {
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    const unsigned target = a.done_target ? a.done_target : gridDim.x;
    if (threadIdx.x == 0) s_last = (atomicAdd(a.done, 1u) == target - 1) ? 1 : 0;
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int q = threadIdx.x; q < a.P; q += kThreads)
            a.chi2[q] = chi2_of(a.hist + (size_t)q * a.nbins, a.obs, a.nbins, a.left_pad, a.S,
                                a.n_states);
    }
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, kMinBlocks) pda_kernel(const PdaArgs a) {
    // MODE 2 is photon mode with direct reads of the caller's host arrays
    // (PdaArgs::hN): its own instantiation, so that the staging code and its
    // registers stay out of the resident photon kernel
    constexpr bool kPhoton = MODE != 0;
    constexpr bool direct = MODE == 2;
    extern __shared__ float4 s_ph4[];
    float *s_ph = reinterpret_cast<float *>(s_ph4);
    __shared__ DevParams sp;
    __shared__ int32_t sN[kMaxTileBursts];
    __shared__ float sT[kMaxTileBursts];
    __shared__ int32_t sOff[kMaxTileBursts + 1];
    __shared__ uint32_t sNm[kMaxTileBursts];    // divisor_of(N) of the tile's bursts
    __shared__ uint8_t sNl[kMaxTileBursts];
    __shared__ uint32_t s_Sm, s_Sl;              // divisor_of(S)
    __shared__ unsigned int sh[kHistBins];
    __shared__ int s_item;
    __shared__ int s_staged;
    __shared__ int s_next;
    __shared__ float s_inv[kInvTable];
    __shared__ uint32_t s_ent[10][kOccEntries];  // occupancy mode: sorted splits
    __shared__ int s_nf[2], s_nb[2];             // their counts, alternating by round
    __shared__ uint8_t s_order[kMaxTileBursts];  // the tile's bursts, longest first
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    // a rejected burst store: nothing to simulate. One read per CTA (the flag
    // may still change while later ranges are validated), so the whole CTA
    // takes the same branch.
    __shared__ int s_abort;
    if (tid == 0) {
        s_abort = (a.abort_flag && __ldcg(a.abort_flag) != 0u) ? 1 : 0;
        const Divisor dS = divisor_of((uint32_t)a.S);
        s_Sm = dS.m;
        s_Sl = dS.l;
    }
    __syncthreads();
    if (s_abort) return;
    if (tid < kInvTable) s_inv[tid] = tid > 0 ? 1.0f / (float)tid : 0.0f;
    // photon mode: the background pair's constants (background_pair)
    __shared__ float s_bgc[4];
    if (kPhoton && tid == 0) {
        const float bgs = a.bg_a + a.bg_d;
        const float pa = a.bg_a / bgs;
        s_bgc[0] = bgs;
        s_bgc[1] = pa;
        s_bgc[2] = 1.0f / pa;
        s_bgc[3] = 1.0f / (1.0f - pa);
    }
    const unsigned lt_mask = (1u << lane) - 1u;
    // direct reads: the tile comes from the caller's host arrays and is
    // written through to the store
    __shared__ int64_t sOI[direct ? kMaxTileBursts + 1 : 1];   // the tile's off_idx
    int lim = 0;
    for (;;) {
        if (tid == 0) {
            s_item = (int)atomicAdd(a.work, 1u);
            s_next = kThreads;
        }
        __syncthreads();
        const int item = s_item;
        if (item >= a.n_items) break;
        const int p = item / a.ntiles;
        const int tile = item - p * a.ntiles;
        const int64_t tb0 = a.b0 + (int64_t)tile * a.tile_b;
        const int nb = (int)min((int64_t)a.tile_b, a.b1 - tb0);
        {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(a.params + p);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
            for (int i = tid; i < kParamWords; i += kThreads) dst[i] = src[i];
        }
        if (!direct) {
            for (int i = tid; i < nb; i += kThreads) {
                sN[i] = a.N[tb0 + i];
                sT[i] = a.T[tb0 + i];
            }
        } else {
            // host memory is microseconds away: N, T and off_idx of the tile
            // in one round trip, off_idx kept in shared memory
            for (int i = tid; i <= nb; i += kThreads) {
                if (i < nb) {
                    sN[i] = a.hN[tb0 + i];
                    sT[i] = a.hT[tb0 + i];
                }
                sOI[i] = a.hOffIdx[tb0 + i];
            }
            __syncthreads();
        }
        // occupancy mode (and photon mode without pr_bin): the bursts'
        // divisors for binning (each thread reads the sN entries it wrote
        // itself; the simulation reads them after a barrier)
        for (int i = tid; (!kPhoton || !GPDA_PR_BIN) && i < nb; i += kThreads) {
            const int32_t n_ = sN[i];
            const Divisor d = divisor_of(n_ > 0 ? (uint32_t)n_ : 1u);
            sNm[i] = d.m;
            sNl[i] = (uint8_t)d.l;
        }
        for (int i = tid; i < a.nbins; i += kThreads) sh[i] = 0u;
        if (kPhoton && a.vflag) {
            // the store's checks for the item's bursts (validate_kernel's),
            // before the reads they bound; offsets follow once staged (direct
            // reads: each thread checks the sN, sT entries it wrote itself)
            unsigned bad = 0u;
            for (int i = tid; i < nb; i += kThreads) {
                const int32_t n_ = direct ? sN[i] : a.N[tb0 + i];
                const float t_ = direct ? sT[i] : a.T[tb0 + i];
                if (n_ < 0 || n_ > (1 << 21)) bad |= 1u;
                if (!(t_ >= 0.0f) || !isfinite(t_)) bad |= 2u;
                const int64_t lo = direct ? sOI[i] : a.off_idx[tb0 + i];
                const int64_t hi = direct ? sOI[i + 1] : a.off_idx[tb0 + i + 1];
                if (hi - lo != (int64_t)n_ || lo < 0 || hi > a.nph) bad |= 4u;
            }
            if (bad) atomicOr(a.vflag, bad);
            if (__syncthreads_or(bad != 0u)) continue;
        }
        if (kPhoton) {
            // Stage the tile's offsets: copy the 16-byte-aligned span that
            // covers [off_idx[tb0], off_idx[tb0+nb]) (the store is padded).
            const int64_t first = direct ? sOI[0] : a.off_idx[tb0];
            const int64_t last = direct ? sOI[nb] : a.off_idx[tb0 + nb];
            const int64_t abase = first & ~(int64_t)3;
            const int64_t aend = (last + 3) & ~(int64_t)3;
            const bool staged = (aend - abase) <= (int64_t)a.smem_cap;
            if (staged) {
                for (int i = tid; i <= nb; i += kThreads)
                    sOff[i] = (int32_t)((direct ? sOI[i] : a.off_idx[tb0 + i]) - abase);
                const int nv = (int)((aend - abase) >> 2);
                if (!direct) {
                    const float4 *src = reinterpret_cast<const float4 *>(a.offsets + abase);
                    // an exactly sized array ends at a photon of some tile:
                    // whole vectors below the tile's last photon, the last
                    // one element by element (zeros past it, which no burst
                    // of this tile reads)
                    const int64_t vend = a.exact_offsets ? last : INT64_MAX;
                    for (int i = tid; i < nv; i += kThreads) {
                        const int64_t e = abase + 4 * (int64_t)i;
                        float4 v;
                        if (e + 4 <= vend) {
                            v = __ldg(src + i);
                        } else {
                            v.x = (e < vend) ? a.offsets[e] : 0.0f;
                            v.y = (e + 1 < vend) ? a.offsets[e + 1] : 0.0f;
                            v.z = (e + 2 < vend) ? a.offsets[e + 2] : 0.0f;
                            v.w = 0.0f;
                        }
                        s_ph4[i] = v;
                    }
                } else {
                    // kStageBatch loads in flight per thread. The host array
                    // is not padded: whole vectors below nph, the last one
                    // element by element (zeros past nph, as in the store's
                    // padding). The span's vectors go to the store too (its
                    // ends overlap the neighbouring tiles' spans, which write
                    // the same values).
                    const float4 *src = reinterpret_cast<const float4 *>(a.hOff + abase);
                    float4 *dst = reinterpret_cast<float4 *>(a.wOff + abase);
                    for (int i0 = tid; i0 < nv; i0 += kStageBatch * kThreads) {
                        float4 v[kStageBatch];
#pragma unroll
                        for (int u = 0; u < kStageBatch; ++u) {
                            const int i = i0 + u * kThreads;
                            const int64_t e = abase + 4 * (int64_t)i;
                            if (i < nv && e + 4 <= a.nph) {
                                v[u] = __ldg(src + i);
                            } else {
                                const bool in = i < nv;
                                v[u].x = (in && e < a.nph) ? a.hOff[e] : 0.0f;
                                v[u].y = (in && e + 1 < a.nph) ? a.hOff[e + 1] : 0.0f;
                                v[u].z = (in && e + 2 < a.nph) ? a.hOff[e + 2] : 0.0f;
                                v[u].w = 0.0f;
                            }
                        }
#pragma unroll
                        for (int u = 0; u < kStageBatch; ++u) {
                            const int i = i0 + u * kThreads;
                            if (i < nv) {
                                s_ph4[i] = v[u];
                                dst[i] = v[u];
                            }
                        }
                    }
                }
            } else if (direct) {
                // a tile too large to stage: copied to the store, from which
                // this CTA then reads it
                for (int64_t j0 = first + tid; j0 < last; j0 += kStageBatch * kThreads) {
                    float v[kStageBatch];
#pragma unroll
                    for (int u = 0; u < kStageBatch; ++u) {
                        const int64_t j = j0 + (int64_t)u * kThreads;
                        v[u] = (j < last) ? a.hOff[j] : 0.0f;
                    }
#pragma unroll
                    for (int u = 0; u < kStageBatch; ++u) {
                        const int64_t j = j0 + (int64_t)u * kThreads;
                        if (j < last) a.wOff[j] = v[u];
                    }
                }
            }
            if (direct) {
                for (int i = tid; i <= nb; i += kThreads) {
                    if (i < nb) {
                        a.wN[tb0 + i] = sN[i];
                        a.wT[tb0 + i] = sT[i];
                    }
                    a.wOffIdx[tb0 + i] = sOI[i];
                }
            }
            if (tid == 0) s_staged = staged ? 1 : 0;
        }
        __syncthreads();
        const int units = nb * a.S;
        const bool staged = kPhoton && s_staged;
        const uint32_t pw = a.pbase + (uint32_t)p;
#if GPDA_LPT
        // the tile's bursts longest first (rank by duration, ties by index):
        // in photon mode the units left at the end of the tile are short
        // ones; in occupancy mode each round's units have similar durations,
        // so the round's barrier waits less for its longest trajectory. A
        // unit's draws depend only on its (burst, sample).
        if (kPhoton || GPDA_LPT_OCC) {
            // rank on an integer key that orders every bit pattern (the
            // float order for numbers, NaNs at the ends), so that the ranks
            // are a permutation of 0..nb-1 whatever the durations hold
            auto key = [](float t) {
                const int k = __float_as_int(t);
                return k ^ ((k >> 31) & 0x7fffffff);
            };
            for (int i = tid; i < nb; i += kThreads) {
                const int ki = key(sT[i]);
                int rank = 0;
                for (int j = 0; j < nb; ++j) {
                    const int kj = key(sT[j]);
                    rank += (kj > ki || (kj == ki && j < i)) ? 1 : 0;
                }
                s_order[rank] = (uint8_t)i;
            }
            __syncthreads();
        }
#endif
        if (kPhoton && a.vflag) {
            // offsets finite and sorted within each burst; a warp per burst
            unsigned bad = 0u;
            for (int i = tid >> 5; i < nb; i += kThreads / 32) {
                const float *o = staged ? (s_ph + sOff[i]) : (a.offsets + a.off_idx[tb0 + i]);
                const int n_ = sN[i];
                for (int j = lane; j < n_; j += 32) {
                    const float x = o[j];
                    if (!isfinite(x)) bad |= 8u;
                    if (j > 0 && x < o[j - 1]) bad |= 16u;
                }
            }
            if (bad) atomicOr(a.vflag, bad);
            if (__syncthreads_or(bad != 0u)) continue;
        }
        if (MODE == 0) {
            // Rounds of kOccRound units per thread. 1. each thread runs its
            // unit's trajectory; 2. background, and the binomial split
            // classified by sampler (the inversion BINV for n min(p,q) < 10,
            // else BTRD): its arguments and remaining random words go to a
            // shared list, BINV from the front, BTRD from the back (1 and 2
            // repeat for the thread's next unit of the round); 3. thread t
            // finishes entries t, t + kThreads, ..., so that few warps mix
            // the two samplers. Every unit continues its own Philox stream:
            // results do not depend on which thread finishes it. The counts
            // of round r live in s_nf/s_nb[r & 1]; the other pair is cleared
            // during the round.
            if (tid == 0) { s_nf[0] = s_nf[1] = 0; s_nb[0] = s_nb[1] = 0; }
            __syncthreads();
            int rr = 0;
            for (int r0 = 0; r0 < units; r0 += kOccEntries, ++rr) {
                const int c = rr & 1;
                for (int k = 0; k < kOccRound; ++k) {
                    const int u = r0 + k * kThreads + tid;
                    const bool act = u < units;
                    Unit U;
                    int bin = -1;
                    if (act) {
                        unit_begin(U, u, a.S, sdiv(s_Sm, s_Sl), tb0, sN, sT, a.seed, pw,
                                   (GPDA_LPT && GPDA_LPT_OCC) ? s_order : nullptr);
                        if (!U.done) {
                            if (GPDA_OCC_PAIRS && !sp.anyV) {
                                for (;;) {
                                    const uint4 w = philox_block_inline(U.r.blk, U.r.c1, U.r.c2, U.r.c3,
                                                                        U.r.k0, U.r.k1);
                                    U.r.blk += 1u;
                                    if (traj_occ_words(U, sp, lim, w.x, w.y) ||
                                        traj_occ_words(U, sp, lim, w.z, w.w))
                                        break;
                                }
                            } else {
                                while (!traj_occ(U, sp, a.r0, lim)) {
                                }
                            }
                        }
                    }
                    if (kOccRound == 1 && GPDA_OCC_MIDSYNC) __syncthreads();
                    if (act && !U.done) {
                        const float eeff = (U.Tb > 0.0f) ? U.acc / U.Tb : sp.E[U.st];
                        U.r.align();
                        int sig;
                        const int ba = background_occ(U.r, U.Nb, a.bg_a * U.Tb, a.bg_d * U.Tb, &sig, lim, s_inv);
                        const float pe = eps_of(eeff, a.gamma, a.ct);
                        if (sig <= 0 || !(pe > 0.0f)) U.A = ba;
                        else if (pe >= 1.0f) U.A = ba + sig;
                        else {
                            const float pp = pe > 0.5f ? 1.0f - pe : pe;
                            const bool inv_sampler = (float)sig * pp < 10.0f;
                            const int slot = inv_sampler ? atomicAdd(&s_nf[c], 1)
                                                         : kOccEntries - 1 - atomicAdd(&s_nb[c], 1);
                            s_ent[0][slot] = (uint32_t)u;
                            s_ent[1][slot] = (uint32_t)sig;
                            s_ent[2][slot] = (uint32_t)ba;
                            s_ent[3][slot] = __float_as_uint(pe);
                            s_ent[4][slot] = U.r.blk;
                            s_ent[5][slot] = (uint32_t)U.r.idx;
                            s_ent[6][slot] = U.r.w0;
                            s_ent[7][slot] = U.r.w1;
                            s_ent[8][slot] = U.r.w2;
                            s_ent[9][slot] = U.r.w3;
                            U.A = -2;                   // finished in phase 3
                        }
                    }
                    if (act && U.A != -2) {
                        const int64_t b = tb0 + U.lb;
                        if (a.unit_out) a.unit_out[((int64_t)p * (a.b1 - a.b0) + (b - a.b0)) * a.S + U.s] = U.A;
                        if (U.Nb > 0 && U.A >= 0) {
                            unsigned v = div_by((unsigned)U.A * (unsigned)a.nbins, sNm[U.lb], sNl[U.lb]);
                            bin = v >= (unsigned)a.nbins ? a.nbins - 1 : (int)v;
                        }
                    }
                    hist_add_warp(sh, bin);
                }
                __syncthreads();
                const int nf = s_nf[c], nbk = s_nb[c];
                if (tid == 0) { s_nf[c ^ 1] = 0; s_nb[c ^ 1] = 0; }
                for (int k = 0; k < kOccRound; ++k) {
                    const int e = k * kThreads + tid;
                    int bin = -1;
                    if (e < nf || e >= kOccEntries - nbk) {
                        const int ue = (int)s_ent[0][e];
                        const int sig = (int)s_ent[1][e];
                        const int ba = (int)s_ent[2][e];
                        const float pe = __uint_as_float(s_ent[3][e]);
                        const Divisor dS = sdiv(s_Sm, s_Sl);
                        const int ke = (int)div_by((uint32_t)ue, dS.m, dS.l), ss = ue - ke * a.S;
                        const int lb = (GPDA_LPT && GPDA_LPT_OCC) ? (int)s_order[ke] : ke;
                        Rng r;
                        r.init(a.seed, pw, (uint32_t)(tb0 + lb), (uint32_t)ss);
                        r.blk = s_ent[4][e];
                        r.idx = (int)s_ent[5][e];
                        r.w0 = s_ent[6][e];
                        r.w1 = s_ent[7][e];
                        r.w2 = s_ent[8][e];
                        r.w3 = s_ent[9][e];
                        const int A = binom(r, sig, pe, lim, s_inv) + ba;
                        const int64_t b = tb0 + lb;
                        if (a.unit_out) a.unit_out[((int64_t)p * (a.b1 - a.b0) + (b - a.b0)) * a.S + ss] = A;
                        unsigned v = div_by((unsigned)A * (unsigned)a.nbins, sNm[lb], sNl[lb]);
                        bin = v >= (unsigned)a.nbins ? a.nbins - 1 : (int)v;
                    }
                    hist_add_warp(sh, bin);
                }
                __syncthreads();
            }
        }
        // photon mode: the binomial tables of the kernel launched before
        // this one (a no-op unless this launch is a programmatic dependent)
        if (kPhoton) asm volatile("griddepcontrol.wait;" ::: "memory");
        // photon mode: one dwell segment per step; a lane whose unit is
        // finished takes the tile's next unit at once
        Unit U;
        bool active = kPhoton && tid < units;
        if (active) unit_begin(U, tid, a.S, sdiv(s_Sm, s_Sl), tb0, sN, sT, a.seed, pw, GPDA_LPT ? s_order : nullptr);
        while (__any_sync(0xffffffffu, active)) {
            bool fin = false;
            int bin = -1;
            if (kPhoton && active) {
                fin = U.done;
                if (!fin) {
                    const float *offs = staged ? (s_ph + sOff[U.lb]) : (a.offsets + a.off_idx[tb0 + U.lb]);
                    fin = step_pho(U, sp, offs, a.gamma, a.ct, a.r0, s_bgc, lim, s_inv,
                                   a.bcdf + (size_t)p * sp.n * kTableRows,
                                   a.bguide + (size_t)p * sp.n * kTableRows);
                }
            }
            if (active) {
                if (fin) {
                    const int64_t b = tb0 + U.lb;
                    if (a.unit_out) a.unit_out[((int64_t)p * (a.b1 - a.b0) + (b - a.b0)) * a.S + U.s] = U.A;
                    if (U.Nb > 0 && U.A >= 0) {
#if GPDA_PR_BIN
                        bin = pr_bin(U.A, U.Nb, a.nbins);
#else
                        // a hardware division here: the shared divisors cost this
                        // loop a register spill
                        unsigned v = (unsigned)U.A * (unsigned)a.nbins / (unsigned)U.Nb;
                        bin = v >= (unsigned)a.nbins ? a.nbins - 1 : (int)v;
#endif
                    }
                }
            }
            // a few lanes finish per step: plain shared-memory atomics
            // (measured 1 % faster than the warp-aggregated form here)
            if (bin >= 0) atomicAdd(&sh[bin], 1u);
            // lanes whose unit finished take the next units of the tile
            const unsigned need = __ballot_sync(0xffffffffu, fin);
            if (need) {
                const int leader = __ffs(need) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(&s_next, __popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (fin) {
                    const int u = base + __popc(need & lt_mask);
                    active = u < units;
                    if (active) unit_begin(U, u, a.S, sdiv(s_Sm, s_Sl), tb0, sN, sT, a.seed, pw,
                                           GPDA_LPT ? s_order : nullptr);
                }
            }
        }
        __syncthreads();
        for (int i = tid; i < a.nbins; i += kThreads) {
            unsigned v = sh[i];
            if (v) atomicAdd(a.hist + (size_t)p * a.nbins + i, (unsigned long long)v);
        }
    }
    if (lim) atomicAdd(a.limit_hits, (unsigned long long)lim);
    if (a.chi2) last_cta_chi2(a);
}

__global__ void chi2_kernel(const unsigned long long *hist, const float *obs, int P, int nbins,
                            int left_pad, int S, int n_states, double *chi2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const unsigned long long *h = hist + (size_t)p * nbins;
    int effN = nbins - left_pad;
    double chi = 0.0;
    for (int i = left_pad; i < nbins; ++i) {
        if (h[i] > 0ull) {
            double mi = (double)h[i] / (double)S;
            double d = (double)obs[i] - mi;
            chi = chi + d * d / mi;
        } else {
            effN -= 1;
        }
    }
    chi2[p] = chi / (double)(effN - n_states * (n_states + 1));
}

// ---------------------------------------------------------------- ref-compat

// drawDisIdx over n weights read through an index map (gen_rand.cuh:35-50)
__device__ __forceinline__ int disidx_init(const float *p, int n, float pv) {
    float acc = 0.0f;
    for (int i = 0; i < n; ++i) {
        acc = acc + p[i];
        if (acc > pv) return i;
    }
    return n - 1;
}

// drawJ_Si2Sj (gen_rand.cuh:78-89): column si of P_i2j without the diagonal
__device__ __forceinline__ int disidx_jump(const float *Pi2j, int n, int si, float pv) {
    float acc = 0.0f;
    const float *col = Pi2j + si * n;
    int j = n - 2;
    for (int ii = 0; ii < n - 1; ++ii) {
        acc = acc + ((ii >= si) ? col[ii + 1] : col[ii]);
        if (acc > pv) { j = ii; break; }
    }
    return (j >= si) ? j + 1 : j;
}

// saturating float->int64 truncation, NaN -> 0
__device__ __forceinline__ int64_t f2i64(double v) {
    if (v != v) return 0;
    if (v >= 9.2233720368547758e18) return INT64_MAX;
    if (v <= -9.2233720368547758e18) return INT64_MIN;
    return (int64_t)v;
}

// draw_P_B_Tr (gen_rand.cuh:92-107) for one time bin
__device__ __forceinline__ float bg_clip(Rng &r, float tot, float tdiff, float rate, int &lim,
                                         const float *inv) {
    int sv = poisson(r, tdiff * rate, lim, inv);
    if ((float)sv <= tot) return (float)sv;
    return floorf(tot * r.u01());
}

__global__ void __launch_bounds__(kThreads) rc_kernel(const RcArgs a) {
    __shared__ DevParams sp;
    __shared__ unsigned int sh[kHistBins];
    __shared__ float s_inv[kInvTable];
    const int tid = threadIdx.x;
    if (tid < kInvTable) s_inv[tid] = tid > 0 ? 1.0f / (float)tid : 0.0f;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(a.params);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
        for (int i = tid; i < kParamWords; i += kThreads) dst[i] = src[i];
    }
    if (a.hist)
        for (int i = tid; i < a.nbins; i += kThreads) sh[i] = 0u;
    __syncthreads();
    const int64_t NN = (int64_t)a.nb * a.R;
    const int64_t tidx = (int64_t)blockIdx.x * kThreads + tid;
    int lim = 0;
    int bin = -1;
    if (tidx < NN) {
        const int lb = (int)(tidx / a.R);
        const uint32_t s = (uint32_t)(tidx - (int64_t)lb * a.R);
        const int64_t b = a.b0 + lb;
        Rng r;
        r.init(a.seed, a.pword, (uint32_t)b, s);
        const int n = sp.n;
        const int phCount = a.phCount[b];
        const int64_t *bad = a.burst_ad + a.istart[b];
        const int64_t *bdd = a.burst_dd + a.istart[b];
        const float Tb = a.T[b];
        const float clk = a.clk_p;
        const float gam = a.gamma, dea = a.de, cht = a.ct, r0 = a.r0;
        float F = 0.0f, mcE = 0.0f;
        int si = disidx_init(sp.pinit, n, r.u01());
        float spent = 0.0f;
        int64_t bin0 = a.start[b], bin1 = a.start[b];
        int binIdxStart = 0;
        for (int seg = 0; Tb > spent && seg < kMaxSeg; ++seg) {
            int sj = disidx_jump(sp.Pi2j, n, si, r.u01());
            float st = logf_(r.u01()) / (-sp.K[si * n + sj]);
            spent = spent + st;
            if (spent >= Tb) bin1 = a.stop[b];
            else bin1 = f2i64((double)((float)bin0 + spent / clk));
            int sdd = 0, sad = 0, f_id = 0, f_ia = 0;
            int ai = 0;
            for (int iinb = binIdxStart; iinb < phCount; ++iinb) {
                int64_t ddx = bdd[iinb], adx = bad[iinb];
                if (ddx >= bin1 || adx >= bin1 || iinb == phCount - 1) {
                    binIdxStart = iinb;
                    float f_if = (gam - cht) * (float)f_id + (1.0f - dea) * (float)f_ia;
                    float f_i;
                    F = F + f_if;
                    if ((double)a.bg_dd_rate < 1e-4) {
                        f_i = floorf((float)((double)f_if + 0.5));
                    } else {
                        float tdiff = (float)(bin1 - bin0) * clk;
                        float rf_ia = (1.0f - dea) * (float)f_ia;
                        float bga = bg_clip(r, rf_ia, tdiff, a.bg_ad_rate, lim, s_inv);
                        float rf_id = (gam - cht) * (float)f_id;
                        float bgd = bg_clip(r, rf_id, tdiff, a.bg_dd_rate, lim, s_inv);
                        f_i = floorf((float)((double)(f_if - bgd - bga) + 0.5));
                    }
                    float de = broaden(r, sp.E[si], r0, sp.V[si]);
                    ai = binom<false>(r, (int)f_i, de, lim, s_inv);
                    break;
                }
                if (ddx > 0) sdd = 1;
                if (adx > 0) sad = 1;
                if (sad && sdd) continue;
                if (sad) f_ia++;
                if (sdd) f_id++;
            }
            mcE = mcE + (float)ai;
            bin0 = bin1;
            si = sj;
        }
        if (F > 0.0f) mcE = mcE / F;
        else mcE = 0.0f;
        a.mcE[tidx] = mcE;
        double z = (double)mcE;
        if (z < 1.0 && z >= 0.0) bin = (int)(z * (double)a.nbins);
    }
    if (a.hist) {
        if (tidx < NN) hist_add(sh, bin);
        __syncthreads();
        for (int i = tid; i < a.nbins; i += kThreads) {
            unsigned v = sh[i];
            if (v) atomicAdd(a.hist + i, (unsigned long long)v);
        }
    }
    if (lim) atomicAdd(a.limit_hits, (unsigned long long)lim);
}

// ---------------------------------------------------------------- binomial tables

// Double-float arithmetic (a value is hi + lo, two FP32 numbers): error-free
// products by fmaf and error-free sums (Dekker, Knuth), about 44 significant
// bits. GB300 runs FP64 at a small fraction of its FP32 rate, so the tables are
// built on the FP32 pipes. Every step is an IEEE FP32 operation or fmaf, in a
// fixed order, so the host reproduces the rows bit for bit.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_fast_sum(float a, float b) {   // |a| >= |b|
    float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_fast_sum(p, e);
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e = e + (a.lo + b.lo);
    return df_fast_sum(s, e);
}
// x / y for float x, y > 0: one correction step
__device__ __forceinline__ DF df_div(float x, DF y) {
    float q = x / y.hi;
    DF qy = df_mul({q, 0.0f}, y);
    float r = (x - qy.hi) - qy.lo;
    return df_fast_sum(q, r / y.hi);
}
// x / y for double-float x, y > 0
__device__ __forceinline__ DF df_div2(DF x, DF y) {
    float q = x.hi / y.hi;
    DF qy = df_mul({q, 0.0f}, y);
    DF rem = df_add(x, {-qy.hi, -qy.lo});
    return df_fast_sum(q, rem.hi / y.hi);
}
// 1/k as a double-float, k >= 1
__device__ __forceinline__ DF df_recip(int k) {
    const float kf = (float)k;
    const float ih = 1.0f / kf;
    return df_fast_sum(ih, fmaf(-ih, kf, 1.0f) / kf);
}

// Row (p, s, n) of the photon-mode binomial tables, pp = bpp[s] <= 1/2,
// qq = 1 - pp, in double-float, one warp per row (kTableLanes lanes):
//  1. relative probabilities w(k) = pmf(k)/pmf(m) around the mode
//     m = min(floor((n+1) pp), n): upward w(k) = w(k-1) * ((n-k+1)/k) * (pp/qq),
//     downward w(k) = w(k+1) * ((k+1)/(n-k)) * (qq/pp). Each side is cut into
//     kTableLanes contiguous chunks; a lane forms the running product inside
//     its chunk, the chunk products are folded left to right across lanes,
//     and w(k) = (product of the earlier chunks) * (running product), rounded
//     to FP32 (far tails underflow harmlessly to 0);
//  2. the cumulative sums of the FP32 w over k = 0..n, chunked the same way
//     (chunk sums folded left to right; W = the fold of all chunks), and
//     cdf[k] = float(cum(k) * (1/W)) clamped to 1, cdf[n] = 1;
//  3. guide[j] = the first k with cdf[k] >= j/(n+1), by binary search.
// The operation order is fixed, so the host reproduces the rows bit for bit.
// Rows go longest first.
constexpr int kTableLanes = 32;
constexpr int kTableWarps = 8;
// 1: the guide entries' searches run four at a time per lane (below)
#ifndef GPDA_GUIDE_ILP
#define GPDA_GUIDE_ILP 1
#endif
// unroll factor of the chunk recurrences (their factors do not depend on
// the running product, so unrolled iterations overlap). Measured with the
// Monte-Carlo kernel it overlaps (photon_3state, the same bits): bisection
// one entry at a time 0.650 ms, four interleaved 0.646 ms, and with the
// recurrences unrolled by 4 0.640 ms (gpda_run_host 0.741 -> 0.731 ms).
#ifndef GPDA_TABLE_UNROLL
#define GPDA_TABLE_UNROLL 4
#endif
constexpr int kTableUnroll = GPDA_TABLE_UNROLL;

__device__ __forceinline__ DF df_shfl(DF v, int src) {
    return {__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

__global__ void __launch_bounds__(kTableLanes * kTableWarps)
binom_table_kernel(const DevParams *params, int P, int n_states, float *cdf_all, GuideEntry *guide_all) {
    __shared__ float s_hi[kTableWarps][kTableN + 1];
    __shared__ float s_lo[kTableWarps][kTableN + 1];
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    const int64_t rid = (int64_t)blockIdx.x * kTableWarps + wl;
    // the Monte-Carlo kernel that follows may start now (programmatic
    // dependent launch): it stages its first tile while the rows are built
    // and waits for them (griddepcontrol.wait) before its first draw
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int64_t total = (int64_t)P * n_states * (kTableN + 1);
    if (rid >= total) return;                       // whole warps leave together
    const int nn = kTableN - (int)(rid % (kTableN + 1));
    const int s = (int)((rid / (kTableN + 1)) % n_states);
    const int p = (int)(rid / ((int64_t)(kTableN + 1) * n_states));
    const size_t row = ((size_t)p * n_states + s) * kTableRows + (size_t)nn * (nn + 1) / 2;
    float *cdf = cdf_all + row;
    GuideEntry *guide = guide_all + row;
    float *hi = s_hi[wl];
    float *lo = s_lo[wl];
    const float pp = params[p].bpp[s];
    const DF qq = df_fast_sum(1.0f, -pp);
    const DF up = df_div(pp, qq);
    const DF down = df_div2(qq, {pp, 0.0f});
    int m = (int)floorf((float)(nn + 1) * pp);
    if (m > nn) m = nn;
    // 1a. upward, k = m+1 .. nn
    {
        const int len = nn - m;
        const int C = (len + kTableLanes - 1) / kTableLanes;
        const int k0 = m + 1 + lane * C;
        const int k1 = min(k0 + C - 1, nn);
        DF w = {1.0f, 0.0f};
#pragma unroll kTableUnroll
        for (int k = k0; k <= k1; ++k) {
            w = df_mul(w, df_mul(df_mul({(float)(nn - k + 1), 0.0f}, df_recip(k)), up));
            hi[k] = w.hi;
            lo[k] = w.lo;
        }
        DF Q = {1.0f, 0.0f};                        // product of the earlier chunks
        for (int i = 0; i < kTableLanes; ++i) {
            DF Pi = df_shfl(w, i);
            if (i < lane) Q = df_mul(Q, Pi);
        }
        for (int k = k0; k <= k1; ++k) {
            DF v = df_mul(Q, {hi[k], lo[k]});
            hi[k] = v.hi + v.lo;
        }
    }
    // 1b. downward, k = m-1 .. 0
    {
        const int len = m;
        const int C = (len + kTableLanes - 1) / kTableLanes;
        const int k0 = m - 1 - lane * C;
        const int k1 = max(k0 - C + 1, 0);
        DF w = {1.0f, 0.0f};
#pragma unroll kTableUnroll
        for (int k = k0; k >= k1; --k) {
            w = df_mul(w, df_mul(df_mul({(float)(k + 1), 0.0f}, df_recip(nn - k)), down));
            hi[k] = w.hi;
            lo[k] = w.lo;
        }
        DF Q = {1.0f, 0.0f};
        for (int i = 0; i < kTableLanes; ++i) {
            DF Pi = df_shfl(w, i);
            if (i < lane) Q = df_mul(Q, Pi);
        }
        for (int k = k0; k >= k1; --k) {
            DF v = df_mul(Q, {hi[k], lo[k]});
            hi[k] = v.hi + v.lo;
        }
    }
    if (lane == 0) hi[m] = 1.0f;
    __syncwarp();
    // 2. cumulative sums of the FP32 w, chunked over k = 0..nn
    const int C2 = (nn + 1 + kTableLanes - 1) / kTableLanes;
    const int c0 = lane * C2;
    const int c1 = min(c0 + C2, nn + 1);             // exclusive
    DF T = {0.0f, 0.0f};
    for (int k = c0; k < c1; ++k) T = df_add(T, {hi[k], 0.0f});
    DF E = {0.0f, 0.0f}, W = {0.0f, 0.0f};           // sum of the earlier chunks; of all
    for (int i = 0; i < kTableLanes; ++i) {
        DF Ti = df_shfl(T, i);
        if (i < lane) E = df_add(E, Ti);
        W = df_add(W, Ti);
    }
    const DF invW = df_div(1.0f, W);
    DF cum = E;
    for (int k = c0; k < c1; ++k) {
        cum = df_add(cum, {hi[k], 0.0f});
        DF v = df_mul(cum, invW);
        float c = v.hi + v.lo;
        c = (k == nn) ? 1.0f : (c < 1.0f ? c : 1.0f);
        lo[k] = c;
        cdf[k] = c;
    }
    __syncwarp();
    // 3. guide entries: first k with cdf[k] >= j/(n+1) (cdf[nn] = 1 ends every
    //    search) and its neighbouring cdf values
    const float gstep = 1.0f / (float)(nn + 1);
#if GPDA_GUIDE_ILP
    // kGuideGroup searches interleaved per lane, each with the row's fixed
    // number of steps and no branch: [base, base + len) holds the answer
    // (cdf[nn] = 1 >= t), and a probe below t moves base past it. The same
    // index as the bisection below, with independent load chains.
    constexpr int kGuideGroup = 4;
    for (int j0 = lane; j0 <= nn; j0 += kGuideGroup * kTableLanes) {
        float t[kGuideGroup];
        int base[kGuideGroup];
#pragma unroll
        for (int g = 0; g < kGuideGroup; ++g) {
            const int j = j0 + g * kTableLanes;
            t[g] = (float)(j <= nn ? j : nn) * gstep;
            base[g] = 0;
        }
        for (int len = nn + 1; len > 1;) {
            const int half = len >> 1;
#pragma unroll
            for (int g = 0; g < kGuideGroup; ++g)
                base[g] = (lo[base[g] + half - 1] < t[g]) ? base[g] + half : base[g];
            len -= half;
        }
#pragma unroll
        for (int g = 0; g < kGuideGroup; ++g) {
            const int j = j0 + g * kTableLanes;
            const int a = base[g];
            if (j <= nn) {
                const float cm = a > 0 ? lo[a - 1] : -1.0f;
                const float c1 = a < nn ? lo[a + 1] : 2.0f;
                guide[j] = make_uint4((unsigned)a, __float_as_uint(lo[a]), __float_as_uint(c1),
                                      __float_as_uint(cm));
            }
        }
    }
#else
    for (int j = lane; j <= nn; j += kTableLanes) {
        const float t = (float)j * gstep;
        int a = 0, b = nn;
        while (a < b) {
            int mid = (a + b) >> 1;
            if (lo[mid] >= t) b = mid; else a = mid + 1;
        }
        const float cm = a > 0 ? lo[a - 1] : -1.0f;
        const float c1 = a < nn ? lo[a + 1] : 2.0f;
        guide[j] = make_uint4((unsigned)a, __float_as_uint(lo[a]), __float_as_uint(c1), __float_as_uint(cm));
    }
#endif
}

// ---------------------------------------------------------------- burst-store validation

// One warp per burst: photon counts in range, durations finite and >= 0,
// off_idx consistent with N and inside [0, nph], offsets finite and sorted
// within the burst.
// Sets bits of *flag (1: N, 2: T, 4: off_idx, 8: offset not finite, 16: unsorted).
__global__ void validate_kernel(const int32_t *N, const float *T, const int64_t *off_idx,
                                const float *offsets, int64_t B, int64_t nph, unsigned int *flag) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned bad = 0u;
    for (int64_t b = warp; b < B; b += nwarps) {
        const int32_t nb = N[b];
        const float tb = T[b];
        if (lane == 0) {
            if (nb < 0 || nb > (1 << 21)) bad |= 1u;
            if (!(tb >= 0.0f) || !isfinite(tb)) bad |= 2u;
        }
        if (off_idx) {
            const int64_t lo = off_idx[b], hi = off_idx[b + 1];
            const bool inside = lo >= 0 && hi <= nph;
            if (lane == 0 && (hi - lo != (int64_t)nb || !inside)) bad |= 4u;
            if (hi - lo == (int64_t)nb && nb > 0 && inside) {
                for (int64_t i = lo + lane; i < hi; i += 32) {
                    const float x = offsets[i];
                    if (!isfinite(x)) bad |= 8u;
                    if (i > lo && x < offsets[i - 1]) bad |= 16u;
                }
            }
        }
    }
    if (bad) atomicOr(flag, bad);
}

// ---------------------------------------------------------------- launchers

cudaError_t launch_binom_tables(const DevParams *params, int P, int n_states, float *cdf,
                                GuideEntry *guide, cudaStream_t st) {
    const int64_t total = (int64_t)P * n_states * (kTableN + 1);
    if (total <= 0) return cudaSuccess;
    binom_table_kernel<<<(unsigned)((total + kTableWarps - 1) / kTableWarps), kTableLanes * kTableWarps, 0, st>>>(
        params, P, n_states, cdf, guide);
    return cudaGetLastError();
}

cudaError_t launch_validate(const int32_t *N, const float *T, const int64_t *off_idx,
                            const float *offsets, int64_t B, int64_t nph, unsigned int *flag,
                            int num_sms, cudaStream_t st) {
    int64_t warps = B;
    int64_t grid = std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)num_sms * 8);
    if (grid < 1) grid = 1;
    validate_kernel<<<(unsigned)grid, 256, 0, st>>>(N, T, off_idx, offsets, B, nph, flag);
    return cudaGetLastError();
}

const void *pda_kernel_fn(int mode) {
    return mode == 0 ? reinterpret_cast<const void *>(&pda_kernel<0>)
                     : reinterpret_cast<const void *>(&pda_kernel<1>);
}

cudaError_t launch_pda(int mode, const PdaArgs &a, int grid, size_t dyn_smem, cudaStream_t st) {
    if (mode != 0 && a.pdl) {
        // programmatic dependent launch after the binomial-table kernel
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = dyn_smem;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if (mode == kModePhotonDirect) return cudaLaunchKernelEx(&cfg, pda_kernel<2>, a);
        return cudaLaunchKernelEx(&cfg, pda_kernel<1>, a);
    }
    if (mode == 0) pda_kernel<0><<<grid, kThreads, dyn_smem, st>>>(a);
    else if (mode == kModePhotonDirect) pda_kernel<2><<<grid, kThreads, dyn_smem, st>>>(a);
    else pda_kernel<1><<<grid, kThreads, dyn_smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t pda_set_smem_limit(int mode, size_t dyn_smem) {
    if (mode == 0) return cudaFuncSetAttribute(pda_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem);
    if (mode == kModePhotonDirect)
        return cudaFuncSetAttribute(pda_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem);
    return cudaFuncSetAttribute(pda_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem);
}

cudaError_t pda_occupancy_blocks(int mode, size_t dyn_smem, int *blocks_per_sm) {
    if (mode == 0) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pda_kernel<0>, kThreads, dyn_smem);
    if (mode == kModePhotonDirect)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pda_kernel<2>, kThreads, dyn_smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pda_kernel<1>, kThreads, dyn_smem);
}

cudaError_t launch_chi2(const unsigned long long *hist, const float *obs, int P, int nbins,
                        int left_pad, int S, int n_states, double *chi2, cudaStream_t st) {
    int threads = 128;
    int grid = (P + threads - 1) / threads;
    chi2_kernel<<<grid, threads, 0, st>>>(hist, obs, P, nbins, left_pad, S, n_states, chi2);
    return cudaGetLastError();
}

cudaError_t launch_rc(const RcArgs &a, cudaStream_t st) {
    int64_t NN = (int64_t)a.nb * a.R;
    if (NN <= 0) return cudaSuccess;
    int64_t grid = (NN + kThreads - 1) / kThreads;
    rc_kernel<<<(unsigned)grid, kThreads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gpda
