// gpda_internal.h — types shared by the host engine and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gpda {

#ifndef GPDA_THREADS
#define GPDA_THREADS 256
#endif
constexpr int kThreads = GPDA_THREADS;   // threads per CTA of the MC kernels (a multiple of 64)
#ifndef GPDA_MIN_BLOCKS
#define GPDA_MIN_BLOCKS 4
#endif
constexpr int kMinBlocks = GPDA_MIN_BLOCKS;  // resident CTAs per SM the register budget targets
constexpr int kMaxTileBursts = 256; // bursts per work item
constexpr int kHistBins = 1024;     // shared-memory histogram capacity

// Per-parameter-set tables (host-derived, read into shared memory per work
// item). The pda part is the physical model, the rc part is the reference's
// genMatK / genP_i2j / genMatP output (src/eigenhelper.cpp:4-53).
struct alignas(16) DevParams {
    int32_t n;
    int32_t anyV;                 // any V[i] > 0 (distance broadening on)
    int32_t pad_[2];
    float E[8];
    float V[8];
    float eps[8];                 // apparent acceptor probability per state
    float kexit[8];               // total exit rate per state
    float inv_kexit[8];           // 1/kexit, +inf for absorbing states
    float init_cdf[8];            // cumulative stationary distribution
    float jump_cdf[64];           // [from*8 + to] cumulative jump probabilities
    float K[64];                  // rc: column-major n x n, leading dim n
    float Pi2j[64];               // rc: column-major jump probabilities
    float pinit[8];               // rc: unnormalised initial weights
    // binomial constants per state, p = eps: pp = min(p, 1-p),
    // logq = logf_(1-pp) (the device log, evaluated on the host), rr = pp/(1-pp)
    float bpp[8];
    float blogq[8];
    float brr[8];
    float pad2_[8];
};
static_assert(sizeof(DevParams) % 16 == 0, "DevParams must be 16-byte sized");
constexpr int kParamWords = (int)(sizeof(DevParams) / 4);

// Photon mode: Binomial(n, eps_s) for n <= kTableN (and V_s = 0) is drawn by
// inversion of a float CDF row built per (parameter set, state, n); a guide
// table of n+1 entries gives the starting index. Row (s, n) of parameter set
// p starts at (p * n_states + s) * kTableRows + n (n + 1) / 2.
#ifndef GPDA_TABLE_N
#define GPDA_TABLE_N 511
#endif
constexpr int kTableN = GPDA_TABLE_N;
constexpr int kTableRows = (kTableN + 1) * (kTableN + 2) / 2;   // entries per (parameter set, state)

// Photon-mode guide entry for cell j of a table row: the first k with
// cdf[k] >= j/(n+1) (x) and the bits of cdf[k-1] (w; -1 for k = 0), cdf[k]
// (y) and cdf[k+1] (z; 2 for k = n), so that one 16-byte load settles almost
// every draw.
using GuideEntry = uint4;

struct PdaArgs {
    const float *bcdf;            // photon mode: CDF rows, P * n_states * kTableRows
    const GuideEntry *bguide;     // photon mode: guide rows, same indexing
    const int32_t *N;
    const float *T;
    const int64_t *off_idx;
    const float *offsets;
    const DevParams *params;
    unsigned long long *hist;     // P x nbins
    int32_t *unit_out;            // optional [P][b1-b0][S]
    unsigned int *work;           // work-item counter, zeroed before launch
    unsigned long long *limit_hits;
    int64_t b0, b1;
    uint64_t seed;
    int32_t P;
    int32_t S;
    int32_t tile_b;               // bursts per work item
    int32_t ntiles;
    int32_t n_items;              // ntiles * P
    int32_t nbins;
    int32_t smem_cap;             // photon staging capacity (floats)
    uint32_t pbase;               // parameter-set word of the counter = pbase + p
    float gamma, ct, r0, bg_a, bg_d;
    // reduced chi-square in the kernel's last CTA (chi2 null: none)
    const float *obs;             // nbins observed counts
    double *chi2;                 // P
    unsigned int *done;           // CTAs finished, zeroed before launch
    // CTAs that count into *done: 0 = this launch's grid; launches over burst
    // ranges that share one counter give the sum of their grids
    uint32_t done_target;
    int32_t left_pad;
    int32_t n_states;
    // nonzero *abort_flag (the burst-store validation's): the kernel does nothing
    const unsigned int *abort_flag;
    // photon mode: non-null = every CTA first checks the bursts of its work
    // item as validate_kernel does (store of nph offsets), ORs the same error
    // bits into *vflag and skips an item that fails
    unsigned int *vflag;
    int64_t nph;
    // resident photon mode: nonzero = the offsets array is exactly
    // off_idx[b1] floats long (a caller's buffer, not the padded store), so
    // the staged span's last vector is read element by element up to the
    // tile's last photon instead of as one 16-byte load
    int32_t exact_offsets;
    // photon mode: launched as a programmatic dependent of the binomial-table
    // kernel just before it on the same stream (launch_pda)
    int32_t pdl;
    // direct reads (launch mode kModePhotonDirect, one parameter set, vflag
    // set): each CTA stages its tile from the caller's page-locked host
    // arrays hN, hT, hOffIdx, hOff (device-mapped; naturally aligned, hOff
    // to 16 bytes) instead of N, T, off_idx, offsets, checks it, and writes
    // it through to the store (wN, wT, wOffIdx, wOff: the arrays behind N,
    // T, off_idx, offsets) before it simulates, so the store is uploaded
    // when the launch ends.
    const int32_t *hN;
    const float *hT;
    const int64_t *hOffIdx;
    const float *hOff;
    int32_t *wN;
    float *wT;
    int64_t *wOffIdx;
    float *wOff;
};

struct RcArgs {
    const int64_t *start, *stop, *istart, *burst_ad, *burst_dd;
    const int32_t *phCount;
    const float *T;
    const DevParams *params;
    float *mcE;                   // [N][R]
    unsigned long long *hist;     // nbins (reference binning) or null
    unsigned long long *limit_hits;
    int64_t b0;
    int32_t nb;
    int32_t R;
    int32_t nbins;
    uint64_t seed;
    uint32_t pword;
    float clk_p, bg_ad_rate, bg_dd_rate;
    float gamma, de, ct, r0;
};

// kernel launchers (gpda_kernels.cu); launch mode kModePhotonDirect is photon
// mode with direct reads of host arrays (PdaArgs::hN)
constexpr int kModePhotonDirect = 2;
cudaError_t launch_pda(int mode, const PdaArgs &a, int grid, size_t dyn_smem, cudaStream_t st);
const void *pda_kernel_fn(int mode);   // the kernel launch_pda(mode) runs
cudaError_t launch_chi2(const unsigned long long *hist, const float *obs, int P, int nbins,
                        int left_pad, int S, int n_states, double *chi2, cudaStream_t st);
cudaError_t launch_rc(const RcArgs &a, cudaStream_t st);
cudaError_t launch_binom_tables(const DevParams *params, int P, int n_states, float *cdf,
                                GuideEntry *guide, cudaStream_t st);
cudaError_t launch_validate(const int32_t *N, const float *T, const int64_t *off_idx,
                            const float *offsets, int64_t B, int64_t nph, unsigned int *flag,
                            int num_sms, cudaStream_t st);
cudaError_t pda_occupancy_blocks(int mode, size_t dyn_smem, int *blocks_per_sm);
cudaError_t pda_set_smem_limit(int mode, size_t dyn_smem);

// host parameter derivation (gpda_params.cpp)
int build_params(int n, const float *args, float gamma, float ct, bool need_pi, DevParams *out);

// ---------------------------------------------------------------- expected histogram
// Differentiable expected-histogram form of the occupancy model. A unit's
// state skeleton (initial state, jump targets) is drawn from the fixed Philox
// uniforms under an anchor parameter set theta0; its dwells are
// -ln(u) / k_exit(s; theta) (reparameterised), and the skeleton carries the
// likelihood-ratio weight W = pi_theta(s0)/pi_theta0(s0) * prod
// P_theta(s_k|s_k-1)/P_theta0(s_k|s_k-1), so that the result is smooth in
// theta and W = 1 at theta = theta0. The binomial split is replaced by its
// bin masses.
constexpr int kExpMaxStates = 4;
constexpr int kExpMaxBins = 64;
constexpr int kExpGrad = 16;        // n + n(n-1) <= 16 gradient components
constexpr int kExpInvN = 4096;      // 1/k table for the binomial recurrence
struct ExpParams {                  // 128 words
    int32_t n, pad_[3];
    float E[4];
    float kexit[4];                 // theta: exit rates
    float inv_kexit[4];             // theta
    float init_cdf[4];              // theta0: cumulative stationary distribution
    float jump_cdf[16];             // theta0: cumulative jump probabilities [from*4 + to]
    float lw_init[4];               // ln pi_theta(s) - ln pi_theta0(s)
    float lw_jump[16];              // ln P_theta(to|from) - ln P_theta0(to|from)
    float pj[16];                   // P_theta(to|from)
    float dlnpi[48];                // d ln pi_theta(s) / d ln K_idx  [s*12 + idx]
    float pad2_[8];
};
static_assert(sizeof(ExpParams) == 128 * 4, "ExpParams layout");

struct ExpArgs {
    const int32_t *N;
    const float *T;
    const ExpParams *params;        // [P]
    const float *obs;               // [nbins]
    const float *inv;               // [kExpInvN] 1/k
    double *part;                   // [P][nblk][nbins]   forward partial sums
    double *hist;                   // [P][nbins]         expected counts (sum over samples)
    double *chi2;                   // [P]
    float *g;                       // [P][nbins]         d chi2 / d hist
    double *gpart;                  // [P][nblk][kExpGrad]
    double *grad;                   // [P][kExpGrad]      [dE(n), dlnK(n(n-1))]
    const double *dchi2;            // [P] upstream gradient, null = 1
    // mass tape (null: none): per unit, its bin masses P(bin) and the sums
    // x * P(x) over each bin, [p][2 nbins][units per set]; the forward writes
    // it and the adjoint reads it instead of walking the binomial again
    float *tape;
    int64_t units_p;                // B * S
    unsigned long long *limit_hits;
    int64_t B;
    int32_t S, P, nbins, left_pad, nblk, nblk_adj, n;
    uint64_t seed;
    float gamma, ct, bg_a, bg_d;
};

cudaError_t launch_exp_forward(const ExpArgs &a, cudaStream_t st);
cudaError_t launch_exp_adjoint(const ExpArgs &a, cudaStream_t st);
cudaError_t launch_exp_inv_table(float *inv, cudaStream_t st);
cudaError_t exp_grid(int n, int nbins, int P, int64_t units, int num_sms, bool tape, int *nblk_fwd,
                     int *nblk_adj);
int build_exp_params(int n, const float *theta, const float *anchor, float gamma, float ct,
                     ExpParams *out);

}  // namespace gpda
