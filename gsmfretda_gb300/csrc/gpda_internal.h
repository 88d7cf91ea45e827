// gpda_internal.h — types shared by the host engine and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gpda {

constexpr int kThreads = 256;       // threads per CTA of the MC kernels
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

struct PdaArgs {
    const float *bcdf;            // photon mode: CDF rows, P * n_states * kTableRows
    const uint16_t *bguide;       // photon mode: guide rows, same indexing
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

// kernel launchers (gpda_kernels.cu)
cudaError_t launch_pda(int mode, const PdaArgs &a, int grid, size_t dyn_smem, cudaStream_t st);
cudaError_t launch_chi2(const unsigned long long *hist, const float *obs, int P, int nbins,
                        int left_pad, int S, int n_states, double *chi2, cudaStream_t st);
cudaError_t launch_rc(const RcArgs &a, cudaStream_t st);
cudaError_t launch_binom_tables(const DevParams *params, int P, int n_states, float *cdf,
                                uint16_t *guide, cudaStream_t st);
cudaError_t launch_validate(const int32_t *N, const float *T, const int64_t *off_idx,
                            const float *offsets, int64_t B, unsigned int *flag, int num_sms,
                            cudaStream_t st);
cudaError_t pda_occupancy_blocks(int mode, size_t dyn_smem, int *blocks_per_sm);
cudaError_t pda_set_smem_limit(int mode, size_t dyn_smem);

// host parameter derivation (gpda_params.cpp)
int build_params(int n, const float *args, float gamma, float ct, bool need_pi, DevParams *out);

}  // namespace gpda
