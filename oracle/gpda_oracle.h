/*
 * gpda_oracle.h — CPU oracle for the photon-burst Monte-Carlo PDA path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker, never the product: only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * It restates, in plain C, the algorithm of gSMFRETda's Monte-Carlo hot path:
 *   - mc_kernel                      src/mc.cu:83-197   (the "ref-compat" mode)
 *   - drawDisIdx / drawTau / drawE /
 *     drawJ_Si2Sj / draw_P_B_Tr      src/gen_rand.cuh:35-107
 *   - rk_binomial (law only)         src/binom.cuh:135-188
 *   - genMatK / genP_i2j / genMatP   src/eigenhelper.cpp:4-53
 *   - parameter layout               src/mc.cu:790-800
 *   - mkhist + reduced chi-square    src/streamWorker.cpp:33-38, 184-206
 * and the physical PDA model ("pda" mode: occupancy-weighted E and
 * photon-by-photon assignment) on the same random counters.
 *
 * Random numbers come from Philox4x32-10 (Salmon et al., SC'11), keyed by the
 * seed and counted by (draw block, sample, burst, parameter set). Every
 * floating-point decision is made in FP32 with the same operation order as the
 * device kernels, so integer outputs (photon splits, histogram counts) are
 * bit-exact against the GPU. The same source (gpda_oracle_core.inc) is also
 * compiled as an FP64 transcription (libm log/exp/cos, double tables) on the
 * same counters; it agrees with the FP32 path wherever rounding does not move
 * a sampling decision and is compared in distribution elsewhere.
 *
 * Parity pinning: the reference ships no golden vectors (all of its tests are
 * statistical with non-deterministic seeds). The oracle is pinned against
 * (a) the reference's own binomial sampler compiled from src/binom.cuh
 * (oracle/_ref), (b) the reference's statistical test thresholds
 * (tests/GenRandTest.cu:170-350) and matrix invariants
 * (tests/ParamsTest.cpp:57-66), and (c) exact analytic limits.
 */
#ifndef GPDA_ORACLE_H
#define GPDA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXS 8

/* Model constants shared by both modes. */
typedef struct {
    int32_t nbins;      /* histogram bins on [0,1] */
    int32_t left_pad;   /* first bin counted in the chi-square (reference: 2) */
    float gamma;        /* pda: detection-efficiency ratio gamma */
    float crosstalk;    /* pda: donor->acceptor leakage alpha */
    float bg_d;         /* pda: donor-channel background rate (1/s) */
    float bg_a;         /* pda: acceptor-channel background rate (1/s) */
    float r0;           /* pda: Foerster radius used by distance broadening */
    /* ref-compat constants, mc_kernel defaults (src/mc.cu:89-91) */
    float rc_gamma;     /* 0.34 */
    float rc_de;        /* DexDirAem 0.08 */
    float rc_ct;        /* Dch2Ach 0.07 */
    float rc_r0;        /* 52 */
} orc_model;

/* Per-parameter-set tables, derived on the host from the reference layout
 * args = [E(n), K off-diagonals (n*n-n, row-major skipping the diagonal), V(n)]. */
typedef struct {
    int32_t n;
    int32_t pad_[3];
    float E[ORC_MAXS];
    float V[ORC_MAXS];
    float eps[ORC_MAXS];        /* apparent acceptor probability of a signal photon */
    float kexit[ORC_MAXS];      /* total exit rate of each state */
    float inv_kexit[ORC_MAXS];  /* 1/kexit, +inf for absorbing states */
    float init_cdf[ORC_MAXS];   /* cumulative stationary distribution */
    float jump_cdf[ORC_MAXS * ORC_MAXS]; /* [from*MAXS + to] cumulative jump probabilities */
    /* ref-compat tables, exactly as the reference builds them (float) */
    float K[ORC_MAXS * ORC_MAXS];    /* column-major n x n, K(i,j) = rate j->i */
    float Pi2j[ORC_MAXS * ORC_MAXS]; /* column-major n x n jump probabilities */
    float pinit[ORC_MAXS];           /* unnormalised initial weights (genMatP) */
} orc_params;

typedef struct {
    int64_t B;
    const int32_t *N;        /* photons per burst */
    const float *T;          /* burst duration (s) */
    const int64_t *off_idx;  /* B+1 prefix offsets into offsets[], or NULL */
    const float *offsets;    /* sorted arrival offsets in [0,T] (s), or NULL */
} orc_bursts;

typedef struct {
    int64_t B;
    const int64_t *start;    /* first photon clock tick of each burst */
    const int64_t *stop;     /* last photon clock tick */
    const int64_t *istart;   /* index of the first photon in burst_ad/dd */
    const int32_t *phCount;  /* photons per burst */
    const int64_t *burst_ad; /* mask_ad * times, per photon */
    const int64_t *burst_dd; /* mask_dd * times, per photon */
    const float *T;          /* burst duration (s) */
    float clk_p;             /* clock period (s) */
    float bg_ad_rate;
    float bg_dd_rate;
} orc_rc_bursts;

enum { ORC_MODE_OCCUPANCY = 0, ORC_MODE_PHOTON = 1 };

/* primitives */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float orc_logf(float x);
float orc_expf(float x);
float orc_cos2pif(float u);

/* draw `count` variates of one sampler; variate i uses the unit stream
 * (seed, param set 0, burst 0, sample i). kind: 0 binomial(n,p) 1 poisson(lam)
 * 2 exponential(rate=lam) 3 normal 4 u01  */
int orc_sample(int kind, uint64_t seed, int32_t n, float p, int64_t count, double *out);

/* photon-mode background pair (A, D) without clipping, `count` variates */
int orc_sample_bgpair(uint64_t seed, float bg_a, float bg_d, float dt, int64_t count, int32_t *A,
                      int32_t *D);

/* categorical draws (mode 0 pda cumulative, 1 drawDisIdx weights, 2 pda jump
 * row, 3 drawJ_Si2Sj column-major matrix); variate i uses sample word i */
int orc_sample_cat(uint64_t seed, int32_t mode, int32_t n, const float *w, int32_t from,
                   int64_t count, int32_t *out);

/* photon-mode binomial table row: cdf of Binomial(nn, pp), pp <= 1/2 */
void orc_binom_cdf_row(float pp, int32_t nn, float *out);

/* host-side parameter derivation (pda + ref-compat tables) */
int orc_build_params(int32_t n, const float *args, const orc_model *m, orc_params *out);

/* pda mode: units (p, b, s) for p < P, b in [b0,b1), s < S; args holds P
 * parameter vectors of n*(n+1) floats. hist: P*nbins counts (accumulated,
 * caller zeroes); unit_out (nullable): acceptor count A per unit, -1 where
 * N==0, layout [p][b-b0][s]. f64 != 0 selects the FP64 transcription.
 * Returns 0, or a negative error code. */
int orc_run_pda(const orc_bursts *bs, int32_t n, const float *args, int32_t P,
                const orc_model *m, int32_t mode, int32_t S, uint64_t seed,
                int64_t b0, int64_t b1, uint64_t *hist, int32_t *unit_out,
                int32_t nthreads, int32_t f64);

/* ref-compat mode (mc_kernel semantics): mcE (nullable) per unit, layout
 * [b-b0][s]; hist (nullable): nbins counts over [0,1) as the reference's
 * histogram. */
int orc_run_refcompat(const orc_rc_bursts *bs, int32_t n, const float *args,
                      const orc_model *m, int32_t S, uint64_t seed,
                      int64_t b0, int64_t b1, uint64_t *hist, float *mcE,
                      int32_t nthreads, int32_t f64);

/* reduced chi-square, FP64, sequential over bins (streamWorker.cpp:197-206) */
double orc_chi2(const uint64_t *hist, const float *ohist, int32_t nbins,
                int32_t left_pad, int32_t S, int32_t n_states);
/* the reference's own FP32 formula, for the shim's host-side path */
float orc_chi2_f32(const float *mhist, const float *ohist, int32_t nbins,
                   int32_t left_pad, int32_t R, int32_t n_states);
/* Boost regular-axis binning of float values on [0,1): inner bins only */
void orc_bin_values(const float *x, int64_t n, int32_t nbins, float *hist_out);

/* Differentiable expected histogram, occupancy form (no reference
 * counterpart; checker of gpda_expected_hist / _adjoint): FP64 except the
 * state skeleton and background counts, which are the FP32 mirror's draws
 * under `anchor` (NULL = params). hist: P*nbins expected counts summed over
 * samples; chi2: P; dE (P*n) and dlogK (P*n(n-1)), nullable, the gradient of
 * chi2 in E and ln K (parameter order). n <= 4, V = 0. */
int orc_expected(const orc_bursts *bs, int32_t n, const float *params, const float *anchor,
                 int32_t P, const orc_model *m, int32_t S, uint64_t seed, const float *obs,
                 double *hist, double *chi2, double *dE, double *dlogK, int32_t nthreads);

/* Replay of the reference kernel's recorded draws (mc_kernel, src/mc.cu:83-197,
 * run by oracle/mcref_harness.cu). One record per draw of a thread, in
 * order; tag & 0xff is the kind, tag >> 8 the binomial's n.
 *   U    d = the Sobol uniform (drawDisIdx, drawJ_Si2Sj, drawTau, the clip of draw_P_B_Tr)
 *   TAU  d = drawTau's value
 *   N    d = curand_normal's value (drawE)
 *   E    d = drawE's value
 *   P    i = curand_poisson's value, d = its mean (draw_P_B_Tr)
 *   B    i = rk_binomial's value, d = its p, tag >> 8 = its n */
enum { ORC_TAPE_U = 1, ORC_TAPE_TAU = 2, ORC_TAPE_N = 3, ORC_TAPE_E = 4, ORC_TAPE_P = 5,
       ORC_TAPE_B = 6 };
typedef struct {
    int32_t tag;
    int32_t i;
    double d;
} orc_tape_rec;
enum { ORC_REPLAY_EXACT = 0, ORC_REPLAY_DIFFERS = 1, ORC_REPLAY_TRUNCATED = 2,
       ORC_REPLAY_OFF_PATH = 3 };
typedef struct {
    int64_t units, exact, differs, truncated, off_path;
    int64_t lambda_mismatch;      /* Poisson means unlike the body's tdiff * rate */
    int64_t binom_arg_mismatch;   /* binomial (n, p) unlike the body's */
    int64_t tau_max_ulp;          /* oracle log vs the reference's drawTau */
    double e_max_abs;             /* oracle drawE formula vs the reference's */
} orc_replay_stats;
/* Thread t = b * R + s (R a power of two, as mc_kernel requires) has
 * tape_len[t] records at tape[t * cap]; tape_len[t] > cap means its tape
 * was cut. mcE_out / status_out (nullable) per thread. */
int orc_rc_replay(const orc_rc_bursts *bs, int32_t n, const float *args, const orc_model *m,
                  int32_t R, const orc_tape_rec *tape, const int32_t *tape_len, int32_t cap,
                  const float *ref_mcE, float *mcE_out, int8_t *status_out,
                  orc_replay_stats *stats);

/* The oracle's own Philox draws of mc_kernel units (seed and counters as
 * orc_run_refcompat uses them) written in the tape format: a self-check of
 * the replay, whose result must equal the recorded mcE_out bit for bit. */
int orc_rc_record(const orc_rc_bursts *bs, int32_t n, const float *args, const orc_model *m,
                  int32_t R, uint64_t seed, int32_t cap, orc_tape_rec *tape, int32_t *tape_len,
                  float *mcE_out);

#ifdef __cplusplus
}
#endif
#endif
