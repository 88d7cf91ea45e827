/*
 * gpda.h — C ABI of the GB300-native photon-burst Monte-Carlo PDA engine.
 *
 * Plain pointers and sizes only; every entry point returns an int status
 * (GPDA_OK = 0, negative on error) and never exits the process. A context is
 * bound to one device and driven by one host thread at a time.
 *
 * Two families of entry points:
 *
 *   gpda_mc_*  — the drop-in for the reference's `mc` engine object
 *                (src/mc.hpp:32-180, src/mc.cu:212-829). Same call sequence
 *                as gpuWorker::run (src/gpuWorker.cpp:69-82), same argument
 *                meaning and parameter layout; kernel semantics are mc_kernel's
 *                (src/mc.cu:83-197) with Philox counters instead of per-thread
 *                Sobol/xorshift states. include/gpda_mc.hpp wraps them in a C++
 *                class with the reference's member names.
 *
 *   gpda_*     — the physical PDA model (occupancy-weighted E, or photon-by-
 *                photon state assignment), fused on device with the
 *                proximity-ratio histogram and the reduced chi-square that
 *                streamWorker::run computes on the host
 *                (src/streamWorker.cpp:184-206).
 *
 * Parameter vectors use the reference layout (src/mc.cu:792-800):
 *   [E(n), K off-diagonals (n*n-n, row-major skipping the diagonal,
 *    K(i,j) = rate j->i as in genMatK, src/eigenhelper.cpp:4-22), V(n)].
 */
#ifndef GPDA_H
#define GPDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPDA_MAX_STATES 8
#define GPDA_MAX_BINS 1024

enum {
    GPDA_OK = 0,
    GPDA_ERR_ARG = -1,       /* invalid argument (sizes, ranges, NULL, unsorted offsets) */
    GPDA_ERR_SINGULAR = -2,  /* rate matrix has no unique stationary distribution */
    GPDA_ERR_CUDA = -3,      /* CUDA runtime error (message in gpda_last_error) */
    GPDA_ERR_NOMEM = -4,     /* device or pinned host allocation failed */
    GPDA_ERR_STATE = -5,     /* call out of order (e.g. run before upload) */
    GPDA_ERR_LIMIT = -6      /* a bounded device loop hit its limit (counted, see gpda_limit_hits) */
};

enum { GPDA_MODE_OCCUPANCY = 0, GPDA_MODE_PHOTON = 1 };

/* Model constants. Defaults: nbins 21, left_pad 2, gamma 1, crosstalk 0.05,
 * bg_d 1500/s, bg_a 800/s, r0 52; ref-compat constants are mc_kernel's
 * defaults gamma 0.34, DexDirAem 0.08, Dch2Ach 0.07, r0 52 (src/mc.cu:89-91). */
typedef struct {
    int32_t nbins;      /* histogram bins on [0,1] (<= GPDA_MAX_BINS) */
    int32_t left_pad;   /* first bin counted in the chi-square (main.cpp:155 passes 2) */
    float gamma;        /* detection-efficiency ratio */
    float crosstalk;    /* donor->acceptor leakage */
    float bg_d;         /* donor-channel background rate (1/s) */
    float bg_a;         /* acceptor-channel background rate (1/s) */
    float r0;           /* Foerster radius for distance broadening (V > 0) */
    float rc_gamma;
    float rc_de;
    float rc_ct;
    float rc_r0;
} gpda_model;

typedef struct gpda_ctx gpda_ctx;

/* Fill *m with the defaults above. */
void gpda_model_defaults(gpda_model *m);

/* Library version string. */
const char *gpda_version(void);

/* ---------------------------------------------------------------- pda */

/* Create a context on `device`. Replaces mc::mc (src/mc.cu:212-315): no RNG
 * state tables, no stream pool; one CUDA stream owned by the context. */
gpda_ctx *gpda_create(int32_t device, const gpda_model *m, int32_t *status);
void gpda_destroy(gpda_ctx *ctx);
/* Message of the last failed call on this context ("" if none). */
const char *gpda_last_error(const gpda_ctx *ctx);

/* Copy a burst set from host memory into HBM. Replaces mc::init_data_gpu
 * (src/mc.cu:456-521) for the pda model: N int32[B] photons per burst,
 * T float[B] durations (s), and for photon mode off_idx int64[B+1] prefix
 * offsets into offsets float[off_idx[B]] (sorted arrival offsets in [0,T],
 * seconds). off_idx/offsets may be NULL for occupancy mode. The store is
 * validated on the device (N in [0,2^21], T finite >= 0, off_idx consistent
 * with N, offsets finite and sorted per burst); GPDA_ERR_ARG if not. Pinned
 * host buffers make the copies asynchronous DMA. */
int32_t gpda_upload_bursts(gpda_ctx *ctx, const int32_t *N, const float *T,
                           const int64_t *off_idx, const float *offsets, int64_t B);

/* Observed histogram (nbins floats) used by the chi-square. Replaces the
 * per-thread mkhist of SgDivSr in streamWorker::run (src/streamWorker.cpp:62-67). */
int32_t gpda_set_observed(gpda_ctx *ctx, const float *ohist, int32_t nbins);

/* Bin observed proximity ratios with the reference's rule (Boost regular axis
 * on [0,1), inner bins only, src/streamWorker.cpp:33-38). Host-only helper. */
int32_t gpda_bin_values(const float *x, int64_t n, int32_t nbins, float *hist_out);

/* Derive the per-parameter-set tables the kernels use (stationary
 * distribution, jump CDFs, exit rates, apparent efficiencies) into a
 * caller buffer of gpda_params_size() floats. Host-only; exposed for tests.
 * Replaces genMatK/genP_i2j/genMatP (src/eigenhelper.cpp:4-53). */
int32_t gpda_params_size(void);
int32_t gpda_build_params(const gpda_model *m, int32_t n_states, const float *args, float *out);

/* One parameter set over bursts [b0,b1), `samples` MC draws per burst:
 * launch + fused histogram (+ chi-square if an observed histogram is set),
 * synchronous. hist_out: nbins uint64 counts (nullable); chi2_out (nullable).
 * Replaces set_params + run_kernel + the host histogram/chi-square
 * (src/mc.cu:567-587, src/streamWorker.cpp:184-206). */
int32_t gpda_run_plain(gpda_ctx *ctx, int32_t mode, int32_t n_states, const float *params,
                       int64_t b0, int64_t b1, int32_t samples, uint64_t seed,
                       uint64_t *hist_out, double *chi2_out);

/* A population of P parameter sets over all bursts in one persistent launch
 * (graph-captured). params: P*n(n+1) floats. hist_out: P*nbins (nullable),
 * chi2_out: P (nullable). Synchronous. */
int32_t gpda_run_batched(gpda_ctx *ctx, int32_t mode, int32_t P, int32_t n_states,
                         const float *params, int32_t samples, uint64_t seed,
                         uint64_t *hist_out, double *chi2_out);

/* Per-unit acceptor counts for parity checking: unit_out int32[P][b1-b0][samples]
 * (host), -1 where N == 0. Same random counters as the runs above. */
int32_t gpda_run_units(gpda_ctx *ctx, int32_t mode, int32_t P, int32_t n_states,
                       const float *params, int64_t b0, int64_t b1, int32_t samples,
                       uint64_t seed, int32_t *unit_out, uint64_t *hist_out);

/* Asynchronous form for resident-data measurement: parameters are staged
 * through pinned memory, results stay on the device until gpda_fetch. */
int32_t gpda_launch(gpda_ctx *ctx, int32_t mode, int32_t P, int32_t n_states,
                    const float *params, int64_t b0, int64_t b1, int32_t samples,
                    uint64_t seed);
int32_t gpda_fetch(gpda_ctx *ctx, uint64_t *hist_out, double *chi2_out);
/* Non-blocking completion check, like mc::streamQuery (src/mc.cu:595-601):
 * 1 = done, 0 = pending, <0 = error. */
int32_t gpda_query(gpda_ctx *ctx);
int32_t gpda_synchronize(gpda_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for event timing by callers. */
void *gpda_stream(gpda_ctx *ctx);
/* Kernel launches issued so far on this context. */
int64_t gpda_launch_count(const gpda_ctx *ctx);
/* Device time (ms, CUDA events on the context stream) of the most recent
 * Monte-Carlo kernel launch alone; waits for it. -1 if none. */
float gpda_kernel_ms(gpda_ctx *ctx);
/* Number of units whose segment/rejection loops hit their bound so far. */
int64_t gpda_limit_hits(gpda_ctx *ctx);

/* Upload and run in one call, the reference-facing path for host data (no
 * reference counterpart: there the copy and the kernel are separate steps).
 * The burst store goes to the device in `ranges` burst ranges (1..64) on a
 * copy stream, each range 1.5 times the size of the one before (range r ends
 * at burst B (1.5^(r+1) - 1) / (1.5^ranges - 1)). Each range is validated on the
 * device as gpda_upload_bursts validates (in photon mode with P <= 4 by the
 * simulating CTAs themselves, each checking its bursts before reading them),
 * and its Monte-Carlo kernel starts as soon as it has arrived, on its own
 * stream, so the copy overlaps the simulation and consecutive ranges'
 * kernels overlap. Every kernel reads the validation flag first and does
 * nothing once a range has been rejected. Results equal gpda_upload_bursts +
 * gpda_run_batched with the same arguments; the store stays uploaded for
 * later calls. A rejected store returns GPDA_ERR_ARG and leaves no store.
 * Direct reads: in photon mode with P = 1, when N, T, off_idx and offsets all
 * lie in page-locked host memory (cudaHostAlloc, cudaMallocHost,
 * cudaHostRegister; naturally aligned, offsets to 16 bytes), no copy is made
 * and `ranges` is not used: one kernel reads the arrays over the host link,
 * each CTA checking and staging its own bursts and writing them through to
 * the device store, with the same results, checks and errors. */
int32_t gpda_run_host(gpda_ctx *ctx, int32_t mode, int32_t P, int32_t n_states, const float *params,
                      const int32_t *N, const float *T, const int64_t *off_idx,
                      const float *offsets, int64_t B, int32_t samples, uint64_t seed,
                      int32_t ranges, uint64_t *hist_out, double *chi2_out);

/* ---- Captured batched launch and tile autotuning (no counterpart in the
 * reference, which launches one kernel per parameter set).
 *
 * gpda_graph_create captures one batched step over all uploaded bursts for
 * (mode, P, n_states, samples) as a CUDA graph: parameter copy, binomial
 * tables (photon mode), histogram reset, the Monte-Carlo kernel, the
 * chi-square (when an observed histogram is set) and the read-back into the
 * context's pinned buffers. gpda_graph_run replays it for P parameter vectors
 * and a seed, with results identical to gpda_run_batched with the same
 * arguments. Uploading bursts, setting the first observed histogram, a
 * larger launch on the context or gpda_autotune drop the graph (then
 * gpda_graph_run returns GPDA_ERR_STATE). */
int32_t gpda_graph_create(gpda_ctx *ctx, int32_t mode, int32_t P, int32_t n_states,
                          int32_t samples);
int32_t gpda_graph_run(gpda_ctx *ctx, const float *params, uint64_t seed, uint64_t *hist_out,
                       double *chi2_out);
/* Times the Monte-Carlo kernel for bursts per work item around the default
 * for (mode, samples) on these parameter vectors and keeps the fastest for
 * later launches of that shape on this context (tile_out, nullable). The
 * tile does not change any result. */
int32_t gpda_autotune(gpda_ctx *ctx, int32_t mode, int32_t P, int32_t n_states,
                      const float *params, int32_t samples, uint64_t seed, int32_t *tile_out);

/* ---- Differentiable expected histogram (occupancy model), no counterpart
 * in the reference: the gradient path of the parameter-server side.
 *
 * Each unit (parameter set p, burst b, dwell sample s < samples) draws its
 * state skeleton and background counts from the same Philox counters as the
 * sampled occupancy model (pword = p), with the skeleton taken from `anchor`
 * (NULL = params) and dwells -ln(u)/k_exit(state; params); the skeleton is
 * weighted by the likelihood ratio of params to anchor (1 when they are
 * equal). The binomial split is replaced by its bin masses, so hist_out
 * (P*nbins, nullable) holds expected counts summed over samples and chi2_out
 * (P) the reduced chi-square against the observed histogram in the same form
 * as gpda_run_plain. Parameter vectors as gpda_run_batched with V = 0;
 * n_states <= 4 and nbins <= 64 (GPDA_ERR_LIMIT beyond). Synchronous. */
int32_t gpda_expected_hist(gpda_ctx *ctx, int32_t P, int32_t n_states, const float *params,
                           const float *anchor, int32_t samples, uint64_t seed,
                           double *hist_out, double *chi2_out);
/* Gradient of dchi2[p] * chi2[p] (dchi2 NULL = 1) with respect to E (dE,
 * P*n) and to the natural logarithm of the off-diagonal rates in parameter
 * order (dlogK, P*n(n-1)), at the same arguments as the preceding
 * gpda_expected_hist on this context (the forward is re-run when they differ).
 * The derivative is pathwise for dwells and E and likelihood-ratio for the
 * skeleton. Synchronous. */
int32_t gpda_expected_hist_adjoint(gpda_ctx *ctx, int32_t P, int32_t n_states,
                                   const float *params, const float *anchor, int32_t samples,
                                   uint64_t seed, const double *dchi2, double *dE, double *dlogK);
/* The forward keeps, per unit, its bin masses and x-weighted bin masses in
 * device memory (4 * P * 2 * nbins * B * samples bytes) so that
 * the adjoint does not walk the binomial again, when the walk is longer than
 * the 2 nbins values a unit reads back (about 6.5 sqrt(mean N) > 2 nbins);
 * above `bytes` (default 16 GiB; 0 turns it off) the adjoint recomputes them
 * instead. Same results either way up to FP32 summation order. */
int32_t gpda_expected_set_tape_limit(gpda_ctx *ctx, int64_t bytes);
/* Forward and gradient (dchi2 = 1) in one call, one synchronisation. */
int32_t gpda_expected_grad(gpda_ctx *ctx, int32_t P, int32_t n_states, const float *params,
                           const float *anchor, int32_t samples, uint64_t seed, double *hist_out,
                           double *chi2_out, double *dE, double *dlogK);

/* No counterpart in the reference. For callers that cannot allocate device
 * memory where they evaluate parameter sets (e.g. a framework whose caching
 * allocator owns the device memory, or a loop that must not pay cudaMalloc's
 * implicit synchronisation): runs the same Monte-Carlo kernel as
 * gpda_run_batched over bursts [0,B) of caller-owned DEVICE arrays (N, T and,
 * for photon mode, off_idx/offsets, with the layout and values
 * gpda_upload_bursts accepts; not re-validated here) and writes P*nbins
 * counts into the DEVICE array hist (zeroed first); with ohist/chi2 (device,
 * nbins floats / P doubles) it also writes the reduced chi-square. params is
 * a HOST array of P*n(n+1) floats, read before the call returns (its tables
 * reach the device as kernel arguments). Arrays are naturally aligned and offsets
 * starts on a 16-byte boundary (GPDA_ERR_ARG otherwise); offsets may be
 * exactly off_idx[B] floats long. Allocates nothing: its scratch is a fixed
 * array of about 21 MB inside the library, held by every device that loads
 * it until exit, which limits P to 64, and in photon mode P*n_states to 8
 * (GPDA_ERR_ARG beyond). Runs asynchronously on `stream` (a cudaStream_t,
 * NULL = legacy default stream) on the current device. Calls share the
 * scratch: calls that overlap on the GPU race and must be serialised by the
 * caller. The first call on a device looks up the scratch address with that
 * device current; make it before any stream capture begins. Loop-limit hits
 * (gpda_limit_hits on a context) are not reported by this entry point. */
int32_t gpda_run_pda_noalloc(const gpda_model *m, int32_t mode, int32_t P, int32_t n_states,
                             const float *params, const int32_t *N, const float *T,
                             const int64_t *off_idx, const float *offsets, int64_t B,
                             int32_t samples, uint64_t seed, uint64_t *hist,
                             const float *ohist, double *chi2, void *stream);

/* ---------------------------------------------------------------- mc drop-in */

typedef struct gpda_mc gpda_mc;

/* mc::mc(devid, streamNum, debug, hdf5size, profiler) (src/mc.cu:212).
 * streamNum 0 picks 2 x asyncEngineCount as the reference does (mc.cu:61-66). */
gpda_mc *gpda_mc_create(int32_t devid, int32_t streamNum, uint8_t debug, uint64_t hdf5size,
                        int32_t profiler, int32_t *status);
void gpda_mc_destroy(gpda_mc *mc);
const char *gpda_mc_last_error(const gpda_mc *mc);
int32_t gpda_mc_stream_num(const gpda_mc *mc);            /* mc::getStreams (mc.cu:317) */
int32_t gpda_mc_sz_burst(const gpda_mc *mc);              /* mc::sz_burst */
int32_t gpda_mc_resample_times(const gpda_mc *mc);        /* mc::reSampleTimes (mc.hpp:87) */
/* mc::set_reSampleTimes (mc.cu:316); any value >= 1 is accepted (the
 * reference rounds down to a power of two because of its index shift). */
int32_t gpda_mc_set_resample_times(gpda_mc *mc, int32_t r);
/* Seed of the Philox key (the reference seeds curand with offset 1234). */
int32_t gpda_mc_set_seed(gpda_mc *mc, uint64_t seed);
/* Model constants of the ref-compat kernel (default: mc_kernel's). */
int32_t gpda_mc_set_model(gpda_mc *mc, const gpda_model *m);

/* mc::init_data_gpu (mc.cu:456-521): host arrays copied into HBM. */
int32_t gpda_mc_init_data_gpu(gpda_mc *mc, const int64_t *istart, const int64_t *start,
                              const int64_t *stop, const int32_t *phCount, int64_t n_bursts,
                              int64_t sz_tag, const int64_t *burst_ad, const int64_t *burst_dd,
                              const float *T_burst_duration, const float *SgDivSr,
                              float clk_p, float bg_ad_rate, float bg_dd_rate);
/* mc::set_nstates (mc.cu:723-781): returns the previous n of stream sid. */
int32_t gpda_mc_set_nstates(gpda_mc *mc, int32_t n, int32_t sid);
/* mc::set_params (mc.cu:790-829): 1 on success, 0 if nargs != n(n+1)
 * (the reference's genMatK size check, eigenhelper.cpp:5-8), <0 on error. */
int32_t gpda_mc_set_params(gpda_mc *mc, int32_t n, int32_t sid, const float *args, int32_t nargs);
/* mc::setBurstBd (mc.cu:523-565): returns N bursts of the range. */
int32_t gpda_mc_setBurstBd(gpda_mc *mc, int32_t cstart, int32_t cstop, int32_t sid);
/* mc::init_randstate (mc.cu:366-454): counter-based RNG needs no state
 * tables; records N. */
int32_t gpda_mc_init_randstate(gpda_mc *mc, int32_t N, int32_t sid);
/* mc::set_params_buff (mc.cu:783-788): the per-thread P_i2j scratch lives in
 * registers here; kept for the call sequence. */
int32_t gpda_mc_set_params_buff(gpda_mc *mc, int32_t oldS_n, int32_t N, int32_t sid);
/* mc::run_kernel (mc.cu:567-587): async launch of the ref-compat kernel on
 * stream sid and async copy of N*reSampleTimes floats into hmcE(sid); also
 * bins the values on device into the stream's histogram. */
int32_t gpda_mc_run_kernel(gpda_mc *mc, int32_t N, int32_t sid);
/* mc::streamQuery (mc.cu:595-601): 1 done, 0 pending. */
int32_t gpda_mc_streamQuery(gpda_mc *mc, int32_t sid);
/* mc::hmcE[sid] (mc.hpp:83): pinned host results of the last run_kernel. */
float *gpda_mc_hmcE(gpda_mc *mc, int32_t sid);
/* The 16 raw bytes of the device UUID into out[16] (mc::gpuuuid, filled by
 * showGPUsInfo, src/mc.cu:43-49; genuid formats them as hex). */
int32_t gpda_mc_gpu_uuid(gpda_mc *mc, char *out);
/* Histogram bins used by the fused on-device histogram (fretHistNum, -f). */
int32_t gpda_mc_set_hist_bins(gpda_mc *mc, int32_t nbins);
/* Device-binned histogram of the last completed run on stream sid (nbins
 * floats, reference binning rule). Call after streamQuery returned 1. */
int32_t gpda_mc_hist(gpda_mc *mc, int32_t sid, float *hist_out);

#ifdef __cplusplus
}
#endif
#endif
