// gpda_engine.cu — host engine and C ABI of the pda model (include/gpda.h).
//
// One context = one device + one CUDA stream + a burst store resident in HBM:
//   N        int32[B]        photons per burst
//   T        float[B]        burst duration (s)
//   off_idx  int64[B+1]      prefix offsets (photon mode)
//   offsets  float[sum N + pad] sorted arrival offsets, padded so that the
//                            kernels can read whole 16-byte vectors
// Per launch: P parameter-set tables (DevParams, staged through pinned
// memory), a P x nbins uint64 histogram, P chi-square values.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpda.h"
#include "gpda_internal.h"

using namespace gpda;

struct gpda_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t cstream = nullptr;      // copies of gpda_run_host
    cudaEvent_t params_ev = nullptr;
    std::vector<cudaEvent_t> range_ev;   // one per burst range of gpda_run_host
    std::vector<cudaStream_t> rstream;   // gpda_run_host: the ranges' kernels
    std::vector<cudaEvent_t> rjoin;      // end of each of those streams
    cudaEvent_t prep_ev = nullptr;       // gpda_run_host: parameters and tables ready
    gpda_model model{};
    int num_sms = 0;
    // burst store
    int64_t B = 0;
    int64_t nph = 0;
    double mean_N = 0.0;
    int32_t *dN = nullptr;
    float *dT = nullptr;
    int64_t *dOffIdx = nullptr;
    float *dOff = nullptr;
    int64_t cap_B = 0;
    int64_t cap_ph = 0;
    bool has_offsets = false;
    unsigned int *dFlag = nullptr;
    unsigned int *hFlag = nullptr;   // pinned
    cudaEvent_t k0 = nullptr, k1 = nullptr;  // around the last MC kernel
    bool timed = false;
    // observed histogram
    float *dObs = nullptr;
    bool has_obs = false;
    // launch scratch
    DevParams *dParams = nullptr;
    DevParams *hParams = nullptr;  // pinned
    int cap_P = 0;
    unsigned long long *dHist = nullptr;
    unsigned long long *hHist = nullptr;  // pinned
    double *dChi2 = nullptr;
    double *hChi2 = nullptr;  // pinned
    int cap_hist = 0;
    unsigned int *dWork = nullptr;
    unsigned long long *dLimit = nullptr;
    int32_t *dUnit = nullptr;
    size_t cap_unit = 0;
    float *dCdf = nullptr;          // photon-mode binomial tables
    GuideEntry *dGuide = nullptr;
    size_t cap_tab = 0;             // in (parameter set, state) tables
    // expected-histogram path
    ExpParams *dExp = nullptr;
    ExpParams *hExp = nullptr;      // pinned
    int cap_exp_P = 0;
    double *dExpPart = nullptr, *dExpGPart = nullptr;
    size_t cap_exp_part = 0;        // in P * nblk
    double *dExpHist = nullptr, *dExpChi2 = nullptr, *dExpGrad = nullptr, *dExpUp = nullptr;
    float *dExpG = nullptr;
    double *hExpOut = nullptr;      // pinned: chi2[P], hist[P][nbins], grad[P][16], up[P]
    int cap_exp_out = 0;            // in P
    float *dExpInv = nullptr;
    float *dTape = nullptr;         // mass tape of the last forward
    size_t cap_tape = 0;            // bytes
    int64_t tape_limit = (int64_t)16 << 30;
    bool exp_valid = false;         // the forward state matches exp_key
    std::vector<float> exp_key;
    int exp_P = 0, exp_nblk = 0;
    // autotuned bursts per work item: {mode, samples, tile}
    std::vector<std::array<int, 3>> tuned;
    // captured batched launch (gpda_graph_create / gpda_graph_run)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaGraphNode_t gnode = nullptr;     // the Monte-Carlo kernel node
    cudaKernelNodeParams gkp{};
    PdaArgs gargs{};
    void *gargv[1] = {nullptr};
    int g_mode = 0, g_P = 0, g_n = 0, g_S = 0, g_kernels = 0;
    bool g_chi2 = false;
    // last launch
    int last_P = 0;
    bool last_chi2 = false;
    int64_t launches = 0;
    int blocks_per_sm[3] = {0, 0, 0};   // resident CTAs per SM by launch mode
    std::string err;
};

namespace {

#ifndef GPDA_SMEM_CAP
#define GPDA_SMEM_CAP 8192
#endif
constexpr int kSmemCapFloats = GPDA_SMEM_CAP;  // photon staging (dynamic shared memory, floats)
constexpr int kMaxRanges = 64;        // burst ranges of gpda_run_host
constexpr int kRangeStreams = 4;      // streams its range kernels are spread over
constexpr int kFusedCheckSets = 4;    // photon run_host: CTAs check the store up to this P
constexpr double kRangeGrowth = 1.5;  // run_host: each burst range 1.5 x the one before
constexpr int kOffPad = 8;            // floats of padding behind the offsets array

int fail(gpda_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(gpda_ctx *c, cudaError_t e, const char *what) {
    return fail(c, GPDA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
    } while (0)

void free_dev(void *p) {
    if (p) cudaFree(p);
}

int check_model(const gpda_model *m) {
    if (!m) return -1;
    if (m->nbins < 1 || m->nbins > GPDA_MAX_BINS) return -1;
    if (m->left_pad < 0 || m->left_pad > m->nbins) return -1;
    if (!(m->gamma > 0.0f && std::isfinite(m->gamma))) return -1;
    if (!(m->crosstalk >= 0.0f && std::isfinite(m->crosstalk))) return -1;
    if (!(m->bg_d >= 0.0f && std::isfinite(m->bg_d))) return -1;
    if (!(m->bg_a >= 0.0f && std::isfinite(m->bg_a))) return -1;
    if (!(m->r0 > 0.0f && m->rc_r0 > 0.0f)) return -1;
    return 0;
}

void free_graph(gpda_ctx *c);

int ensure_scratch(gpda_ctx *c, int P) {
    int nb = c->model.nbins;
    if (P > c->cap_P || P * nb > c->cap_hist) free_graph(c);   // the graph holds these buffers
    if (P > c->cap_P) {
        free_dev(c->dParams);
        if (c->hParams) cudaFreeHost(c->hParams);
        c->dParams = nullptr;
        c->hParams = nullptr;
        c->cap_P = 0;
        CK(cudaMalloc(&c->dParams, sizeof(DevParams) * (size_t)P));
        CK(cudaMallocHost(&c->hParams, sizeof(DevParams) * (size_t)P));
        c->cap_P = P;
    }
    if (P * nb > c->cap_hist) {
        free_dev(c->dHist);
        free_dev(c->dChi2);
        if (c->hHist) cudaFreeHost(c->hHist);
        if (c->hChi2) cudaFreeHost(c->hChi2);
        c->dHist = nullptr; c->dChi2 = nullptr; c->hHist = nullptr; c->hChi2 = nullptr;
        c->cap_hist = 0;
        CK(cudaMalloc(&c->dHist, sizeof(unsigned long long) * (size_t)P * nb));
        CK(cudaMalloc(&c->dChi2, sizeof(double) * (size_t)P));
        CK(cudaMallocHost(&c->hHist, sizeof(unsigned long long) * (size_t)P * nb));
        CK(cudaMallocHost(&c->hChi2, sizeof(double) * (size_t)P));
        c->cap_hist = P * nb;
    }
    return GPDA_OK;
}

// Bursts per work item for a launch over nb bursts and P parameter sets: the
// tuned value for (mode, S), else ~GPDA_TILE_UNITS units (photon mode: tiles
// whose offsets fit the shared-memory staging). Occupancy mode then caps it
// so that the launch has at least 4 work items per resident CTA (a single
// parameter set otherwise leaves CTAs idle at the end), down to one round of
// kThreads units. Photon mode keeps its tiles: there a lane takes the tile's
// next unit as soon as its own is done, and tiles of fewer units per lane
// measured slower than the end-of-launch imbalance they remove. Direct reads
// of host arrays (gpda_run_host) take ~GPDA_TILE_UNITS_DIRECT units and no
// tuned value: each CTA's staging there waits on the host link, and smaller
// tiles spread those waits. Measured on photon_3state (100 samples per
// burst): 3,200 units (32 bursts) against 2,048 (21), resident kernel 0.652
// -> 0.642 ms, direct reads 0.742 -> 0.752 ms per call; occupancy mode on 64
// parameter sets, untuned, 15.60 -> 15.04 ms. The same bits at any tile.
#ifndef GPDA_TILE_UNITS
#define GPDA_TILE_UNITS 3200
#endif
#ifndef GPDA_TILE_UNITS_DIRECT
#define GPDA_TILE_UNITS_DIRECT 2048
#endif
// photon mode: launch the Monte-Carlo kernel as a programmatic dependent of
// the binomial-table kernel (1) or after it completes (0)
#ifndef GPDA_PDL
#define GPDA_PDL 1
#endif

int tile_bursts(const gpda_ctx *c, int mode, int S, int64_t nb, int P, bool direct = false) {
    int tb = 0;
    for (const auto &t : c->tuned)
        if (!direct && t[0] == mode && t[1] == S) tb = t[2];
    if (tb == 0) {
        tb = ((direct ? GPDA_TILE_UNITS_DIRECT : GPDA_TILE_UNITS) + S - 1) / S;
        if (mode == GPDA_MODE_PHOTON && c->mean_N > 0.0) {
            int fit = (int)(0.6 * kSmemCapFloats / c->mean_N);
            tb = std::min(tb, std::max(fit, 1));
        }
    }
    if (mode == GPDA_MODE_OCCUPANCY) {
        const int64_t slots = 4 * (int64_t)c->num_sms * std::max(1, c->blocks_per_sm[mode]);
        const int64_t cap = std::max<int64_t>(nb * (int64_t)std::max(P, 1) / slots, (kThreads + S - 1) / S);
        if (cap < tb) tb = (int)cap;
    }
    return std::max(1, std::min(tb, kMaxTileBursts));
}

void free_graph(gpda_ctx *c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->gnode = nullptr;
    c->g_P = 0;
}

// Parameters to the device, photon tables, histogram reset (stream-ordered).
int prepare_launch(gpda_ctx *c, int mode, int P, int n, const float *params) {
    int rc = ensure_scratch(c, P);
    if (rc) return rc;
    // the pinned parameter staging may still be read by the previous copy
    CK(cudaEventSynchronize(c->params_ev));
    const size_t stride = (size_t)n * (n + 1);
    for (int p = 0; p < P; ++p) {
        int r = build_params(n, params + stride * p, c->model.gamma, c->model.crosstalk, true, &c->hParams[p]);
        if (r == -2) return fail(c, GPDA_ERR_SINGULAR, "rate matrix has no unique stationary distribution (parameter set " + std::to_string(p) + ")");
        if (r != 0) return fail(c, GPDA_ERR_ARG, "invalid parameter vector " + std::to_string(p));
    }
    const int nbins = c->model.nbins;
    CK(cudaMemcpyAsync(c->dParams, c->hParams, sizeof(DevParams) * P, cudaMemcpyHostToDevice, c->stream));
    CK(cudaEventRecord(c->params_ev, c->stream));
    // resets first, then the tables right before the Monte-Carlo kernel,
    // which runs as their programmatic dependent (GPDA_PDL); the kernel's
    // events enclose both
    CK(cudaMemsetAsync(c->dHist, 0, sizeof(unsigned long long) * (size_t)P * nbins, c->stream));
    CK(cudaMemsetAsync(c->dWork, 0, 2 * sizeof(unsigned int), c->stream));
    CK(cudaEventRecord(c->k0, c->stream));
    if (mode == GPDA_MODE_PHOTON) {
        const size_t ntab = (size_t)P * n;
        if (ntab > c->cap_tab) {
            CK(cudaStreamSynchronize(c->stream));
            free_graph(c);
            free_dev(c->dCdf);
            free_dev(c->dGuide);
            c->dCdf = nullptr; c->dGuide = nullptr; c->cap_tab = 0;
            CK(cudaMalloc(&c->dCdf, sizeof(float) * kTableRows * ntab));
            CK(cudaMalloc(&c->dGuide, sizeof(GuideEntry) * kTableRows * ntab));
            c->cap_tab = ntab;
        }
        CK(launch_binom_tables(c->dParams, P, n, c->dCdf, c->dGuide, c->stream));
        c->launches += 1;
    }
    c->last_P = P;
    c->last_chi2 = false;
    return GPDA_OK;
}

// Arguments and grid of the Monte-Carlo kernel over bursts [b0, b1) of all P
// parameter sets, adding into the histogram; with_chi2: the last CTA also
// writes the chi-square; abort_flag: see PdaArgs. The caller zeroes *work and
// *done (c->dWork[0] and [1] unless it sets others).
int range_args(gpda_ctx *c, int mode, int P, int n, int64_t b0, int64_t b1, int S, uint64_t seed,
               int32_t *dUnit, bool with_chi2, const unsigned int *abort_flag, PdaArgs &a,
               int &grid) {
    a = PdaArgs{};
    a.bcdf = c->dCdf;
    a.bguide = c->dGuide;
    a.N = c->dN;
    a.T = c->dT;
    a.off_idx = c->dOffIdx;
    a.offsets = c->dOff;
    a.params = c->dParams;
    a.hist = c->dHist;
    a.unit_out = dUnit;
    a.work = c->dWork;
    a.limit_hits = c->dLimit;
    a.b0 = b0;
    a.b1 = b1;
    a.seed = seed;
    a.P = P;
    a.S = S;
    a.tile_b = tile_bursts(c, mode, S, b1 - b0, P);
    int64_t ntiles = (b1 - b0 + a.tile_b - 1) / a.tile_b;
    if (ntiles * P > (int64_t)INT32_MAX) return fail(c, GPDA_ERR_ARG, "too many work items");
    a.ntiles = (int)ntiles;
    a.n_items = (int)(ntiles * P);
    a.nbins = c->model.nbins;
    a.smem_cap = kSmemCapFloats;
    a.pbase = 0u;
    a.gamma = c->model.gamma;
    a.ct = c->model.crosstalk;
    a.r0 = c->model.r0;
    a.bg_a = c->model.bg_a;
    a.bg_d = c->model.bg_d;
    if (with_chi2) {        // chi-square in the kernel's last CTA
        a.obs = c->dObs;
        a.chi2 = c->dChi2;
        a.done = c->dWork + 1;
        a.left_pad = c->model.left_pad;
        a.n_states = n;
    }
    a.abort_flag = abort_flag;
    grid = (int)std::min<int64_t>(a.n_items, (int64_t)c->num_sms * c->blocks_per_sm[mode]);
    return GPDA_OK;
}

// The Monte-Carlo kernel over bursts [b0, b1) on the context stream (see
// range_args), timed by the context's events.
int enqueue_range(gpda_ctx *c, int mode, int P, int n, int64_t b0, int64_t b1, int S,
                  uint64_t seed, int32_t *dUnit, bool with_chi2, const unsigned int *abort_flag) {
    if (b1 == b0) return GPDA_OK;
    PdaArgs a;
    int grid = 0;
    int rc = range_args(c, mode, P, n, b0, b1, S, seed, dUnit, with_chi2, abort_flag, a, grid);
    if (rc) return rc;
    size_t dyn = (mode == GPDA_MODE_PHOTON) ? sizeof(float) * kSmemCapFloats : 0;
    a.pdl = (mode == GPDA_MODE_PHOTON && GPDA_PDL) ? 1 : 0;   // right after the tables
    CK(launch_pda(mode, a, grid, dyn, c->stream));
    CK(cudaEventRecord(c->k1, c->stream));
    c->timed = true;
    c->launches += 1;
    c->last_chi2 = with_chi2;
    return GPDA_OK;
}

// The device address of a host array [p, p + bytes) in page-locked memory
// (cudaHostAlloc, cudaMallocHost, cudaHostRegister), checked at both ends;
// null for any other memory.
const void *mapped_host(const void *p, size_t bytes) {
    if (!p || bytes == 0) return nullptr;
    cudaPointerAttributes a0{}, a1{};
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    const char *q = static_cast<const char *>(p) + (bytes - 1);
    if (cudaPointerGetAttributes(&a1, q) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
        return nullptr;
    if (static_cast<const char *>(a1.devicePointer) - static_cast<const char *>(a0.devicePointer) !=
        (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

// End of a gpda_run_host call: the store's check flag, histogram and
// chi-square to the host (one synchronisation), then the flag's verdict.
int host_run_results(gpda_ctx *c, int P, uint64_t *hist_out, double *chi2_out) {
    const int nb = c->model.nbins;
    CK(cudaMemcpyAsync(c->hFlag, c->dFlag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    if (hist_out) CK(cudaMemcpyAsync(c->hHist, c->dHist, sizeof(unsigned long long) * (size_t)P * nb, cudaMemcpyDeviceToHost, c->stream));
    if (chi2_out && c->has_obs) CK(cudaMemcpyAsync(c->hChi2, c->dChi2, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    unsigned f = *c->hFlag;
    if (f) {
        c->B = 0;
        std::string why;
        if (f & 1u) why += " N outside [0, 2^21];";
        if (f & 2u) why += " T not finite and >= 0;";
        if (f & 4u) why += " off_idx inconsistent with N;";
        if (f & 8u) why += " offset not finite;";
        if (f & 16u) why += " offsets not sorted within a burst;";
        return fail(c, GPDA_ERR_ARG, "burst store rejected:" + why);
    }
    if (hist_out) std::memcpy(hist_out, c->hHist, sizeof(uint64_t) * (size_t)P * nb);
    if (chi2_out) {
        if (c->has_obs) std::memcpy(chi2_out, c->hChi2, sizeof(double) * P);
        else for (int p = 0; p < P; ++p) chi2_out[p] = NAN;
    }
    return GPDA_OK;
}

int do_launch(gpda_ctx *c, int mode, int P, int n, const float *params, int64_t b0, int64_t b1,
              int S, uint64_t seed, int32_t *dUnit) {
    if (mode != GPDA_MODE_OCCUPANCY && mode != GPDA_MODE_PHOTON) return fail(c, GPDA_ERR_ARG, "mode");
    if (P < 1 || n < 1 || n > GPDA_MAX_STATES || S < 1 || !params) return fail(c, GPDA_ERR_ARG, "P, n_states, samples or params");
    if (c->B == 0 || !c->dN) return fail(c, GPDA_ERR_STATE, "no bursts uploaded");
    if (b0 < 0 || b1 < b0 || b1 > c->B) return fail(c, GPDA_ERR_ARG, "burst range");
    if (mode == GPDA_MODE_PHOTON && !c->has_offsets) return fail(c, GPDA_ERR_STATE, "photon mode needs arrival offsets");
    if ((int64_t)(b1 - b0) * S > (int64_t)INT32_MAX) return fail(c, GPDA_ERR_ARG, "too many units per parameter set");
    CK(cudaSetDevice(c->device));
    int rc = prepare_launch(c, mode, P, n, params);
    if (rc) return rc;
    return enqueue_range(c, mode, P, n, b0, b1, S, seed, dUnit, c->has_obs, nullptr);
}

// ---------------------------------------------------------------- expected histogram

int exp_prepare(gpda_ctx *c, int P, int n, const float *params, const float *anchor, int S,
                uint64_t seed, ExpArgs &a) {
    if (P < 1 || n < 1 || S < 1 || !params) return fail(c, GPDA_ERR_ARG, "P, n_states, samples or params");
    if (n > kExpMaxStates) return fail(c, GPDA_ERR_LIMIT, "expected histogram: at most 4 states");
    if (c->model.nbins > kExpMaxBins) return fail(c, GPDA_ERR_LIMIT, "expected histogram: at most 64 bins");
    if (c->B == 0 || !c->dN) return fail(c, GPDA_ERR_STATE, "no bursts uploaded");
    if (!c->has_obs) return fail(c, GPDA_ERR_STATE, "no observed histogram");
    if (c->B * (int64_t)S > (int64_t)1 << 40) return fail(c, GPDA_ERR_ARG, "too many units");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));   // pinned staging and scratch are free
    const int nb = c->model.nbins;
    // The mass tape: per unit 2 nbins floats, when it fits under the limit and
    // the binomial walk it replaces is longer than the tape entries a unit
    // reads back (a walk covers about 13 standard deviations of the signal
    // count, about 6.5 sqrt(N) terms at p = 1/2). Measured: 20,000 bursts of
    // mean N 150 with 21 bins, 0.57 -> 0.46 ms a step with the tape; 1e6
    // bursts of mean N 67 with 41 bins, 12.9 -> 13.9 ms a step with it.
    const int64_t units_p = c->B * (int64_t)S;
    const double tape_bytes = 4.0 * P * 2.0 * nb * (double)units_p;
    bool tape = tape_bytes <= (double)c->tape_limit && 6.5 * std::sqrt(c->mean_N) > 2.0 * nb;
    if (tape && (size_t)tape_bytes > c->cap_tape) {
        free_dev(c->dTape);
        c->dTape = nullptr;
        c->cap_tape = 0;
        if (cudaMalloc(&c->dTape, (size_t)tape_bytes) == cudaSuccess) c->cap_tape = (size_t)tape_bytes;
        else { cudaGetLastError(); c->dTape = nullptr; tape = false; }   // walk the binomial again
    }
    int nblk = 1, nblk_adj = 1;
    CK(exp_grid(n, nb, P, units_p, c->num_sms, tape, &nblk, &nblk_adj));
    if (!c->dExpInv) {
        CK(cudaMalloc(&c->dExpInv, sizeof(float) * kExpInvN));
        CK(launch_exp_inv_table(c->dExpInv, c->stream));
        c->launches += 1;
    }
    if (P > c->cap_exp_out) {
        free_dev(c->dExp); free_dev(c->dExpHist); free_dev(c->dExpChi2); free_dev(c->dExpGrad);
        free_dev(c->dExpUp); free_dev(c->dExpG);
        if (c->hExp) cudaFreeHost(c->hExp);
        if (c->hExpOut) cudaFreeHost(c->hExpOut);
        c->dExp = nullptr; c->dExpHist = nullptr; c->dExpChi2 = nullptr; c->dExpGrad = nullptr;
        c->dExpUp = nullptr; c->dExpG = nullptr; c->hExp = nullptr; c->hExpOut = nullptr;
        c->cap_exp_out = 0;
        CK(cudaMalloc(&c->dExp, sizeof(ExpParams) * P));
        CK(cudaMallocHost(&c->hExp, sizeof(ExpParams) * P));
        CK(cudaMalloc(&c->dExpHist, sizeof(double) * (size_t)P * kExpMaxBins));
        CK(cudaMalloc(&c->dExpChi2, sizeof(double) * P));
        CK(cudaMalloc(&c->dExpGrad, sizeof(double) * (size_t)P * kExpGrad));
        CK(cudaMalloc(&c->dExpUp, sizeof(double) * P));
        CK(cudaMalloc(&c->dExpG, sizeof(float) * (size_t)P * kExpMaxBins));
        CK(cudaMallocHost(&c->hExpOut, sizeof(double) * (size_t)P * (2 + kExpMaxBins + kExpGrad)));
        c->cap_exp_out = P;
    }
    const size_t parts = (size_t)P * std::max(nblk, nblk_adj);
    if (parts > c->cap_exp_part) {
        free_dev(c->dExpPart); free_dev(c->dExpGPart);
        c->dExpPart = nullptr; c->dExpGPart = nullptr; c->cap_exp_part = 0;
        CK(cudaMalloc(&c->dExpPart, sizeof(double) * parts * kExpMaxBins));
        CK(cudaMalloc(&c->dExpGPart, sizeof(double) * parts * kExpGrad));
        c->cap_exp_part = parts;
    }
    const size_t stride = (size_t)n * (n + 1);
    for (int p = 0; p < P; ++p) {
        const float *th = params + stride * p;
        const float *an = anchor ? anchor + stride * p : th;
        int r = build_exp_params(n, th, an, c->model.gamma, c->model.crosstalk, &c->hExp[p]);
        if (r == -2) return fail(c, GPDA_ERR_SINGULAR, "rate matrix has no unique stationary distribution (parameter set " + std::to_string(p) + ")");
        if (r != 0) return fail(c, GPDA_ERR_ARG, "invalid parameter vector " + std::to_string(p) + " (the expected form needs V = 0)");
    }
    CK(cudaMemcpyAsync(c->dExp, c->hExp, sizeof(ExpParams) * P, cudaMemcpyHostToDevice, c->stream));
    a = ExpArgs{};
    a.N = c->dN;
    a.T = c->dT;
    a.params = c->dExp;
    a.obs = c->dObs;
    a.inv = c->dExpInv;
    a.part = c->dExpPart;
    a.hist = c->dExpHist;
    a.chi2 = c->dExpChi2;
    a.g = c->dExpG;
    a.gpart = c->dExpGPart;
    a.grad = c->dExpGrad;
    a.dchi2 = nullptr;
    a.tape = tape ? c->dTape : nullptr;
    a.units_p = units_p;
    a.limit_hits = c->dLimit;
    a.B = c->B;
    a.S = S;
    a.P = P;
    a.nbins = nb;
    a.left_pad = c->model.left_pad;
    a.nblk = nblk;
    a.nblk_adj = nblk_adj;
    a.n = n;
    a.seed = seed;
    a.gamma = c->model.gamma;
    a.ct = c->model.crosstalk;
    a.bg_a = c->model.bg_a;
    a.bg_d = c->model.bg_d;
    return GPDA_OK;
}

std::vector<float> exp_make_key(int P, int n, const float *params, const float *anchor, int S,
                                uint64_t seed) {
    const size_t m = (size_t)P * n * (n + 1);
    std::vector<float> k;
    k.reserve(2 * m + 6);
    k.push_back((float)P);
    k.push_back((float)n);
    k.push_back((float)S);
    float sw[2];
    std::memcpy(sw, &seed, 8);
    k.push_back(sw[0]);
    k.push_back(sw[1]);
    k.insert(k.end(), params, params + m);
    k.push_back(anchor ? 1.0f : 0.0f);
    if (anchor) k.insert(k.end(), anchor, anchor + m);
    return k;
}

bool exp_same_key(const std::vector<float> &a, const std::vector<float> &b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), sizeof(float) * a.size()) == 0;
}

// forward + (optionally) adjoint; outputs copied once at the end
int exp_run(gpda_ctx *c, int P, int n, const float *params, const float *anchor, int S,
            uint64_t seed, double *hist_out, double *chi2_out, bool adjoint, const double *dchi2,
            double *dE, double *dlogK) {
    auto key = exp_make_key(P, n, params, anchor, S, seed);
    ExpArgs a;
    bool need_fwd = !(adjoint && c->exp_valid && exp_same_key(key, c->exp_key)) || hist_out || chi2_out;
    int rc = exp_prepare(c, P, n, params, anchor, S, seed, a);
    if (rc) { c->exp_valid = false; return rc; }
    const int nb = c->model.nbins;
    double *hc = c->hExpOut;                                 // chi2[P]
    double *hh = hc + P;                                     // hist[P][nbins]
    double *hg = hh + (size_t)P * kExpMaxBins;               // grad[P][16]
    double *hu = hg + (size_t)P * kExpGrad;                  // up[P]
    CK(cudaEventRecord(c->k0, c->stream));
    if (need_fwd) {
        c->exp_valid = false;
        CK(launch_exp_forward(a, c->stream));
        c->launches += 2;
        c->exp_key = key;
        c->exp_P = P;
        c->exp_nblk = a.nblk;
    }
    if (adjoint) {
        if (dchi2) {
            std::memcpy(hu, dchi2, sizeof(double) * P);
            CK(cudaMemcpyAsync(c->dExpUp, hu, sizeof(double) * P, cudaMemcpyHostToDevice, c->stream));
            a.dchi2 = c->dExpUp;
        }
        CK(launch_exp_adjoint(a, c->stream));
        c->launches += 2;
    }
    CK(cudaEventRecord(c->k1, c->stream));
    c->timed = true;
    if (chi2_out) CK(cudaMemcpyAsync(hc, c->dExpChi2, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
    if (hist_out) CK(cudaMemcpyAsync(hh, c->dExpHist, sizeof(double) * (size_t)P * nb, cudaMemcpyDeviceToHost, c->stream));
    if (adjoint) CK(cudaMemcpyAsync(hg, c->dExpGrad, sizeof(double) * (size_t)P * kExpGrad, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->exp_valid = true;
    if (chi2_out) std::memcpy(chi2_out, hc, sizeof(double) * P);
    if (hist_out) std::memcpy(hist_out, hh, sizeof(double) * (size_t)P * nb);
    if (adjoint) {
        const int nk = n * (n - 1);
        for (int p = 0; p < P; ++p) {
            if (dE) for (int i = 0; i < n; ++i) dE[(size_t)p * n + i] = hg[(size_t)p * kExpGrad + i];
            if (dlogK) for (int k = 0; k < nk; ++k) dlogK[(size_t)p * nk + k] = hg[(size_t)p * kExpGrad + n + k];
        }
    }
    return GPDA_OK;
}

}  // namespace

extern "C" {

void gpda_model_defaults(gpda_model *m) {
    m->nbins = 21;
    m->left_pad = 2;
    m->gamma = 1.0f;
    m->crosstalk = 0.05f;
    m->bg_d = 1500.0f;
    m->bg_a = 800.0f;
    m->r0 = 52.0f;
    m->rc_gamma = 0.34f;
    m->rc_de = 0.08f;
    m->rc_ct = 0.07f;
    m->rc_r0 = 52.0f;
}

const char *gpda_version(void) { return "gpda 0.1 sm_103a"; }

gpda_ctx *gpda_create(int32_t device, const gpda_model *m, int32_t *status) {
    auto set = [&](int s) { if (status) *status = s; };
    gpda_model mm;
    if (m) mm = *m; else gpda_model_defaults(&mm);
    if (check_model(&mm)) { set(GPDA_ERR_ARG); return nullptr; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        set(GPDA_ERR_CUDA);
        return nullptr;
    }
    gpda_ctx *c = new gpda_ctx();
    c->device = device;
    c->model = mm;
    auto bad = [&](cudaError_t e) {
        if (e == cudaSuccess) return false;
        set(GPDA_ERR_CUDA);
        gpda_destroy(c);
        return true;
    };
    if (bad(cudaSetDevice(device))) return nullptr;
    if (bad(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking))) return nullptr;
    if (bad(cudaEventCreateWithFlags(&c->params_ev, cudaEventDisableTiming))) return nullptr;
    if (bad(cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking))) return nullptr;
    if (bad(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device))) return nullptr;
    // work items, CTAs done, then one work counter per burst range of gpda_run_host
    if (bad(cudaMalloc(&c->dWork, (2 + kMaxRanges) * sizeof(unsigned int)))) return nullptr;
    if (bad(cudaMalloc(&c->dLimit, sizeof(unsigned long long)))) return nullptr;
    if (bad(cudaMemset(c->dLimit, 0, sizeof(unsigned long long)))) return nullptr;
    if (bad(cudaMalloc(&c->dObs, sizeof(float) * GPDA_MAX_BINS))) return nullptr;
    if (bad(cudaMalloc(&c->dFlag, sizeof(unsigned int)))) return nullptr;
    if (bad(cudaMallocHost(&c->hFlag, sizeof(unsigned int)))) return nullptr;
    if (bad(cudaEventCreate(&c->k0))) return nullptr;
    if (bad(cudaEventCreate(&c->k1))) return nullptr;
    if (bad(cudaEventRecord(c->params_ev, c->stream))) return nullptr;
    if (bad(pda_occupancy_blocks(0, 0, &c->blocks_per_sm[0]))) return nullptr;
    // the photon kernels' staging may take them past the 48 KB default
    if (bad(pda_set_smem_limit(1, sizeof(float) * kSmemCapFloats))) return nullptr;
    if (bad(pda_set_smem_limit(kModePhotonDirect, sizeof(float) * kSmemCapFloats))) return nullptr;
    if (bad(pda_occupancy_blocks(1, sizeof(float) * kSmemCapFloats, &c->blocks_per_sm[1]))) return nullptr;
    if (bad(pda_occupancy_blocks(kModePhotonDirect, sizeof(float) * kSmemCapFloats,
                                 &c->blocks_per_sm[kModePhotonDirect]))) return nullptr;
    for (int i = 0; i < 3; ++i) c->blocks_per_sm[i] = std::max(1, c->blocks_per_sm[i]);
    set(GPDA_OK);
    return c;
}

void gpda_destroy(gpda_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_dev(c->dN); free_dev(c->dT); free_dev(c->dOffIdx); free_dev(c->dOff);
    free_dev(c->dObs); free_dev(c->dParams); free_dev(c->dHist); free_dev(c->dChi2);
    free_dev(c->dWork); free_dev(c->dLimit); free_dev(c->dUnit); free_dev(c->dFlag);
    free_dev(c->dCdf); free_dev(c->dGuide);
    free_graph(c);
    free_dev(c->dExp); free_dev(c->dExpPart); free_dev(c->dExpGPart); free_dev(c->dExpHist);
    free_dev(c->dExpChi2); free_dev(c->dExpGrad); free_dev(c->dExpUp); free_dev(c->dExpG);
    free_dev(c->dExpInv);
    free_dev(c->dTape);
    if (c->hExp) cudaFreeHost(c->hExp);
    if (c->hExpOut) cudaFreeHost(c->hExpOut);
    if (c->hFlag) cudaFreeHost(c->hFlag);
    if (c->k0) cudaEventDestroy(c->k0);
    if (c->k1) cudaEventDestroy(c->k1);
    if (c->hParams) cudaFreeHost(c->hParams);
    if (c->hHist) cudaFreeHost(c->hHist);
    if (c->hChi2) cudaFreeHost(c->hChi2);
    if (c->params_ev) cudaEventDestroy(c->params_ev);
    for (auto e : c->range_ev) cudaEventDestroy(e);
    for (auto e : c->rjoin) cudaEventDestroy(e);
    for (auto st : c->rstream) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    if (c->prep_ev) cudaEventDestroy(c->prep_ev);
    if (c->cstream) { cudaStreamSynchronize(c->cstream); cudaStreamDestroy(c->cstream); }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *gpda_last_error(const gpda_ctx *c) { return c ? c->err.c_str() : "null context"; }

int32_t gpda_upload_bursts(gpda_ctx *c, const int32_t *N, const float *T, const int64_t *off_idx,
                           const float *offsets, int64_t B) {
    if (!c) return GPDA_ERR_ARG;
    if (B < 1 || B > (int64_t)INT32_MAX || !N || !T) return fail(c, GPDA_ERR_ARG, "B, N or T");
    if ((off_idx == nullptr) != (offsets == nullptr)) return fail(c, GPDA_ERR_ARG, "off_idx and offsets go together");
    int64_t nph = 0;
    if (off_idx) {
        if (off_idx[0] != 0 || off_idx[B] < 0) return fail(c, GPDA_ERR_ARG, "off_idx[0] must be 0 and off_idx[B] >= 0");
        nph = off_idx[B];
    }
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    c->B = 0;
    c->exp_valid = false;
    free_graph(c);
    // grow-only device store; contents are validated on the device below
    if (B > c->cap_B) {
        free_dev(c->dN); free_dev(c->dT); free_dev(c->dOffIdx);
        c->dN = nullptr; c->dT = nullptr; c->dOffIdx = nullptr; c->cap_B = 0;
        CK(cudaMalloc(&c->dN, sizeof(int32_t) * B));
        CK(cudaMalloc(&c->dT, sizeof(float) * B));
        CK(cudaMalloc(&c->dOffIdx, sizeof(int64_t) * (B + 1)));
        c->cap_B = B;
    }
    if (off_idx && nph > c->cap_ph) {
        free_dev(c->dOff);
        c->dOff = nullptr; c->cap_ph = 0;
        CK(cudaMalloc(&c->dOff, sizeof(float) * (nph + kOffPad)));
        c->cap_ph = nph;
    }
    CK(cudaMemcpyAsync(c->dN, N, sizeof(int32_t) * B, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->dT, T, sizeof(float) * B, cudaMemcpyHostToDevice, c->stream));
    c->has_offsets = off_idx != nullptr;
    if (off_idx) {
        CK(cudaMemcpyAsync(c->dOffIdx, off_idx, sizeof(int64_t) * (B + 1), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(c->dOff + nph, 0, sizeof(float) * kOffPad, c->stream));
        if (nph > 0) CK(cudaMemcpyAsync(c->dOff, offsets, sizeof(float) * nph, cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaMemsetAsync(c->dFlag, 0, sizeof(unsigned int), c->stream));
    CK(launch_validate(c->dN, c->dT, off_idx ? c->dOffIdx : nullptr, off_idx ? c->dOff : nullptr, B,
                       nph, c->dFlag, c->num_sms, c->stream));
    c->launches += 1;
    CK(cudaMemcpyAsync(c->hFlag, c->dFlag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    unsigned f = *c->hFlag;
    if (f) {
        std::string why;
        if (f & 1u) why += " N outside [0, 2^21];";
        if (f & 2u) why += " T not finite and >= 0;";
        if (f & 4u) why += " off_idx inconsistent with N;";
        if (f & 8u) why += " offset not finite;";
        if (f & 16u) why += " offsets not sorted within a burst;";
        return fail(c, GPDA_ERR_ARG, "burst store rejected:" + why);
    }
    double sumN = 0.0;
    if (off_idx) sumN = (double)nph;
    else for (int64_t b = 0; b < B; ++b) sumN += N[b];
    c->B = B;
    c->nph = nph;
    c->mean_N = sumN / (double)B;
    return GPDA_OK;
}

int32_t gpda_set_observed(gpda_ctx *c, const float *ohist, int32_t nbins) {
    if (!c) return GPDA_ERR_ARG;
    c->exp_valid = false;
    if (!c->has_obs) {
        cudaStreamSynchronize(c->stream);
        free_graph(c);          // a graph captured without the chi-square node
    }
    if (!ohist || nbins != c->model.nbins) return fail(c, GPDA_ERR_ARG, "observed histogram must have model.nbins bins");
    CK(cudaSetDevice(c->device));
    CK(cudaMemcpyAsync(c->dObs, ohist, sizeof(float) * nbins, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->has_obs = true;
    return GPDA_OK;
}

int32_t gpda_bin_values(const float *x, int64_t n, int32_t nbins, float *hist_out) {
    if ((!x && n > 0) || n < 0 || !hist_out || nbins < 1) return GPDA_ERR_ARG;
    for (int i = 0; i < nbins; ++i) hist_out[i] = 0.0f;
    for (int64_t k = 0; k < n; ++k) {
        double z = (double)x[k];
        if (z < 1.0 && z >= 0.0) hist_out[(int)(z * (double)nbins)] += 1.0f;
    }
    return GPDA_OK;
}

int32_t gpda_params_size(void) { return kParamWords; }

int32_t gpda_build_params(const gpda_model *m, int32_t n, const float *args, float *out) {
    gpda_model mm;
    if (m) mm = *m; else gpda_model_defaults(&mm);
    if (!out) return GPDA_ERR_ARG;
    DevParams p;
    int r = build_params(n, args, mm.gamma, mm.crosstalk, true, &p);
    if (r == -2) return GPDA_ERR_SINGULAR;
    if (r != 0) return GPDA_ERR_ARG;
    std::memcpy(out, &p, sizeof(p));
    return GPDA_OK;
}

int32_t gpda_launch(gpda_ctx *c, int32_t mode, int32_t P, int32_t n, const float *params,
                    int64_t b0, int64_t b1, int32_t S, uint64_t seed) {
    if (!c) return GPDA_ERR_ARG;
    return do_launch(c, mode, P, n, params, b0, b1, S, seed, nullptr);
}

int32_t gpda_fetch(gpda_ctx *c, uint64_t *hist_out, double *chi2_out) {
    if (!c) return GPDA_ERR_ARG;
    if (c->last_P == 0) return fail(c, GPDA_ERR_STATE, "nothing launched");
    CK(cudaSetDevice(c->device));
    const int P = c->last_P, nb = c->model.nbins;
    if (hist_out) CK(cudaMemcpyAsync(c->hHist, c->dHist, sizeof(unsigned long long) * (size_t)P * nb, cudaMemcpyDeviceToHost, c->stream));
    if (chi2_out && c->last_chi2) CK(cudaMemcpyAsync(c->hChi2, c->dChi2, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (hist_out) std::memcpy(hist_out, c->hHist, sizeof(uint64_t) * (size_t)P * nb);
    if (chi2_out) {
        if (c->last_chi2) std::memcpy(chi2_out, c->hChi2, sizeof(double) * P);
        else for (int p = 0; p < P; ++p) chi2_out[p] = NAN;
    }
    return GPDA_OK;
}

int32_t gpda_run_plain(gpda_ctx *c, int32_t mode, int32_t n, const float *params, int64_t b0,
                       int64_t b1, int32_t S, uint64_t seed, uint64_t *hist_out, double *chi2_out) {
    if (!c) return GPDA_ERR_ARG;
    int r = do_launch(c, mode, 1, n, params, b0, b1, S, seed, nullptr);
    if (r) return r;
    return gpda_fetch(c, hist_out, chi2_out);
}

int32_t gpda_run_batched(gpda_ctx *c, int32_t mode, int32_t P, int32_t n, const float *params,
                         int32_t S, uint64_t seed, uint64_t *hist_out, double *chi2_out) {
    if (!c) return GPDA_ERR_ARG;
    int r = do_launch(c, mode, P, n, params, 0, c->B, S, seed, nullptr);
    if (r) return r;
    return gpda_fetch(c, hist_out, chi2_out);
}

int32_t gpda_run_units(gpda_ctx *c, int32_t mode, int32_t P, int32_t n, const float *params,
                       int64_t b0, int64_t b1, int32_t S, uint64_t seed, int32_t *unit_out,
                       uint64_t *hist_out) {
    if (!c) return GPDA_ERR_ARG;
    if (!unit_out || b1 < b0 || P < 1 || S < 1) return fail(c, GPDA_ERR_ARG, "unit_out, range, P or S");
    size_t cnt = (size_t)P * (size_t)(b1 - b0) * (size_t)S;
    CK(cudaSetDevice(c->device));
    if (cnt > c->cap_unit) {
        CK(cudaStreamSynchronize(c->stream));
        free_dev(c->dUnit);
        c->dUnit = nullptr;
        c->cap_unit = 0;
        CK(cudaMalloc(&c->dUnit, sizeof(int32_t) * std::max<size_t>(cnt, 1)));
        c->cap_unit = cnt;
    }
    int r = do_launch(c, mode, P, n, params, b0, b1, S, seed, c->dUnit);
    if (r) return r;
    if (cnt) CK(cudaMemcpyAsync(unit_out, c->dUnit, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, c->stream));
    return gpda_fetch(c, hist_out, nullptr);
}

int32_t gpda_query(gpda_ctx *c) {
    if (!c) return GPDA_ERR_ARG;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamQuery(c->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return cuda_fail(c, e, "cudaStreamQuery");
}

int32_t gpda_synchronize(gpda_ctx *c) {
    if (!c) return GPDA_ERR_ARG;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    return GPDA_OK;
}

void *gpda_stream(gpda_ctx *c) { return c ? (void *)c->stream : nullptr; }

int64_t gpda_launch_count(const gpda_ctx *c) { return c ? c->launches : 0; }

float gpda_kernel_ms(gpda_ctx *c) {
    if (!c || !c->timed) return -1.0f;
    cudaSetDevice(c->device);
    if (cudaEventSynchronize(c->k1) != cudaSuccess) return -1.0f;
    float ms = -1.0f;
    if (cudaEventElapsedTime(&ms, c->k0, c->k1) != cudaSuccess) return -1.0f;
    return ms;
}

int64_t gpda_limit_hits(gpda_ctx *c) {
    if (!c) return GPDA_ERR_ARG;
    unsigned long long v = 0;
    cudaSetDevice(c->device);
    if (cudaMemcpyAsync(&v, c->dLimit, sizeof(v), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return GPDA_ERR_CUDA;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return GPDA_ERR_CUDA;
    return (int64_t)v;
}

int32_t gpda_expected_hist(gpda_ctx *c, int32_t P, int32_t n, const float *params,
                           const float *anchor, int32_t S, uint64_t seed, double *hist_out,
                           double *chi2_out) {
    if (!c) return GPDA_ERR_ARG;
    if (!chi2_out) return fail(c, GPDA_ERR_ARG, "chi2_out");
    return exp_run(c, P, n, params, anchor, S, seed, hist_out, chi2_out, false, nullptr, nullptr, nullptr);
}

int32_t gpda_expected_hist_adjoint(gpda_ctx *c, int32_t P, int32_t n, const float *params,
                                   const float *anchor, int32_t S, uint64_t seed,
                                   const double *dchi2, double *dE, double *dlogK) {
    if (!c) return GPDA_ERR_ARG;
    if (!dE && !dlogK) return fail(c, GPDA_ERR_ARG, "dE or dlogK");
    return exp_run(c, P, n, params, anchor, S, seed, nullptr, nullptr, true, dchi2, dE, dlogK);
}

int32_t gpda_expected_grad(gpda_ctx *c, int32_t P, int32_t n, const float *params,
                           const float *anchor, int32_t S, uint64_t seed, double *hist_out,
                           double *chi2_out, double *dE, double *dlogK) {
    if (!c) return GPDA_ERR_ARG;
    if (!chi2_out) return fail(c, GPDA_ERR_ARG, "chi2_out");
    return exp_run(c, P, n, params, anchor, S, seed, hist_out, chi2_out, true, nullptr, dE, dlogK);
}

int32_t gpda_graph_create(gpda_ctx *c, int32_t mode, int32_t P, int32_t n, int32_t S) {
    if (!c) return GPDA_ERR_ARG;
    if (mode != GPDA_MODE_OCCUPANCY && mode != GPDA_MODE_PHOTON) return fail(c, GPDA_ERR_ARG, "mode");
    if (P < 1 || n < 1 || n > GPDA_MAX_STATES || S < 1) return fail(c, GPDA_ERR_ARG, "P, n_states or samples");
    if (c->B == 0 || !c->dN) return fail(c, GPDA_ERR_STATE, "no bursts uploaded");
    if (mode == GPDA_MODE_PHOTON && !c->has_offsets) return fail(c, GPDA_ERR_STATE, "photon mode needs arrival offsets");
    if (c->B * (int64_t)S > (int64_t)INT32_MAX) return fail(c, GPDA_ERR_ARG, "too many units per parameter set");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    free_graph(c);
    int rc = ensure_scratch(c, P);
    if (rc) return rc;
    if (mode == GPDA_MODE_PHOTON && (size_t)P * n > c->cap_tab) {
        free_dev(c->dCdf);
        free_dev(c->dGuide);
        c->dCdf = nullptr; c->dGuide = nullptr; c->cap_tab = 0;
        CK(cudaMalloc(&c->dCdf, sizeof(float) * kTableRows * (size_t)P * n));
        CK(cudaMalloc(&c->dGuide, sizeof(GuideEntry) * kTableRows * (size_t)P * n));
        c->cap_tab = (size_t)P * n;
    }
    const int nbins = c->model.nbins;
    PdaArgs a{};
    a.bcdf = c->dCdf; a.bguide = c->dGuide;
    a.N = c->dN; a.T = c->dT; a.off_idx = c->dOffIdx; a.offsets = c->dOff;
    a.params = c->dParams; a.hist = c->dHist; a.unit_out = nullptr; a.work = c->dWork;
    a.limit_hits = c->dLimit;
    a.b0 = 0; a.b1 = c->B; a.seed = 0; a.P = P; a.S = S;
    a.tile_b = tile_bursts(c, mode, S, c->B, P);
    int64_t ntiles = (c->B + a.tile_b - 1) / a.tile_b;
    if (ntiles * P > (int64_t)INT32_MAX) return fail(c, GPDA_ERR_ARG, "too many work items");
    a.ntiles = (int)ntiles; a.n_items = (int)(ntiles * P); a.nbins = nbins;
    a.smem_cap = kSmemCapFloats; a.pbase = 0u;
    a.gamma = c->model.gamma; a.ct = c->model.crosstalk; a.r0 = c->model.r0;
    a.bg_a = c->model.bg_a; a.bg_d = c->model.bg_d;
    if (c->has_obs) {
        a.obs = c->dObs; a.chi2 = c->dChi2; a.done = c->dWork + 1;
        a.left_pad = c->model.left_pad; a.n_states = n;
    }
    const size_t dyn = (mode == GPDA_MODE_PHOTON) ? sizeof(float) * kSmemCapFloats : 0;
    const int grid = (int)std::min<int64_t>(a.n_items, (int64_t)c->num_sms * c->blocks_per_sm[mode]);
    // one stream capture of the whole batched step
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int kernels = 0;
    cudaError_t e = cudaMemcpyAsync(c->dParams, c->hParams, sizeof(DevParams) * P, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && mode == GPDA_MODE_PHOTON) { e = launch_binom_tables(c->dParams, P, n, c->dCdf, c->dGuide, c->stream); kernels++; }
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dHist, 0, sizeof(unsigned long long) * (size_t)P * nbins, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dWork, 0, 2 * sizeof(unsigned int), c->stream);
    if (e == cudaSuccess) { e = launch_pda(mode, a, grid, dyn, c->stream); kernels++; }
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->hHist, c->dHist, sizeof(unsigned long long) * (size_t)P * nbins, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && c->has_obs) e = cudaMemcpyAsync(c->hChi2, c->dChi2, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return cuda_fail(c, e != cudaSuccess ? e : e2, "graph capture");
    }
    c->graph = g;
    // the Monte-Carlo kernel node, whose seed each replay sets
    size_t nn = 0;
    CK(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CK(cudaGraphGetNodes(g, nodes.data(), &nn));
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nd, &t));
        if (t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp{};
        CK(cudaGraphKernelNodeGetParams(nd, &kp));
        if (kp.func == pda_kernel_fn(mode)) {
            c->gnode = nd;
            c->gkp = kp;
        }
    }
    if (!c->gnode) { free_graph(c); return fail(c, GPDA_ERR_STATE, "graph capture: kernel node not found"); }
    CK(cudaGraphInstantiate(&c->gexec, g, 0));
    c->gargs = a;
    c->gargv[0] = &c->gargs;
    c->gkp.kernelParams = c->gargv;
    c->gkp.extra = nullptr;
    c->g_mode = mode; c->g_P = P; c->g_n = n; c->g_S = S; c->g_kernels = kernels;
    c->g_chi2 = c->has_obs;
    return GPDA_OK;
}

int32_t gpda_graph_run(gpda_ctx *c, const float *params, uint64_t seed, uint64_t *hist_out,
                       double *chi2_out) {
    if (!c) return GPDA_ERR_ARG;
    if (!c->gexec) return fail(c, GPDA_ERR_STATE, "no captured launch (gpda_graph_create first)");
    if (!params) return fail(c, GPDA_ERR_ARG, "params");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));    // pinned staging is free
    const int P = c->g_P, n = c->g_n, nb = c->model.nbins;
    const size_t stride = (size_t)n * (n + 1);
    for (int p = 0; p < P; ++p) {
        int r = build_params(n, params + stride * p, c->model.gamma, c->model.crosstalk, true, &c->hParams[p]);
        if (r == -2) return fail(c, GPDA_ERR_SINGULAR, "rate matrix has no unique stationary distribution (parameter set " + std::to_string(p) + ")");
        if (r != 0) return fail(c, GPDA_ERR_ARG, "invalid parameter vector " + std::to_string(p));
    }
    c->gargs.seed = seed;
    CK(cudaGraphExecKernelNodeSetParams(c->gexec, c->gnode, &c->gkp));
    CK(cudaEventRecord(c->k0, c->stream));
    CK(cudaGraphLaunch(c->gexec, c->stream));
    CK(cudaEventRecord(c->k1, c->stream));
    c->timed = true;
    c->launches += c->g_kernels;
    c->last_P = P;
    c->last_chi2 = c->g_chi2;
    CK(cudaStreamSynchronize(c->stream));
    if (hist_out) std::memcpy(hist_out, c->hHist, sizeof(uint64_t) * (size_t)P * nb);
    if (chi2_out) {
        if (c->g_chi2) std::memcpy(chi2_out, c->hChi2, sizeof(double) * P);
        else for (int p = 0; p < P; ++p) chi2_out[p] = NAN;
    }
    return GPDA_OK;
}

int32_t gpda_autotune(gpda_ctx *c, int32_t mode, int32_t P, int32_t n, const float *params,
                      int32_t S, uint64_t seed, int32_t *tile_out) {
    if (!c) return GPDA_ERR_ARG;
    if (mode != GPDA_MODE_OCCUPANCY && mode != GPDA_MODE_PHOTON) return fail(c, GPDA_ERR_ARG, "mode");
    CK(cudaSetDevice(c->device));
    // forget an earlier choice for this shape, then time candidates around the default
    for (size_t i = 0; i < c->tuned.size(); ++i)
        if (c->tuned[i][0] == mode && c->tuned[i][1] == S) { c->tuned.erase(c->tuned.begin() + i); break; }
    const int base = tile_bursts(c, mode, S, c->B, P);
    std::vector<int> cand;
    for (int f : {-2, -1, 0, 1, 2}) {
        int t = f < 0 ? base >> (-f) : base << f;
        t = std::max(1, std::min(t, kMaxTileBursts));
        if (std::find(cand.begin(), cand.end(), t) == cand.end()) cand.push_back(t);
    }
    int best = base;
    float best_ms = 1e30f;
    for (int t : cand) {
        c->tuned.push_back({mode, S, t});
        float ms = 0.0f;
        for (int r = 0; r < 3; ++r) {
            int rc = do_launch(c, mode, P, n, params, 0, c->B, S, seed + (uint64_t)r, nullptr);
            if (rc) { c->tuned.pop_back(); return rc; }
            float k = gpda_kernel_ms(c);
            if (r > 0) ms += k;      // the first launch warms the caches
        }
        c->tuned.pop_back();
        if (ms < best_ms) { best_ms = ms; best = t; }
    }
    CK(cudaStreamSynchronize(c->stream));
    free_graph(c);               // a captured launch uses the old tile
    c->tuned.push_back({mode, S, best});
    if (tile_out) *tile_out = best;
    return GPDA_OK;
}

int32_t gpda_run_host(gpda_ctx *c, int32_t mode, int32_t P, int32_t n, const float *params,
                      const int32_t *N, const float *T, const int64_t *off_idx, const float *offsets,
                      int64_t B, int32_t S, uint64_t seed, int32_t ranges, uint64_t *hist_out,
                      double *chi2_out) {
    if (!c) return GPDA_ERR_ARG;
    if (mode != GPDA_MODE_OCCUPANCY && mode != GPDA_MODE_PHOTON) return fail(c, GPDA_ERR_ARG, "mode");
    if (P < 1 || n < 1 || n > GPDA_MAX_STATES || S < 1 || !params) return fail(c, GPDA_ERR_ARG, "P, n_states, samples or params");
    if (B < 1 || B > (int64_t)INT32_MAX || !N || !T) return fail(c, GPDA_ERR_ARG, "B, N or T");
    if ((off_idx == nullptr) != (offsets == nullptr)) return fail(c, GPDA_ERR_ARG, "off_idx and offsets go together");
    if (mode == GPDA_MODE_PHOTON && !off_idx) return fail(c, GPDA_ERR_ARG, "photon mode needs arrival offsets");
    if (B * (int64_t)S > (int64_t)INT32_MAX) return fail(c, GPDA_ERR_ARG, "too many units per parameter set");
    if (ranges < 1 || ranges > kMaxRanges) return fail(c, GPDA_ERR_ARG, "ranges in [1, 64]");
    int64_t nph = 0;
    if (off_idx) {
        if (off_idx[0] != 0 || off_idx[B] < 0) return fail(c, GPDA_ERR_ARG, "off_idx[0] must be 0 and off_idx[B] >= 0");
        nph = off_idx[B];
    }
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    c->B = 0;
    c->exp_valid = false;
    free_graph(c);
    if (B > c->cap_B) {
        free_dev(c->dN); free_dev(c->dT); free_dev(c->dOffIdx);
        c->dN = nullptr; c->dT = nullptr; c->dOffIdx = nullptr; c->cap_B = 0;
        CK(cudaMalloc(&c->dN, sizeof(int32_t) * B));
        CK(cudaMalloc(&c->dT, sizeof(float) * B));
        CK(cudaMalloc(&c->dOffIdx, sizeof(int64_t) * (B + 1)));
        c->cap_B = B;
    }
    if (off_idx && nph > c->cap_ph) {
        free_dev(c->dOff);
        c->dOff = nullptr; c->cap_ph = 0;
        CK(cudaMalloc(&c->dOff, sizeof(float) * (nph + kOffPad)));
        c->cap_ph = nph;
    }
    c->has_offsets = off_idx != nullptr;
    c->nph = nph;
    c->mean_N = (double)nph / (double)B;
    // Direct reads: in photon mode with one parameter set, page-locked host
    // arrays are read by the kernel itself over the host link, each CTA
    // staging its tile and writing it through to the store (PdaArgs::hN).
    // One launch starts at once; the host link moves the store no faster
    // than the copy engine, but the transfer now spreads over the whole
    // simulation instead of preceding the first range's. Any other memory
    // goes through the copy engine in burst ranges below.
    if (mode == GPDA_MODE_PHOTON && P == 1) {
        const void *hN = mapped_host(N, sizeof(int32_t) * (size_t)B);
        const void *hT = mapped_host(T, sizeof(float) * (size_t)B);
        const void *hOI = mapped_host(off_idx, sizeof(int64_t) * (size_t)(B + 1));
        const void *hOff = nph > 0 ? mapped_host(offsets, sizeof(float) * (size_t)nph) : c->dOff;
        auto aligned = [](const void *p, uintptr_t to) { return (reinterpret_cast<uintptr_t>(p) % to) == 0u; };
        if (hN && hT && hOI && hOff && aligned(hN, 4) && aligned(hT, 4) && aligned(hOI, 8) &&
            aligned(hOff, 16)) {
            CK(cudaMemsetAsync(c->dFlag, 0, sizeof(unsigned int), c->stream));
            CK(cudaMemsetAsync(c->dOff + nph, 0, sizeof(float) * kOffPad, c->stream));
            c->B = B;
            int rc = prepare_launch(c, mode, P, n, params);
            PdaArgs a;
            int grid = 0;
            if (!rc) rc = range_args(c, mode, P, n, 0, B, S, seed, nullptr, c->has_obs, nullptr, a, grid);
            if (rc) {
                cudaStreamSynchronize(c->stream);
                c->B = 0;
                return rc;
            }
            a.tile_b = tile_bursts(c, mode, S, B, P, true);
            if ((B + a.tile_b - 1) / a.tile_b > (int64_t)INT32_MAX) {
                cudaStreamSynchronize(c->stream);
                c->B = 0;
                return fail(c, GPDA_ERR_ARG, "too many work items");
            }
            a.ntiles = (int)((B + a.tile_b - 1) / a.tile_b);
            a.n_items = a.ntiles;   // one parameter set
            grid = (int)std::min<int64_t>(a.n_items, (int64_t)c->num_sms * c->blocks_per_sm[kModePhotonDirect]);
            a.vflag = c->dFlag;
            a.nph = nph;
            a.hN = static_cast<const int32_t *>(hN);
            a.hT = static_cast<const float *>(hT);
            a.hOffIdx = static_cast<const int64_t *>(hOI);
            a.hOff = static_cast<const float *>(hOff);
            a.wN = c->dN;
            a.wT = c->dT;
            a.wOffIdx = c->dOffIdx;
            a.wOff = c->dOff;
            a.pdl = GPDA_PDL;       // right after the tables (prepare_launch)
            cudaError_t e = launch_pda(kModePhotonDirect, a, grid, sizeof(float) * kSmemCapFloats, c->stream);
            if (e != cudaSuccess) {
                cudaStreamSynchronize(c->stream);
                c->B = 0;
                return fail(c, GPDA_ERR_CUDA, cudaGetErrorString(e));
            }
            c->launches += 1;
            CK(cudaEventRecord(c->k1, c->stream));
            c->timed = true;
            c->last_chi2 = c->has_obs;
            return host_run_results(c, P, hist_out, chi2_out);
        }
    }
    while ((int)c->range_ev.size() < ranges) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->range_ev.push_back(e);
    }
    while ((int)c->rstream.size() < kRangeStreams) {
        cudaStream_t st;
        cudaEvent_t e;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        c->rstream.push_back(st);
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->rjoin.push_back(e);
    }
    if (!c->prep_ev) CK(cudaEventCreateWithFlags(&c->prep_ev, cudaEventDisableTiming));
    if (!off_idx) {
        double sumN = 0.0;
        for (int64_t b = 0; b < B; ++b) sumN += N[b];
        c->mean_N = sumN / (double)B;
    }
    // range r ends at burst B (g^r - 1) / (g^ranges - 1), g = kRangeGrowth:
    // each range is g times the one before, so the copy of the next range
    // (the copy engine moves a burst about twice as fast as the kernel
    // simulates it) hides under the simulation of this one and only the
    // first, smallest copy is exposed
    auto edge = [&](int r) -> int64_t {
        if (r >= ranges) return B;
        return (int64_t)((double)B * (std::pow(kRangeGrowth, r) - 1.0) /
                         (std::pow(kRangeGrowth, ranges) - 1.0));
    };
    // In photon mode with few parameter sets the kernel's CTAs check their
    // own bursts (PdaArgs::vflag) and no validate_kernel runs: each of those
    // launches had to wait for SMs held by the previous range's kernel.
    const bool fused = mode == GPDA_MODE_PHOTON && P <= kFusedCheckSets;
    const int nr = std::min(ranges, kRangeStreams);
    auto drain = [&]() {
        cudaStreamSynchronize(c->cstream);
        for (int k = 0; k < nr; ++k) cudaStreamSynchronize(c->rstream[k]);
        cudaStreamSynchronize(c->stream);
        c->B = 0;
    };
    // The copy stream first (the host prepares the parameters while the
    // first range is in flight): the flag reset, then each range's copies
    // (and validation), each range closed by its event.
    CK(cudaMemsetAsync(c->dFlag, 0, sizeof(unsigned int), c->cstream));
    if (off_idx) CK(cudaMemsetAsync(c->dOff + nph, 0, sizeof(float) * kOffPad, c->cstream));
    c->B = B;                       // the ranges below address the new store
    for (int r = 0; r < ranges; ++r) {
        const int64_t b0 = edge(r), b1 = edge(r + 1);
        if (b1 > b0) {
            CK(cudaMemcpyAsync(c->dN + b0, N + b0, sizeof(int32_t) * (b1 - b0), cudaMemcpyHostToDevice, c->cstream));
            CK(cudaMemcpyAsync(c->dT + b0, T + b0, sizeof(float) * (b1 - b0), cudaMemcpyHostToDevice, c->cstream));
            if (off_idx) {
                CK(cudaMemcpyAsync(c->dOffIdx + b0, off_idx + b0, sizeof(int64_t) * (b1 - b0 + 1), cudaMemcpyHostToDevice, c->cstream));
                const int64_t p0 = off_idx[b0], p1 = off_idx[b1];
                if (p0 >= 0 && p1 > p0 && p1 <= nph)
                    CK(cudaMemcpyAsync(c->dOff + p0, offsets + p0, sizeof(float) * (p1 - p0), cudaMemcpyHostToDevice, c->cstream));
                else if (!(p0 >= 0 && p1 >= p0 && p1 <= nph)) {
                    // host-visible inconsistency: the device check would flag it too
                    drain();
                    return fail(c, GPDA_ERR_ARG, "burst store rejected: off_idx inconsistent with N;");
                }
            }
            if (!fused) {
                CK(launch_validate(c->dN + b0, c->dT + b0, off_idx ? c->dOffIdx + b0 : nullptr,
                                   off_idx ? c->dOff : nullptr, b1 - b0, nph, c->dFlag, c->num_sms, c->cstream));
                c->launches += 1;
            }
        }
        CK(cudaEventRecord(c->range_ev[r], c->cstream));
    }
    // The compute stream: parameters, tables, histogram and counter resets.
    // Each range's kernel then runs on one of kRangeStreams streams as soon
    // as its copy is in, so the last CTAs of one range overlap the first of
    // the next. Every range has its own work counter; the CTAs-done counter
    // is shared, and the last CTA of all of them writes the chi-square.
    int rc = prepare_launch(c, mode, P, n, params);
    if (rc) { drain(); return rc; }
    std::vector<PdaArgs> ra(ranges);
    std::vector<int> rgrid(ranges, 0);
    uint32_t total = 0;
    for (int r = 0; r < ranges; ++r) {
        const int64_t b0 = edge(r), b1 = edge(r + 1);
        if (b1 == b0) continue;
        rc = range_args(c, mode, P, n, b0, b1, S, seed, nullptr, c->has_obs, c->dFlag, ra[r], rgrid[r]);
        if (rc) { drain(); return rc; }
        ra[r].work = c->dWork + 2 + r;
        if (fused) {
            ra[r].vflag = c->dFlag;
            ra[r].nph = nph;
        }
        total += (uint32_t)rgrid[r];
    }
    for (int r = 0; r < ranges; ++r) ra[r].done_target = total;
    CK(cudaMemsetAsync(c->dWork, 0, (size_t)(2 + ranges) * sizeof(unsigned int), c->stream));
    CK(cudaEventRecord(c->prep_ev, c->stream));
    CK(cudaEventRecord(c->k0, c->stream));
    const size_t dyn = (mode == GPDA_MODE_PHOTON) ? sizeof(float) * kSmemCapFloats : 0;
    for (int r = 0; r < ranges; ++r) {
        if (rgrid[r] == 0) continue;
        cudaStream_t st = c->rstream[r % nr];
        CK(cudaStreamWaitEvent(st, c->prep_ev, 0));
        CK(cudaStreamWaitEvent(st, c->range_ev[r], 0));
        cudaError_t e = launch_pda(mode, ra[r], rgrid[r], dyn, st);
        if (e != cudaSuccess) { drain(); return fail(c, GPDA_ERR_CUDA, cudaGetErrorString(e)); }
        c->launches += 1;
    }
    for (int k = 0; k < nr; ++k) {
        CK(cudaEventRecord(c->rjoin[k], c->rstream[k]));
        CK(cudaStreamWaitEvent(c->stream, c->rjoin[k], 0));
    }
    CK(cudaStreamWaitEvent(c->stream, c->range_ev[ranges - 1], 0));
    CK(cudaEventRecord(c->k1, c->stream));
    c->timed = true;
    c->last_chi2 = c->has_obs;
    return host_run_results(c, P, hist_out, chi2_out);
}

int32_t gpda_expected_set_tape_limit(gpda_ctx *c, int64_t bytes) {
    if (!c) return GPDA_ERR_ARG;
    if (bytes < 0) return fail(c, GPDA_ERR_ARG, "bytes");
    c->tape_limit = bytes;
    c->exp_valid = false;
    return GPDA_OK;
}

}  // extern "C"
