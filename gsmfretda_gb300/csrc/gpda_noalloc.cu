// gpda_noalloc.cu — the Monte-Carlo PDA kernel behind an entry point that
// allocates no memory (gpda_run_pda_noalloc in include/gpda.h).
//
// Who needs it: callers that cannot allocate device memory on the path where
// they evaluate parameter sets. Typical cases are a host framework whose
// caching allocator already owns (almost) all of the device memory, where a
// cudaMalloc behind its back fails or fragments the pool, and a tight
// evaluation loop that must not pay the implicit device synchronisation of
// cudaMalloc/cudaFree. Such a caller passes device buffers for the bursts and
// for the histogram it wants back; everything else the kernel needs as
// scratch (the per-parameter-set tables, the work-item counter and the
// loop-limit counter) lives in one fixed array inside this library.
//
// The array is a file-scope __device__ array of kNoAllocScratchBytes bytes
// (about 21 MB): every device that loads the library holds a copy until the
// process exits. It limits a call to kNoAllocMaxP (64) parameter sets, and in
// photon mode to kNoAllocMaxTables (8) parameter-set x state binomial tables
// (P * n_states <= 8).
// All calls share it and it keeps the last call's contents; the counters are
// cleared on every call, but calls whose work overlaps on the GPU (different
// streams, or different host threads without ordering between them) race on
// it and must be serialised by the caller (one stream, or events).
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current; make that first call
// before any stream capture begins.
// The caller's arrays are read in place: offsets must start on a 16-byte
// boundary (the photon staging reads it as float4), and it may be exactly
// off_idx[B] floats long (the last vector of every tile is read element by
// element). Units whose bounded loops hit their limit are counted in the
// scratch but not reported by this entry point.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/gpda.h"
#include "gpda_internal.h"

using namespace gpda;

namespace {

constexpr int kNoAllocMaxP = 64;
constexpr int kNoAllocMaxTables = 8;   // photon mode: P * n_states (parameter set, state) tables
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    DevParams params[kNoAllocMaxP];
    unsigned int work;
    unsigned int pad_[3];
    unsigned long long limit_hits;
    float cdf[kNoAllocMaxTables * kTableRows];
    GuideEntry guide[kNoAllocMaxTables * kTableRows];
};
constexpr size_t kNoAllocScratchBytes = sizeof(NoAllocScratch);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct DeviceSetup {
    NoAllocScratch *scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = 0;
    int blocks_per_sm[2] = {0, 0};
    bool done = false;
};
DeviceSetup g_setup[kNoAllocMaxDevices];
std::mutex g_setup_mu;

constexpr int kSmemCapFloats = 8192;  // same photon staging capacity as the context-based path

// The parameter tables reach the scratch as kernel arguments: a launch takes
// its own copy of them, so nothing refers to this call's stack once it has
// returned (a cudaMemcpyAsync from a pageable stack array would). 24 tables
// make 27,264 bytes, within the 32,764-byte argument limit of sm_70 and later.
constexpr int kParamsPerLaunch = 24;
struct ParamBatch {
    DevParams p[kParamsPerLaunch];
};
static_assert(sizeof(ParamBatch) <= 32764, "kernel argument limit");

__global__ void noalloc_params_kernel(const ParamBatch b, int count, DevParams *dst) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(b.p);
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    for (int i = threadIdx.x; i < count * kParamWords; i += blockDim.x) d[i] = src[i];
}

int setup_device(int dev, DeviceSetup **out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup &s = g_setup[dev];
    if (!s.done) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return GPDA_ERR_CUDA;
        }
        s.scratch = static_cast<NoAllocScratch *>(p);
        if (cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            pda_occupancy_blocks(0, 0, &s.blocks_per_sm[0]) != cudaSuccess ||
            pda_occupancy_blocks(1, sizeof(float) * kSmemCapFloats, &s.blocks_per_sm[1]) != cudaSuccess) {
            cudaGetLastError();
            return GPDA_ERR_CUDA;
        }
        s.blocks_per_sm[0] = std::max(1, s.blocks_per_sm[0]);
        s.blocks_per_sm[1] = std::max(1, s.blocks_per_sm[1]);
        s.done = true;
    }
    *out = &s;
    return GPDA_OK;
}

}  // namespace

extern "C" int32_t gpda_run_pda_noalloc(const gpda_model *m, int32_t mode, int32_t P, int32_t n_states,
                                        const float *params, const int32_t *N, const float *T,
                                        const int64_t *off_idx, const float *offsets, int64_t B,
                                        int32_t samples, uint64_t seed, uint64_t *hist,
                                        const float *ohist, double *chi2, void *stream) {
    gpda_model mm;
    if (m) mm = *m; else gpda_model_defaults(&mm);
    if (mode != GPDA_MODE_OCCUPANCY && mode != GPDA_MODE_PHOTON) return GPDA_ERR_ARG;
    if (P < 1 || P > kNoAllocMaxP) return GPDA_ERR_ARG;   // beyond the fixed scratch
    if (n_states < 1 || n_states > GPDA_MAX_STATES || samples < 1 || !params) return GPDA_ERR_ARG;
    if (!N || !T || !hist || B < 1 || B * (int64_t)samples > (int64_t)INT32_MAX) return GPDA_ERR_ARG;
    if (mode == GPDA_MODE_PHOTON && (!off_idx || !offsets)) return GPDA_ERR_ARG;
    auto aligned = [](const void *p, uintptr_t to) { return (reinterpret_cast<uintptr_t>(p) % to) == 0u; };
    if (!aligned(N, 4) || !aligned(T, 4) || !aligned(hist, 8) || (chi2 && !aligned(chi2, 8)) ||
        (ohist && !aligned(ohist, 4)))
        return GPDA_ERR_ARG;
    if (mode == GPDA_MODE_PHOTON && (!aligned(off_idx, 8) || !aligned(offsets, 16))) return GPDA_ERR_ARG;
    if (mode == GPDA_MODE_PHOTON && P * n_states > kNoAllocMaxTables) return GPDA_ERR_ARG;
    if ((ohist == nullptr) != (chi2 == nullptr)) return GPDA_ERR_ARG;
    if (mm.nbins < 1 || mm.nbins > GPDA_MAX_BINS || mm.left_pad < 0 || mm.left_pad > mm.nbins ||
        !(mm.gamma > 0.0f) || !(mm.crosstalk >= 0.0f) || !(mm.bg_a >= 0.0f) || !(mm.bg_d >= 0.0f) ||
        !(mm.r0 > 0.0f))
        return GPDA_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
        cudaGetLastError();
        return GPDA_ERR_CUDA;
    }
    DeviceSetup *su = nullptr;
    int rc = setup_device(dev, &su);
    if (rc) return rc;

    // parameter tables: built on this thread's stack in batches, each batch
    // passed by value to a copy kernel (see ParamBatch); all are checked
    // before anything is enqueued
    ParamBatch batch[(kNoAllocMaxP + kParamsPerLaunch - 1) / kParamsPerLaunch];
    const size_t stride = (size_t)n_states * (n_states + 1);
    for (int p = 0; p < P; ++p) {
        int r = build_params(n_states, params + stride * p, mm.gamma, mm.crosstalk, true,
                             &batch[p / kParamsPerLaunch].p[p % kParamsPerLaunch]);
        if (r == -2) return GPDA_ERR_SINGULAR;
        if (r != 0) return GPDA_ERR_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NoAllocScratch *sc = su->scratch;
    const int nbins = mm.nbins;
    for (int p0 = 0; p0 < P; p0 += kParamsPerLaunch) {
        int count = std::min(kParamsPerLaunch, P - p0);
        DevParams *dst = sc->params + p0;
        void *kargs[] = {&batch[p0 / kParamsPerLaunch], &count, &dst};
        if (cudaLaunchKernel(reinterpret_cast<const void *>(noalloc_params_kernel), dim3(1), dim3(256), kargs,
                             0, st) != cudaSuccess) {
            cudaGetLastError();
            return GPDA_ERR_CUDA;
        }
    }
    if (cudaMemsetAsync(&sc->work, 0, sizeof(unsigned int), st) != cudaSuccess ||
        cudaMemsetAsync(&sc->limit_hits, 0, sizeof(unsigned long long), st) != cudaSuccess ||
        cudaMemsetAsync(hist, 0, sizeof(uint64_t) * (size_t)P * nbins, st) != cudaSuccess) {
        cudaGetLastError();
        return GPDA_ERR_CUDA;
    }
    if (mode == GPDA_MODE_PHOTON &&
        launch_binom_tables(sc->params, P, n_states, sc->cdf, sc->guide, st) != cudaSuccess)
        return GPDA_ERR_CUDA;
    PdaArgs a{};
    a.bcdf = sc->cdf;
    a.bguide = sc->guide;
    a.N = N;
    a.T = T;
    a.off_idx = off_idx;
    a.offsets = offsets;
    a.exact_offsets = 1;          // the caller's array need not be padded
    a.params = sc->params;
    a.hist = reinterpret_cast<unsigned long long *>(hist);
    a.unit_out = nullptr;
    a.work = &sc->work;
    a.limit_hits = &sc->limit_hits;
    a.b0 = 0;
    a.b1 = B;
    a.seed = seed;
    a.P = P;
    a.S = samples;
    // tile size only changes scheduling, never results (counters are per unit)
    int tb = (2048 + samples - 1) / samples;
    if (mode == GPDA_MODE_PHOTON) tb = std::min(tb, 32);
    a.tile_b = std::max(1, std::min(tb, kMaxTileBursts));
    int64_t ntiles = (B + a.tile_b - 1) / a.tile_b;
    if (ntiles * P > (int64_t)INT32_MAX) return GPDA_ERR_ARG;
    a.ntiles = (int)ntiles;
    a.n_items = (int)(ntiles * P);
    a.nbins = nbins;
    a.smem_cap = kSmemCapFloats;
    a.pbase = 0u;
    a.gamma = mm.gamma;
    a.ct = mm.crosstalk;
    a.r0 = mm.r0;
    a.bg_a = mm.bg_a;
    a.bg_d = mm.bg_d;
    size_t dyn = (mode == GPDA_MODE_PHOTON) ? sizeof(float) * kSmemCapFloats : 0;
    int grid = (int)std::min<int64_t>(a.n_items, (int64_t)su->num_sms * su->blocks_per_sm[mode]);
    if (launch_pda(mode, a, grid, dyn, st) != cudaSuccess) return GPDA_ERR_CUDA;
    if (ohist) {
        if (launch_chi2(a.hist, ohist, P, nbins, mm.left_pad, samples, n_states, chi2, st) != cudaSuccess)
            return GPDA_ERR_CUDA;
    }
    return GPDA_OK;
}
