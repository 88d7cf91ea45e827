// gpda_mc.cu — the drop-in for the reference's `mc` engine object
// (src/mc.hpp:32-180, src/mc.cu:212-829), as a C ABI (include/gpda.h) with a
// C++ class over it (include/gpda_mc.hpp).
//
// Kept from the reference: the per-stream state (n states, parameter tables,
// N bursts, pinned hmcE results), the call sequence of gpuWorker::run
// (src/gpuWorker.cpp:69-82), the argument meaning of every call, and the
// semantics of mc_kernel (ref-compat kernel in gpda_kernels.cu), including
// that the kernel always simulates bursts [0, N) of the data set: mc::run_kernel
// passes no burst offset (src/mc.cu:571-576).
// Changed: no curand state tables (counter-based Philox: init_randstate and
// set_params_buff have nothing to allocate), errors are returned instead of
// exit(), and the device also bins the values into the reference's histogram.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpda.h"
#include "gpda_internal.h"

using namespace gpda;

namespace {

struct McStream {
    cudaStream_t st = nullptr;
    int s_n = 0;
    int oldN = 0;
    int begin = 0, end = 0;
    bool have_params = false;
    DevParams *dParams = nullptr;
    DevParams *hParams = nullptr;   // pinned
    float *dMcE = nullptr;
    float *hMcE = nullptr;          // pinned (mc::hmcE[sid])
    size_t cap = 0;
    unsigned long long *dHist = nullptr;
    unsigned long long *hHist = nullptr;  // pinned
    uint32_t calls = 0;
};

}  // namespace

struct gpda_mc {
    int devid = 0;
    int streamNum = 0;
    gpda_model model{};
    uint64_t seed = 1234;
    int R = 4;              // reSampleTimes (src/mc.cu:308)
    int nbins = 200;        // fretHistNum default (cmdline.ggo, -f 200)
    int64_t B = 0;
    int64_t sz_tag = 0;
    int64_t *dStart = nullptr, *dStop = nullptr, *dIstart = nullptr, *dAd = nullptr, *dDd = nullptr;
    int32_t *dPh = nullptr;
    float *dT = nullptr, *dSg = nullptr;
    float clk_p = 0.0f, bg_ad = 0.0f, bg_dd = 0.0f;
    bool inited = false;
    unsigned long long *dLimit = nullptr;
    std::vector<McStream> streams;
    std::string err;
};

namespace {

int mfail(gpda_mc *m, int code, const std::string &msg) {
    if (m) m->err = msg;
    return code;
}

#define MCK(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return mfail(m, GPDA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

bool valid_sid(const gpda_mc *m, int sid) { return m && sid >= 0 && sid < m->streamNum; }

}  // namespace

extern "C" {

gpda_mc *gpda_mc_create(int32_t devid, int32_t streamNum, uint8_t debug, uint64_t hdf5size,
                        int32_t profiler, int32_t *status) {
    (void)debug; (void)hdf5size; (void)profiler;
    auto set = [&](int s) { if (status) *status = s; };
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || devid < 0 || devid >= ndev || streamNum < 0) {
        cudaGetLastError();
        set(devid < 0 || streamNum < 0 ? GPDA_ERR_ARG : GPDA_ERR_CUDA);
        return nullptr;
    }
    gpda_mc *m = new gpda_mc();
    m->devid = devid;
    gpda_model_defaults(&m->model);
    auto bad = [&](cudaError_t e) {
        if (e == cudaSuccess) return false;
        set(GPDA_ERR_CUDA);
        gpda_mc_destroy(m);
        return true;
    };
    if (bad(cudaSetDevice(devid))) return nullptr;
    if (streamNum == 0) {
        // showGPUsInfo: 2 x asyncEngineCount when copies overlap kernels (src/mc.cu:61-66)
        int engines = 0;
        if (bad(cudaDeviceGetAttribute(&engines, cudaDevAttrAsyncEngineCount, devid))) return nullptr;
        streamNum = engines > 0 ? 2 * engines : 1;
    }
    m->streamNum = streamNum;
    m->streams.resize(streamNum);
    for (auto &s : m->streams) {
        if (bad(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking))) return nullptr;
        if (bad(cudaMalloc(&s.dParams, sizeof(DevParams)))) return nullptr;
        if (bad(cudaMallocHost(&s.hParams, sizeof(DevParams)))) return nullptr;
        if (bad(cudaMalloc(&s.dHist, sizeof(unsigned long long) * GPDA_MAX_BINS))) return nullptr;
        if (bad(cudaMallocHost(&s.hHist, sizeof(unsigned long long) * GPDA_MAX_BINS))) return nullptr;
    }
    if (bad(cudaMalloc(&m->dLimit, sizeof(unsigned long long)))) return nullptr;
    if (bad(cudaMemset(m->dLimit, 0, sizeof(unsigned long long)))) return nullptr;
    set(GPDA_OK);
    return m;
}

void gpda_mc_destroy(gpda_mc *m) {
    if (!m) return;
    cudaSetDevice(m->devid);
    for (auto &s : m->streams) {
        if (s.st) cudaStreamSynchronize(s.st);
        if (s.dParams) cudaFree(s.dParams);
        if (s.hParams) cudaFreeHost(s.hParams);
        if (s.dMcE) cudaFree(s.dMcE);
        if (s.hMcE) cudaFreeHost(s.hMcE);
        if (s.dHist) cudaFree(s.dHist);
        if (s.hHist) cudaFreeHost(s.hHist);
        if (s.st) cudaStreamDestroy(s.st);
    }
    void *bufs[] = {m->dStart, m->dStop, m->dIstart, m->dAd, m->dDd, m->dPh, m->dT, m->dSg, m->dLimit};
    for (void *p : bufs)
        if (p) cudaFree(p);
    delete m;
}

const char *gpda_mc_last_error(const gpda_mc *m) { return m ? m->err.c_str() : "null mc"; }
int32_t gpda_mc_stream_num(const gpda_mc *m) { return m ? m->streamNum : GPDA_ERR_ARG; }
int32_t gpda_mc_sz_burst(const gpda_mc *m) { return m ? (int32_t)m->B : GPDA_ERR_ARG; }
int32_t gpda_mc_resample_times(const gpda_mc *m) { return m ? m->R : GPDA_ERR_ARG; }

int32_t gpda_mc_set_resample_times(gpda_mc *m, int32_t r) {
    if (!m || r < 1) return mfail(m, GPDA_ERR_ARG, "reSampleTimes must be >= 1");
    m->R = r;
    return GPDA_OK;
}

int32_t gpda_mc_set_seed(gpda_mc *m, uint64_t seed) {
    if (!m) return GPDA_ERR_ARG;
    m->seed = seed;
    return GPDA_OK;
}

int32_t gpda_mc_set_model(gpda_mc *m, const gpda_model *mm) {
    if (!m || !mm) return GPDA_ERR_ARG;
    if (!(mm->rc_r0 > 0.0f)) return mfail(m, GPDA_ERR_ARG, "rc_r0");
    m->model = *mm;
    return GPDA_OK;
}

int32_t gpda_mc_gpu_uuid(gpda_mc *m, char *out) {
    if (!m || !out) return GPDA_ERR_ARG;
    cudaDeviceProp prop;
    MCK(cudaGetDeviceProperties(&prop, m->devid));
    std::memcpy(out, prop.uuid.bytes, 16);
    return GPDA_OK;
}

int32_t gpda_mc_set_hist_bins(gpda_mc *m, int32_t nbins) {
    if (!m || nbins < 1 || nbins > GPDA_MAX_BINS) return mfail(m, GPDA_ERR_ARG, "nbins");
    m->nbins = nbins;
    return GPDA_OK;
}

int32_t gpda_mc_init_data_gpu(gpda_mc *m, const int64_t *istart, const int64_t *start,
                              const int64_t *stop, const int32_t *phCount, int64_t n_bursts,
                              int64_t sz_tag, const int64_t *burst_ad, const int64_t *burst_dd,
                              const float *T, const float *SgDivSr, float clk_p,
                              float bg_ad_rate, float bg_dd_rate) {
    if (!m) return GPDA_ERR_ARG;
    if (n_bursts < 1 || n_bursts > (int64_t)INT32_MAX || sz_tag < 0 || !istart || !start || !stop ||
        !phCount || !T || (sz_tag > 0 && (!burst_ad || !burst_dd)))
        return mfail(m, GPDA_ERR_ARG, "init_data_gpu arguments");
    for (int64_t b = 0; b < n_bursts; ++b) {
        if (phCount[b] < 0 || istart[b] < 0 || istart[b] + phCount[b] > sz_tag)
            return mfail(m, GPDA_ERR_ARG, "photon range of burst " + std::to_string(b) + " outside burst_ad/dd");
    }
    if (!(clk_p > 0.0f)) return mfail(m, GPDA_ERR_ARG, "clk_p");
    MCK(cudaSetDevice(m->devid));
    MCK(cudaDeviceSynchronize());
    void *old[] = {m->dStart, m->dStop, m->dIstart, m->dAd, m->dDd, m->dPh, m->dT, m->dSg};
    for (void *p : old)
        if (p) cudaFree(p);
    m->dStart = m->dStop = m->dIstart = m->dAd = m->dDd = nullptr;
    m->dPh = nullptr; m->dT = m->dSg = nullptr;
    const size_t B = (size_t)n_bursts;
    MCK(cudaMalloc(&m->dStart, 8 * B));
    MCK(cudaMalloc(&m->dStop, 8 * B));
    MCK(cudaMalloc(&m->dIstart, 8 * B));
    MCK(cudaMalloc(&m->dPh, 4 * B));
    MCK(cudaMalloc(&m->dT, 4 * B));
    MCK(cudaMalloc(&m->dSg, 4 * B));
    MCK(cudaMalloc(&m->dAd, 8 * std::max<size_t>(sz_tag, 1)));
    MCK(cudaMalloc(&m->dDd, 8 * std::max<size_t>(sz_tag, 1)));
    MCK(cudaMemcpy(m->dStart, start, 8 * B, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->dStop, stop, 8 * B, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->dIstart, istart, 8 * B, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->dPh, phCount, 4 * B, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->dT, T, 4 * B, cudaMemcpyHostToDevice));
    if (SgDivSr) MCK(cudaMemcpy(m->dSg, SgDivSr, 4 * B, cudaMemcpyHostToDevice));
    if (sz_tag > 0) {
        MCK(cudaMemcpy(m->dAd, burst_ad, 8 * (size_t)sz_tag, cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(m->dDd, burst_dd, 8 * (size_t)sz_tag, cudaMemcpyHostToDevice));
    }
    m->B = n_bursts;
    m->sz_tag = sz_tag;
    m->clk_p = clk_p;
    m->bg_ad = bg_ad_rate;
    m->bg_dd = bg_dd_rate;
    m->inited = true;
    return GPDA_OK;
}

int32_t gpda_mc_set_nstates(gpda_mc *m, int32_t n, int32_t sid) {
    if (!valid_sid(m, sid)) return mfail(m, GPDA_ERR_ARG, "sid");
    if (n < 2 || n > GPDA_MAX_STATES) return mfail(m, GPDA_ERR_ARG, "n states must be in [2,8]");
    McStream &s = m->streams[sid];
    int r = n;
    if (s.s_n != n) {
        r = s.s_n;
        MCK(cudaSetDevice(m->devid));
        MCK(cudaStreamSynchronize(s.st));
        s.s_n = n;
        s.have_params = false;
    }
    return r;
}

int32_t gpda_mc_set_params(gpda_mc *m, int32_t n, int32_t sid, const float *args, int32_t nargs) {
    if (!valid_sid(m, sid)) return mfail(m, GPDA_ERR_ARG, "sid");
    if (n < 2 || n > GPDA_MAX_STATES || !args) return mfail(m, GPDA_ERR_ARG, "n or args");
    if (nargs != n * (n + 1)) return 0;   // genMatK's size check fails (eigenhelper.cpp:5-8)
    McStream &s = m->streams[sid];
    MCK(cudaSetDevice(m->devid));
    MCK(cudaStreamSynchronize(s.st));
    int r = build_params(n, args, m->model.gamma, m->model.crosstalk, false, s.hParams);
    if (r != 0) return mfail(m, GPDA_ERR_ARG, "invalid parameter vector");
    MCK(cudaMemcpyAsync(s.dParams, s.hParams, sizeof(DevParams), cudaMemcpyHostToDevice, s.st));
    MCK(cudaStreamSynchronize(s.st));
    s.s_n = n;
    s.have_params = true;
    return 1;
}

int32_t gpda_mc_setBurstBd(gpda_mc *m, int32_t cstart, int32_t cstop, int32_t sid) {
    if (!valid_sid(m, sid)) return mfail(m, GPDA_ERR_ARG, "sid");
    if (!m->inited) return mfail(m, GPDA_ERR_STATE, "init_data_gpu first");
    const int sz = (int)m->B;
    int rcstart = cstart, rcstop = cstop;
    if (cstop >= sz || cstop < 0) rcstop = sz;
    if (cstart >= rcstop || cstart < 0) rcstart = 0;  // cstart == -1: the whole data set
    int N = rcstop - rcstart;
    McStream &s = m->streams[sid];
    if (s.end - s.begin != N) {
        s.begin = rcstart;
        s.end = rcstop;
    }
    size_t need = (size_t)N * (size_t)m->R;
    if (need > s.cap) {
        MCK(cudaSetDevice(m->devid));
        MCK(cudaStreamSynchronize(s.st));
        if (s.dMcE) cudaFree(s.dMcE);
        if (s.hMcE) cudaFreeHost(s.hMcE);
        s.dMcE = nullptr; s.hMcE = nullptr; s.cap = 0;
        MCK(cudaMalloc(&s.dMcE, sizeof(float) * std::max<size_t>(need, 1)));
        MCK(cudaHostAlloc(&s.hMcE, sizeof(float) * std::max<size_t>(need, 1), cudaHostAllocDefault));
        s.cap = need;
    }
    return N;
}

int32_t gpda_mc_init_randstate(gpda_mc *m, int32_t N, int32_t sid) {
    if (!valid_sid(m, sid)) return mfail(m, GPDA_ERR_ARG, "sid");
    m->streams[sid].oldN = (N == -1) ? (int)m->B : N;
    return GPDA_OK;
}

int32_t gpda_mc_set_params_buff(gpda_mc *m, int32_t oldS_n, int32_t N, int32_t sid) {
    (void)oldS_n; (void)N;
    if (!valid_sid(m, sid)) return mfail(m, GPDA_ERR_ARG, "sid");
    return GPDA_OK;
}

int32_t gpda_mc_run_kernel(gpda_mc *m, int32_t N, int32_t sid) {
    if (!valid_sid(m, sid)) return mfail(m, GPDA_ERR_ARG, "sid");
    McStream &s = m->streams[sid];
    if (!m->inited || !s.have_params) return mfail(m, GPDA_ERR_STATE, "init_data_gpu and set_params first");
    if (N < 0 || N > m->B) return mfail(m, GPDA_ERR_ARG, "N");
    if ((size_t)N * (size_t)m->R > s.cap) return mfail(m, GPDA_ERR_STATE, "setBurstBd for this N first");
    MCK(cudaSetDevice(m->devid));
    RcArgs a{};
    a.start = m->dStart; a.stop = m->dStop; a.istart = m->dIstart;
    a.burst_ad = m->dAd; a.burst_dd = m->dDd; a.phCount = m->dPh; a.T = m->dT;
    a.params = s.dParams;
    a.mcE = s.dMcE;
    a.hist = s.dHist;
    a.limit_hits = m->dLimit;
    a.b0 = 0;
    a.nb = N;
    a.R = m->R;
    a.nbins = m->nbins;
    a.seed = m->seed + (uint64_t)sid;
    a.pword = s.calls++;
    a.clk_p = m->clk_p; a.bg_ad_rate = m->bg_ad; a.bg_dd_rate = m->bg_dd;
    a.gamma = m->model.rc_gamma; a.de = m->model.rc_de; a.ct = m->model.rc_ct; a.r0 = m->model.rc_r0;
    MCK(cudaMemsetAsync(s.dHist, 0, sizeof(unsigned long long) * m->nbins, s.st));
    MCK(launch_rc(a, s.st));
    size_t cnt = (size_t)N * m->R;
    if (cnt) MCK(cudaMemcpyAsync(s.hMcE, s.dMcE, sizeof(float) * cnt, cudaMemcpyDeviceToHost, s.st));
    MCK(cudaMemcpyAsync(s.hHist, s.dHist, sizeof(unsigned long long) * m->nbins, cudaMemcpyDeviceToHost, s.st));
    return GPDA_OK;
}

int32_t gpda_mc_streamQuery(gpda_mc *m, int32_t sid) {
    if (!valid_sid(m, sid)) return 0;
    cudaSetDevice(m->devid);
    cudaError_t e = cudaStreamQuery(m->streams[sid].st);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return mfail(m, GPDA_ERR_CUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(e));
}

float *gpda_mc_hmcE(gpda_mc *m, int32_t sid) {
    if (!valid_sid(m, sid)) return nullptr;
    return m->streams[sid].hMcE;
}

int32_t gpda_mc_hist(gpda_mc *m, int32_t sid, float *hist_out) {
    if (!valid_sid(m, sid) || !hist_out) return mfail(m, GPDA_ERR_ARG, "sid or hist_out");
    McStream &s = m->streams[sid];
    MCK(cudaSetDevice(m->devid));
    MCK(cudaStreamSynchronize(s.st));
    for (int i = 0; i < m->nbins; ++i) hist_out[i] = (float)s.hHist[i];
    return GPDA_OK;
}

}  // extern "C"
