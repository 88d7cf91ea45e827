// gpda_mc.hpp — C++ drop-in for the reference's `mc` engine object
// (src/mc.hpp:32-180), header-only over the C ABI in gpda.h.
//
// Same public members and method signatures as the reference, so the
// reference's gpuWorker::run (src/gpuWorker.cpp:38-88) and
// streamWorker::run (src/streamWorker.cpp:39-246) compile against it
// unchanged: set_nstates, set_params, setBurstBd, init_randstate,
// set_params_buff, run_kernel, streamQuery, hmcE[sid], reSampleTimes,
// workerNum, devid, gpuuuid, sz_burst.
//
// Error behaviour follows the reference: CUDA failures print the failing call
// and exit(EXIT_FAILURE) (src/cuda_tools.hpp:22-27); set_params returns false
// on a parameter vector of the wrong size (src/eigenhelper.cpp:5-8).
#pragma once

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gpda.h"

typedef float retype;

class mc {
  public:
    int devid;
    char gpuuuid[33];
    std::atomic_int workerNum;
    retype **hmcE;
    int *s_n;
    int sz_burst;
    int reSampleTimes;

    mc(int id, int _streamNum = 16, unsigned char debug = 0, std::uintmax_t hdf5size = 0,
       bool profiler = false)
        : devid(id), hmcE(nullptr), s_n(nullptr), sz_burst(0), reSampleTimes(4) {
        int32_t st = 0;
        h_ = gpda_mc_create(id, _streamNum, debug, (uint64_t)hdf5size, profiler ? 1 : 0, &st);
        if (!h_) die("gpda_mc_create", st);
        streamNum_ = gpda_mc_stream_num(h_);
        workerNum.store(streamNum_);
        std::memset(gpuuuid, 0, sizeof(gpuuuid));
        gpda_mc_gpu_uuid(h_, gpuuuid);
        hmcE = new retype *[streamNum_]();
        s_n = new int[streamNum_]();
        reSampleTimes = gpda_mc_resample_times(h_);
    }
    ~mc() {
        gpda_mc_destroy(h_);
        delete[] hmcE;
        delete[] s_n;
    }
    mc(const mc &) = delete;
    mc &operator=(const mc &) = delete;

    // the C ABI selects the device on every call
    void set_gpuid() {}

    // `getStreams(&streamNum)` is how the reference reads the stream count
    void getStreams(int *numStream) {
        if (numStream) *numStream = streamNum_;
    }

    void init_data_gpu(std::vector<int64_t> &istart, std::vector<int64_t> &start,
                       std::vector<int64_t> &stop, std::vector<int> &phCount, long _sz_tag,
                       int64_t *burst_ad, int64_t *burst_dd, std::vector<float> &T_burst_duration,
                       std::vector<float> &SgDivSr, float &iclk_p, float &ibg_ad_rate,
                       float &ibg_dd_rate) {
        static_assert(sizeof(int) == sizeof(int32_t), "phCount is int32");
        check(gpda_mc_init_data_gpu(h_, istart.data(), start.data(), stop.data(),
                                    reinterpret_cast<const int32_t *>(phCount.data()),
                                    (int64_t)start.size(), (int64_t)_sz_tag, burst_ad, burst_dd,
                                    T_burst_duration.data(), SgDivSr.data(), iclk_p, ibg_ad_rate,
                                    ibg_dd_rate),
              "init_data_gpu");
        sz_burst = gpda_mc_sz_burst(h_);
        data_inited_ = true;
    }

    // the reference sizes an unused "conversion buffer" here; nothing to reserve
    bool get_max_conversion_capacity(int max_stateNum = 8) {
        (void)max_stateNum;
        return data_inited_;
    }

    int set_nstates(int n, int sid) {
        int r = check(gpda_mc_set_nstates(h_, n, sid), "set_nstates");
        s_n[sid] = n;
        return r;
    }

    bool set_params(int n, int sid, std::vector<float> &args) {
        int r = check(gpda_mc_set_params(h_, n, sid, args.data(), (int32_t)args.size()), "set_params");
        return r == 1;
    }

    int setBurstBd(int cstart, int cstop, int sid) {
        int N = check(gpda_mc_setBurstBd(h_, cstart, cstop, sid), "setBurstBd");
        hmcE[sid] = gpda_mc_hmcE(h_, sid);
        return N;
    }

    void set_reSampleTimes(int t) {
        check(gpda_mc_set_resample_times(h_, t), "set_reSampleTimes");
        reSampleTimes = t;
    }

    void init_randstate(int N, int sid) { check(gpda_mc_init_randstate(h_, N, sid), "init_randstate"); }

    void set_params_buff(int oldS_n, int N_sid, int sid) {
        check(gpda_mc_set_params_buff(h_, oldS_n, N_sid, sid), "set_params_buff");
    }

    void run_kernel(int N, int sid) {
        check(gpda_mc_run_kernel(h_, N, sid), "run_kernel");
        hmcE[sid] = gpda_mc_hmcE(h_, sid);
    }

    bool streamQuery(int sid) { return check(gpda_mc_streamQuery(h_, sid), "streamQuery") == 1; }

    void get_res(int sid, int N) { (void)sid; (void)N; }

    // additions: device-binned histogram of the last run (reference binning)
    void set_hist_bins(int nbins) { check(gpda_mc_set_hist_bins(h_, nbins), "set_hist_bins"); }
    void hist(int sid, float *out) { check(gpda_mc_hist(h_, sid, out), "hist"); }
    void set_seed(uint64_t seed) { check(gpda_mc_set_seed(h_, seed), "set_seed"); }
    gpda_mc *handle() { return h_; }

  private:
    gpda_mc *h_ = nullptr;
    int streamNum_ = 0;
    bool data_inited_ = false;

    int check(int rc, const char *what) {
        if (rc < 0) {
            std::fprintf(stderr, "%s returned %d (%s)\n", what, rc, gpda_mc_last_error(h_));
            std::exit(EXIT_FAILURE);
        }
        return rc;
    }
    [[noreturn]] static void die(const char *what, int st) {
        std::fprintf(stderr, "%s failed with status %d\n", what, st);
        std::exit(EXIT_FAILURE);
    }
};
