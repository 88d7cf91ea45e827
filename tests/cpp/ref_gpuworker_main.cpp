// Runs the reference's own GPU thread, gpuWorker::run (src/gpuWorker.cpp:38-88,
// compiled unchanged from the reference's sources against include/gpda_mc.hpp),
// and plays the stream thread's side of the hand-off the way
// streamWorker::run does (src/streamWorker.cpp:146-184): parameters in,
// dataready = 2, wait for dataready == 4, read hmcE[sid]. Writes the values
// and the device histogram like tests/cpp/mc_dropin.cpp.
//
// usage: ref_gpuworker <in.bin> <out.bin>   (file formats as mc_dropin.cpp)
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <mutex>
#include <thread>
#include <vector>

#include "gpuWorker.hpp"

template <class T> static bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }

int main(int argc, char **argv) {
    using namespace std::chrono_literals;
    if (argc != 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 2; }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t B, sz_tag; int32_t n, R, nbins, sid, cstart, cstop; uint64_t seed; float clk_p, bg_ad, bg_dd;
    bool ok = rd(f, &B, 1) && rd(f, &sz_tag, 1) && rd(f, &n, 1) && rd(f, &R, 1) && rd(f, &nbins, 1) &&
              rd(f, &seed, 1) && rd(f, &clk_p, 1) && rd(f, &bg_ad, 1) && rd(f, &bg_dd, 1) &&
              rd(f, &sid, 1) && rd(f, &cstart, 1) && rd(f, &cstop, 1);
    std::vector<int64_t> istart(B), start(B), stop(B), bad(sz_tag), bdd(sz_tag);
    std::vector<int> ph(B);
    std::vector<float> T(B), sg(B), args(n * (n + 1));
    ok = ok && rd(f, istart.data(), B) && rd(f, start.data(), B) && rd(f, stop.data(), B) &&
         rd(f, ph.data(), B) && rd(f, bad.data(), sz_tag) && rd(f, bdd.data(), sz_tag) &&
         rd(f, T.data(), B) && rd(f, sg.data(), B) && rd(f, args.data(), args.size());
    fclose(f);
    if (!ok) { fprintf(stderr, "short input\n"); return 2; }

    mc pdamc(0, 2, 0, 0, false);
    pdamc.set_seed(seed);
    pdamc.set_hist_bins(nbins);
    if (R != pdamc.reSampleTimes) pdamc.set_reSampleTimes(R);
    pdamc.init_data_gpu(istart, start, stop, ph, (long)sz_tag, bad.data(), bdd.data(), T, sg, clk_p,
                        bg_ad, bg_dd);
    int streamNum = 0;
    pdamc.getStreams(&streamNum);
    if (sid < 0 || sid >= streamNum) { fprintf(stderr, "sid out of range\n"); return 2; }
    // the shared state main() allocates (src/main.cpp:27-39)
    std::vector<std::mutex> m(streamNum);
    std::vector<std::condition_variable> cv(streamNum);
    std::vector<int> dataready(streamNum, 0), s_n(streamNum, 0), ga_start(streamNum, 0),
        ga_stop(streamNum, 0), N(streamNum, 0);
    std::vector<std::vector<float>> params(streamNum);
    gpuWorker gw(&pdamc, streamNum, &sg, nbins, m.data(), cv.data(), dataready.data(), s_n.data(),
                 params.data(), ga_start.data(), ga_stop.data(), N.data(), 0);
    std::thread gpu(&gpuWorker::run, &gw, pdamc.sz_burst);
    {
        std::unique_lock<std::mutex> lck(m[sid]);
        s_n[sid] = n;
        params[sid] = args;
        ga_start[sid] = cstart;
        ga_stop[sid] = cstop;
        dataready[sid] = 2;
    }
    cv[sid].notify_one();
    int got = 0;
    for (int tries = 0; tries < 240 && !got; ++tries) {      // at most 2 minutes
        std::unique_lock<std::mutex> lck(m[sid]);
        got = cv[sid].wait_for(lck, 500ms, [&] { return dataready[sid] == 4; });
    }
    std::vector<float> vals, hist(nbins);
    int Nsid = 0;
    if (got) {
        Nsid = N[sid];
        vals.assign(pdamc.hmcE[sid], pdamc.hmcE[sid] + (size_t)Nsid * pdamc.reSampleTimes);
        pdamc.hist(sid, hist.data());
    }
    pdamc.workerNum.store(0);   // ends gpuWorker::run's loop
    gpu.join();
    if (!got) { fprintf(stderr, "gpuWorker never reached dataready == 4\n"); return 4; }
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 2;
    fwrite(&Nsid, 4, 1, o);
    fwrite(vals.data(), sizeof(float), vals.size(), o);
    fwrite(hist.data(), sizeof(float), nbins, o);
    fclose(o);
    printf("streams=%d N=%d\n", streamNum, Nsid);
    return 0;
}
