// Drives the `mc` drop-in (include/gpda_mc.hpp) through gpuWorker::run's call
// sequence (src/gpuWorker.cpp:71-81) on one stream and writes hmcE and the
// device histogram to a binary file for comparison with the oracle.
//
// usage: mc_dropin <in.bin> <out.bin>
//   in.bin: int64 B, int64 sz_tag, int32 n, int32 R, int32 nbins, uint64 seed,
//           float clk_p, bg_ad, bg_dd, int32 sid, int32 cstart, int32 cstop,
//           then istart[B], start[B], stop[B] (int64), phCount[B] (int32),
//           burst_ad[sz_tag], burst_dd[sz_tag] (int64), T[B], SgDivSr[B] (float),
//           args[n(n+1)] (float)
//   out.bin: int32 N, float hmcE[N*R], float hist[nbins]
#include <cstdio>
#include <vector>

#include "gpda_mc.hpp"

template <class T> static bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }

int main(int argc, char **argv) {
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
    int streamNum = 0;
    pdamc.getStreams(&streamNum);
    pdamc.set_seed(seed);
    pdamc.set_hist_bins(nbins);
    if (R != pdamc.reSampleTimes) pdamc.set_reSampleTimes(R);
    pdamc.init_data_gpu(istart, start, stop, ph, (long)sz_tag, bad.data(), bdd.data(), T, sg, clk_p,
                        bg_ad, bg_dd);
    pdamc.get_max_conversion_capacity();
    // gpuWorker::run, state 2 (src/gpuWorker.cpp:71-81)
    int Nprev = 0;
    int oldS_n = pdamc.set_nstates(n, sid);
    if (!pdamc.set_params(n, sid, args)) { fprintf(stderr, "set_params rejected\n"); return 3; }
    int N_sid = pdamc.setBurstBd(cstart, cstop, sid);
    if (N_sid != Nprev) pdamc.init_randstate(N_sid, sid);
    if (oldS_n != n || N_sid != Nprev) pdamc.set_params_buff(oldS_n, N_sid, sid);
    pdamc.run_kernel(N_sid, sid);
    // state 3 -> 4 (src/gpuWorker.cpp:51-58)
    while (!pdamc.streamQuery(sid)) {
    }
    std::vector<float> hist(nbins);
    pdamc.hist(sid, hist.data());
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 2;
    fwrite(&N_sid, 4, 1, o);
    fwrite(pdamc.hmcE[sid], sizeof(float), (size_t)N_sid * R, o);
    fwrite(hist.data(), sizeof(float), nbins, o);
    fclose(o);
    printf("streams=%d workers=%d N=%d\n", streamNum, pdamc.workerNum.load(), N_sid);
    return 0;
}
