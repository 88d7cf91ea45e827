// mcref_harness.cu — runs the reference's own Monte-Carlo kernel (mc_kernel,
// src/mc.cu:83-197) with its own RNG set-up (setup_kernel, src/gen_rand.cuh:7-25,
// seeded as mc::init_randstate does, src/mc.cu:366-454) and records every
// draw its helpers make, for the oracle's replay (orc_rc_replay).
//
// TEST INFRASTRUCTURE ONLY. oracle/build_mcref.py extracts mc_kernel's text
// and copies gen_rand.cuh and binom.cuh from the reference tree into the
// git-ignored oracle/_ref/mcref/, and compiles this file against them into
// oracle/_ref/libmcref.so. Nothing of the reference is committed; nothing
// here is shipped or linked by the product.
//
// What this file supplies that mc_kernel takes from elsewhere:
//   - rk_state and retype as src/mc.hpp:19-30 and src/loadHdf5.hpp:8 declare
//     them (binom.cuh and mc_kernel name their fields and types);
//   - matXfMapper: the kernel's one use of Eigen (src/mc.cu:112,122) is a
//     column-major accessor over the K table, m(i, j) = data[j * rows + i];
//   - recorders: curand_uniform, curand_normal and curand_poisson (inside
//     gen_rand.cuh's helpers) and drawTau, drawE and rk_binomial (called by
//     mc_kernel) are redirected by macros to wrappers that call the original
//     and append (kind, value[, argument]) to the calling thread's tape. The
//     tape format is orc_tape_rec (oracle/gpda_oracle.h).
#include <cuda_runtime.h>
#include <curand.h>
#include <curand_kernel.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

using std::min;

typedef float retype;
typedef struct {
    unsigned int xor128[4];
    double gauss;
    int has_gauss;
    int has_binomial;
    int nsave, m;
    double psave, r, q, fm, p1, xm, xl, xr, c, laml, lamr, p2, p3, p4;
} rk_state;

struct matXfMapper {
    const float *data;
    int rows;
    __device__ matXfMapper(float *d, int r, int) : data(d), rows(r) {}
    __device__ float operator()(int i, int j) const { return data[j * rows + i]; }
};

// ---------------------------------------------------------------- tape
struct TapeRec {
    int32_t tag;     // kind | (binomial n << 8)
    int32_t i;
    double d;
};
enum { kU = 1, kTau = 2, kN = 3, kE = 4, kP = 5, kB = 6 };

__device__ TapeRec *g_tape;
__device__ int32_t *g_tape_len;
__device__ int32_t g_tape_cap;

__device__ __forceinline__ void tape_put(int32_t tag, int32_t i, double d) {
    if (g_tape == nullptr) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t k = g_tape_len[t]++;
    if (k < g_tape_cap) g_tape[(size_t)t * g_tape_cap + k] = TapeRec{tag, i, d};
}

__device__ float rec_uniform(curandStateScrambledSobol64 *s) {
    const float v = curand_uniform(s);
    tape_put(kU, 0, (double)v);
    return v;
}
__device__ float rec_normal(curandStateScrambledSobol64 *s) {
    const float v = curand_normal(s);
    tape_put(kN, 0, (double)v);
    return v;
}
__device__ unsigned int rec_poisson(curandStateScrambledSobol64 *s, double lambda) {
    const unsigned int v = curand_poisson(s, lambda);
    tape_put(kP, (int32_t)v, lambda);
    return v;
}
#define curand_uniform(s) rec_uniform(s)
#define curand_normal(s) rec_normal(s)
#define curand_poisson(s, l) rec_poisson(s, l)
#include "binom.cuh"
#include "gen_rand.cuh"
#undef curand_uniform
#undef curand_normal
#undef curand_poisson

__device__ float rec_drawTau(float k, curandStateScrambledSobol64 *st, int randN = 10,
                             float precision = 1e-6) {
    const float v = drawTau(k, st, randN, precision);
    tape_put(kTau, 0, (double)v);
    return v;
}
__device__ float rec_drawE(float e, float r0, float v, curandStateScrambledSobol64 *st) {
    const float x = drawE(e, r0, v, st);
    tape_put(kE, 0, (double)x);
    return x;
}
__device__ long rec_rk_binomial(rk_state *st, int n, double p) {
    const long v = rk_binomial(st, n, p);
    tape_put(kB | (n << 8), (int32_t)v, p);
    return v;
}
// diagnostics (g_tape_debug): draw_P_B_Tr's time bin and photon total as
// the kernel passes them (kinds 7 and 8, before the call's own records)
__device__ int32_t g_tape_debug;
__device__ bool rec_draw_P_B_Tr(float *bc, float *totPhoton, int timebin, float *timesp, float bg_rate,
                                curandStateScrambledSobol64 *state) {
    if (g_tape_debug) {
        tape_put(7, 0, (double)*timesp);
        tape_put(8, 0, (double)*totPhoton);
    }
    return draw_P_B_Tr(bc, totPhoton, timebin, timesp, bg_rate, state);
}
#define drawTau rec_drawTau
#define drawE rec_drawE
#define rk_binomial rec_rk_binomial
#define draw_P_B_Tr rec_draw_P_B_Tr
#include "mc_kernel.inc"
#undef drawTau
#undef drawE
#undef rk_binomial
#undef draw_P_B_Tr

// The thread-to-burst shift mc_kernel computes, idx = tidx >> (int)log2((double)R)
// (src/mc.cu:101): the same expression on the device, for R.
__global__ void shift_probe(int R, int *out) { *out = (int)log2((double)R); }

// ---------------------------------------------------------------- host
namespace {

template <class T>
T *dev_copy(const T *h, size_t n, int *err) {
    T *d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * (n ? n : 1)) != cudaSuccess) { *err = 1; return nullptr; }
    if (h && n && cudaMemcpy(d, h, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) *err = 1;
    return d;
}

}  // namespace

extern "C" {

// The shift mc_kernel uses on this device for reSampleTimes = R (-1 on a
// CUDA error). With this toolchain it can be one short of log2(R): then the
// kernel gives every burst 2^shift samples and its N * R threads reach
// bursts up to N * R / 2^shift - 1, past N.
int mcref_shift(int32_t R) {
    int *d = nullptr, h = -1;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return -1;
    shift_probe<<<1, 1>>>(R, d);
    if (cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) h = -1;
    cudaFree(d);
    return h;
}

// Runs setup_kernel + mc_kernel with reSampleTimes = R (a power of two) as
// mc::init_randstate and mc::run_kernel do, over the nb bursts given, and
// copies the values back. The kernel's thread-to-burst shift s (mcref_shift)
// decides the layout: it is launched for N = nb * 2^s / R bursts, so that its
// N * R threads map onto exactly the nb bursts given, 2^s samples each, and
// no thread reads past them; *r_eff = 2^s and mcE[nb * 2^s] is (burst,
// sample)-major. tape_cap > 0: the draws of thread t go to
// tape[t * tape_cap ...] (16-byte records) and their count to tape_len[t];
// debug != 0 adds the diagnostic records (kinds 7, 8; not replayable).
// Returns 0, or a CUDA / cuRAND error code (message on stderr).
int mcref_run(const int64_t *start, const int64_t *stop, const int64_t *istart,
              const int32_t *phCount, int64_t nb, const int64_t *burst_ad,
              const int64_t *burst_dd, int64_t nph, const float *T, float clk_p,
              float bg_ad_rate, float bg_dd_rate, int32_t s_n, const float *gpe,
              const float *gpv, const float *gpk, const float *gpp_i2j, const float *gpp,
              int32_t R, int32_t tape_cap, float *mcE_out, void *tape_out,
              int32_t *tape_len_out, int32_t debug, int32_t *r_eff) {
    if (nb < 1 || R < 1 || (R & (R - 1)) != 0 || s_n < 2) return -1;
    const int sh = mcref_shift(R);
    if (sh < 0 || sh > 20) return -1;
    const int64_t reff = (int64_t)1 << sh;
    if ((nb * reff) % R != 0 || nb * reff > (1 << 22)) return -1;
    const int nkern = (int)(nb * reff / R);          // the kernel's N
    const int NN = (int)(nb * reff);                 // = nkern * R threads
    *r_eff = (int32_t)reff;
    int err = 0;
    int64_t *d_start = dev_copy(start, nb, &err), *d_stop = dev_copy(stop, nb, &err);
    int64_t *d_istart = dev_copy(istart, nb, &err);
    int32_t *d_ph = dev_copy(phCount, nb, &err);
    int64_t *d_ad = dev_copy(burst_ad, nph, &err), *d_dd = dev_copy(burst_dd, nph, &err);
    float *d_T = dev_copy(T, nb, &err);
    float *d_e = dev_copy(gpe, s_n, &err), *d_v = dev_copy(gpv, s_n, &err);
    float *d_k = dev_copy(gpk, (size_t)s_n * s_n, &err);
    float *d_pij = dev_copy(gpp_i2j, (size_t)s_n * s_n, &err);
    float *d_p = dev_copy(gpp, s_n, &err);
    float *d_scratch = dev_copy<float>(nullptr, (size_t)NN * s_n, &err);
    float *d_mcE = dev_copy<float>(nullptr, NN, &err);
    rk_state *d_states = dev_copy<rk_state>(nullptr, NN, &err);
    curandStateScrambledSobol64 *d_q = dev_copy<curandStateScrambledSobol64>(nullptr, NN, &err);
    unsigned long long *d_dir = dev_copy<unsigned long long>(nullptr, (size_t)NN * 64, &err);
    unsigned long long *d_scr = dev_copy<unsigned long long>(nullptr, NN, &err);
    TapeRec *d_tape = nullptr;
    int32_t *d_tlen = nullptr;
    if (tape_cap > 0) {
        d_tape = dev_copy<TapeRec>(nullptr, (size_t)NN * tape_cap, &err);
        d_tlen = dev_copy<int32_t>(nullptr, NN, &err);
        if (!err && cudaMemset(d_tlen, 0, sizeof(int32_t) * NN) != cudaSuccess) err = 1;
    }
    int rc = 0;
    if (err) {
        fprintf(stderr, "mcref: allocation or copy failed: %s\n", cudaGetErrorString(cudaGetLastError()));
        rc = 2;
    }
    // the direction vectors and scramble constants of 20,000 dimensions,
    // repeated every 20,000 threads (src/mc.cu:312-314, 426-444)
    curandDirectionVectors64_t *hv = nullptr;
    unsigned long long *hs = nullptr;
    if (!rc && (curandGetDirectionVectors64(&hv, CURAND_SCRAMBLED_DIRECTION_VECTORS_64_JOEKUO6) !=
                    CURAND_STATUS_SUCCESS ||
                curandGetScrambleConstants64(&hs) != CURAND_STATUS_SUCCESS)) {
        fprintf(stderr, "mcref: cuRAND direction vectors unavailable\n");
        rc = 3;
    }
    for (int n0 = 0; !rc && n0 < NN; n0 += 20000) {
        const int size = min(20000, NN - n0);
        if (cudaMemcpy(d_scr + n0, hs, sizeof(unsigned long long) * size, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_dir + (size_t)n0 * 64, hv, sizeof(curandDirectionVectors64_t) * size,
                       cudaMemcpyHostToDevice) != cudaSuccess)
            rc = 4;
    }
    int minGrid = 0, blockSize = 0;
    if (!rc && cudaOccupancyMaxPotentialBlockSize(&minGrid, &blockSize, mc_kernel, 0, 0) != cudaSuccess) rc = 5;
    const int grid = blockSize > 0 ? (NN + blockSize - 1) / blockSize : 0;
    if (!rc) {
        TapeRec *none = nullptr;
        int32_t *nolen = nullptr;
        cudaMemcpyToSymbol(g_tape, &none, sizeof(none));
        cudaMemcpyToSymbol(g_tape_len, &nolen, sizeof(nolen));
        setup_kernel<<<grid, blockSize>>>(d_states, 0, NN, d_dir, d_scr, d_q);
        if (cudaDeviceSynchronize() != cudaSuccess) rc = 6;
    }
    if (!rc) {
        cudaMemcpyToSymbol(g_tape, &d_tape, sizeof(d_tape));
        cudaMemcpyToSymbol(g_tape_len, &d_tlen, sizeof(d_tlen));
        cudaMemcpyToSymbol(g_tape_cap, &tape_cap, sizeof(tape_cap));
        cudaMemcpyToSymbol(g_tape_debug, &debug, sizeof(debug));
        mc_kernel<<<grid, blockSize>>>(d_start, d_stop, d_ad, d_dd, d_istart, d_ph, d_T, clk_p,
                                       bg_ad_rate, bg_dd_rate, d_e, d_v, d_k, d_pij, d_p, d_scratch,
                                       nkern, s_n, d_q, d_states, d_mcE, R);
        if (cudaDeviceSynchronize() != cudaSuccess) rc = 7;
    }
    if (!rc && cudaMemcpy(mcE_out, d_mcE, sizeof(float) * NN, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 8;
    if (!rc && tape_cap > 0 &&
        (cudaMemcpy(tape_out, d_tape, sizeof(TapeRec) * (size_t)NN * tape_cap, cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(tape_len_out, d_tlen, sizeof(int32_t) * NN, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = 9;
    if (rc > 5) fprintf(stderr, "mcref: %s\n", cudaGetErrorString(cudaGetLastError()));
    void *bufs[] = {d_start, d_stop, d_istart, d_ph, d_ad, d_dd, d_T, d_e, d_v, d_k, d_pij, d_p,
                    d_scratch, d_mcE, d_states, d_q, d_dir, d_scr, d_tape, d_tlen};
    for (void *b : bufs)
        if (b) cudaFree(b);
    return rc;
}

}  // extern "C"
