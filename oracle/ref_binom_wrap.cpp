// Host build of the reference's own binomial sampler (src/binom.cuh) for
// pinning the oracle. TEST INFRASTRUCTURE ONLY: compiled by oracle/build_ref.py
// from the reference tree into oracle/_ref/ (never committed, never shipped).
//
// binom.cuh needs only C math, an empty __device__ and the rk_state type of
// src/mc.hpp:19-30 (its fields are named by binom.cuh, so the declaration
// below has to match them).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>
using std::min;
#define __device__
typedef struct {
    unsigned int xor128[4];
    double gauss;
    int has_gauss;
    int has_binomial;
    int nsave, m;
    double psave, r, q, fm, p1, xm, xl, xr, c, laml, lamr, p2, p3, p4;
} rk_state;
#include REF_BINOM_CUH

extern "C" {
// count variates of Binomial(n, p) from one xorshift128 stream seeded by rk_seed
void ref_binomial_many(unsigned long long seed, int n, double p, long count, long *out) {
    rk_state st;
    rk_seed(seed, &st);
    for (long i = 0; i < count; ++i) out[i] = rk_binomial(&st, n, p);
}
// the reference's multinomial (csd_int_multinomial) for moment checks
void ref_multinomial_many(unsigned long long seed, int K, int N, const float *p, long count, int *out) {
    rk_state st;
    rk_seed(seed, &st);
    std::vector<float> pp(p, p + K);
    for (long i = 0; i < count; ++i) csd_int_multinomial(&st, K, N, pp.data(), out + i * K);
}
}
