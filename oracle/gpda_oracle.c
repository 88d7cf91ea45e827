/*
 * gpda_oracle.c — CPU oracle for the photon-burst Monte-Carlo PDA path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product). See
 * gpda_oracle.h for what is restated and which reference lines it follows.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fno-fast-math -shared -fPIC
 * (oracle/build_oracle.py). -ffp-contract=off is required: every FP32
 * operation must round exactly where the device code rounds.
 */
#include "gpda_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): multipliers and Weyl key increments from the
 * paper; 10 rounds, key bumped between rounds. */
#define PHX_M0 0xD2511F53u
#define PHX_M1 0xCD9E8D57u
#define PHX_W0 0x9E3779B9u
#define PHX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHX_M0 * c0;
        uint64_t p1 = (uint64_t)PHX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += PHX_W0; k1 += PHX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* One unit's draw stream: counter (block, sample, burst, param-set word). */
typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int idx;
} orc_rng;

static inline void rng_init(orc_rng *r, uint64_t seed, uint32_t pword, uint32_t b, uint32_t s) {
    r->key[0] = (uint32_t)seed;
    r->key[1] = (uint32_t)(seed >> 32);
    r->ctr[0] = 0; r->ctr[1] = s; r->ctr[2] = b; r->ctr[3] = pword;
    r->idx = 4;
}
/* the next draw starts a fresh block (the rest of the current one is dropped) */
static inline void rng_align(orc_rng *r) { r->idx = 4; }
static inline uint32_t rng_next(orc_rng *r) {
    if (r->idx == 4) {
        orc_philox4x32_10(r->ctr, r->key, r->buf);
        r->ctr[0] += 1u;
        r->idx = 0;
    }
    return r->buf[r->idx++];
}

/* ------------------------------------------------------------------ */
/* FP32 elementary functions, written from the mathematics (no libm, no
 * vendor code): identical operation order on the device makes them
 * bit-reproducible. Constants are float(1/k) etc., given in hex. */
static inline float f_from_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t bits_from_f(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

#define C_LN2_HI 0x1.62e430p-1f     /* float(ln 2) */
#define C_LN2_LO -0x1.05c610p-29f   /* ln 2 - C_LN2_HI */
#define C_LOG2E 0x1.715476p+0f
#define C_SQRT2 0x1.6a09e6p+0f

/* log(x): x = 2^e m, m in [sqrt(2)/2, sqrt(2)); log m = 2 atanh(s),
 * s = (m-1)/(m+1), atanh series to s^9. */
float orc_logf(float x) {
    if (x != x) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return x;
    uint32_t bits = bits_from_f(x);
    int e = 0;
    if ((bits >> 23) == 0u) {           /* subnormal: scale by 2^24 */
        x = x * 0x1p24f;
        bits = bits_from_f(x);
        e = -24;
    }
    e += (int)(bits >> 23) - 127;
    float m = f_from_bits((bits & 0x007FFFFFu) | 0x3F800000u);
    if (m > C_SQRT2) { m = m * 0.5f; e += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float poly = fmaf(z, fmaf(z, fmaf(z, 0x1.c71c72p-3f, 0x1.24924ap-2f), 0x1.99999ap-2f), 0x1.555556p-1f);
    float lm = fmaf(s * z, poly, 2.0f * s);
    float ef = (float)e;
    return fmaf(ef, C_LN2_HI, fmaf(ef, C_LN2_LO, lm));
}

/* exp(x): x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r to r^7. */
float orc_expf(float x) {
    if (x != x) return x;
    if (x > 88.72284f) return INFINITY;
    if (x < -103.97208f) return 0.0f;
    float kf = rintf(x * C_LOG2E);
    float r = fmaf(-kf, C_LN2_HI, x);
    r = fmaf(-kf, C_LN2_LO, r);
    float p = 0x1.a01a02p-13f;
    p = fmaf(p, r, 0x1.6c16c2p-10f);
    p = fmaf(p, r, 0x1.111112p-7f);
    p = fmaf(p, r, 0x1.555556p-5f);
    p = fmaf(p, r, 0x1.555556p-3f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int k = (int)kf;
    if (k >= -126 && k <= 127) return p * f_from_bits((uint32_t)(k + 127) << 23);
    int k1 = k / 2, k2 = k - k1;
    return (p * f_from_bits((uint32_t)(k1 + 127) << 23)) * f_from_bits((uint32_t)(k2 + 127) << 23);
}

/* cos(2 pi u) for u in [0,1]: fold to w in [0,1/2], cos(2 pi w) = sin(2 pi (1/4 - w)),
 * sine Taylor series to theta^13. */
float orc_cos2pif(float u) {
    float w = (u > 0.5f) ? 1.0f - u : u;
    float rr = 0.25f - w;
    float th = rr * 0x1.921fb6p+2f;
    float t2 = th * th;
    float p = 0x1.612462p-33f;
    p = fmaf(p, t2, -0x1.ae6456p-26f);
    p = fmaf(p, t2, 0x1.71de3ap-19f);
    p = fmaf(p, t2, -0x1.a01a02p-13f);
    p = fmaf(p, t2, 0x1.111112p-7f);
    p = fmaf(p, t2, -0x1.555556p-3f);
    p = fmaf(p, t2, 1.0f);
    return th * p;
}

/* Stirling correction fc(k) = ln k! - ((k+1/2) ln(k+1) - (k+1) + ln(2 pi)/2),
 * k = 0..9, from lgamma in double (Hoermann 1993, BTRD). */
static const float FC_TAB[10] = {
    8.106146680e-02f, 4.134069596e-02f, 2.767792568e-02f, 2.079067210e-02f,
    1.664469119e-02f, 1.387612882e-02f, 1.189670995e-02f, 1.041126526e-02f,
    9.255462183e-03f, 8.330563433e-03f};
/* ln k!, k = 0..9 */
static const float LF_TAB[10] = {
    0.0f, 0.0f, 0.693147182f, 1.791759491f, 3.178053856f,
    4.787491798f, 6.579251289f, 8.525161743f, 10.60460281f, 12.80182743f};
static const double FC_TAB_D[10] = {
    0.08106146679532733, 0.04134069595540946, 0.027677925684997717, 0.02079067210376584,
    0.01664469118982126, 0.013876128823072875, 0.011896709945893313, 0.010411265261973668,
    0.00925546218270945, 0.008330563433359472};

/* saturating float->int64 truncation with NaN -> 0 (PTX cvt.rzi.s64 semantics) */
static inline int64_t f2i64(double v) {
    if (v != v) return 0;
    if (v >= 9.2233720368547758e18) return INT64_MAX;
    if (v <= -9.2233720368547758e18) return INT64_MIN;
    return (int64_t)v;
}

/* ------------------------------------------------------------------ */
/* Host parameter derivation in double (the product derives the same way). */
typedef struct {
    int n;
    double E[ORC_MAXS], V[ORC_MAXS];
    double Kd[ORC_MAXS * ORC_MAXS];   /* column-major with leading dim n, diag = -column sum */
    double kexit[ORC_MAXS];
    double jump_cdf[ORC_MAXS * ORC_MAXS];
    double init_cdf[ORC_MAXS];
} orc_derived;

/* K(i,j) (rate j->i) from the reference's off-diagonal layout
 * (eigenhelper.cpp:4-22): i<j -> args[i*(n-1)+j-1], i>j -> args[i*(n-1)+j]. */
static inline float koff_at(const float *koff, int n, int i, int j) {
    return (i < j) ? koff[i * (n - 1) + j - 1] : koff[i * (n - 1) + j];
}

static int derive_double(int n, const float *args, orc_derived *d, int need_pi) {
    if (n < 1 || n > ORC_MAXS) return -1;
    const float *koff = args + n;
    const float *V = args + n * n;
    d->n = n;
    double kmax = 1.0;
    for (int i = 0; i < n; ++i) {
        float e = args[i], v = V[i];
        if (!(e >= 0.0f && e <= 1.0f)) return -1;
        if (!(v >= 0.0f && v < INFINITY)) return -1;
        d->E[i] = e; d->V[i] = v;
    }
    for (int j = 0; j < n; ++j) {
        double colsum = 0.0;
        for (int i = 0; i < n; ++i) {
            if (i == j) continue;
            float k = koff_at(koff, n, i, j);
            if (!(k >= 0.0f && k < INFINITY)) return -1;
            d->Kd[j * n + i] = (double)k;
            colsum += (double)k;
            if ((double)k > kmax) kmax = (double)k;
        }
        d->Kd[j * n + j] = -colsum;
        d->kexit[j] = colsum;
        double acc = 0.0;
        for (int i = 0; i < n; ++i) {
            if (colsum > 0.0) {
                if (i != j) acc += d->Kd[j * n + i];
                d->jump_cdf[j * ORC_MAXS + i] = acc / colsum;
            } else {
                d->jump_cdf[j * ORC_MAXS + i] = 1.0;
            }
        }
    }
    if (!need_pi) {
        for (int i = 0; i < n; ++i) d->init_cdf[i] = (double)(i + 1) / (double)n;
        return 0;
    }
    /* stationary distribution: K pi = 0 with the last equation replaced by
     * sum(pi) = 1, Gaussian elimination with partial pivoting. */
    double A[ORC_MAXS][ORC_MAXS + 1];
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) A[i][j] = d->Kd[j * n + i];
        A[i][n] = 0.0;
    }
    for (int j = 0; j < n; ++j) A[n - 1][j] = 1.0;
    A[n - 1][n] = 1.0;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        if (!(fabs(A[piv][c]) > 1e-13 * kmax)) return -2;
        if (piv != c)
            for (int k = 0; k <= n; ++k) { double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
        for (int r = c + 1; r < n; ++r) {
            double f = A[r][c] / A[c][c];
            for (int k = c; k <= n; ++k) A[r][k] = A[r][k] - f * A[c][k];
        }
    }
    double pi[ORC_MAXS];
    for (int r = n - 1; r >= 0; --r) {
        double s = A[r][n];
        for (int k = r + 1; k < n; ++k) s = s - A[r][k] * pi[k];
        pi[r] = s / A[r][r];
    }
    double sum = 0.0;
    for (int i = 0; i < n; ++i) { if (!(pi[i] > 0.0)) pi[i] = 0.0; sum += pi[i]; }
    if (!(sum > 0.0)) return -2;
    double acc = 0.0;
    for (int i = 0; i < n; ++i) { acc += pi[i] / sum; d->init_cdf[i] = acc; }
    return 0;
}

/* Reference float tables, in the reference's operation order:
 * genMatK (eigenhelper.cpp:4-22), genP_i2j (:24-38), genMatP (:39-53). */
static void ref_tables_f(int n, const float *args, float *K, float *P, float *pinit) {
    const float *koff = args + n;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            K[i + j * n] = (i == j) ? 0.0f : koff_at(koff, n, i, j);
    for (int j = 0; j < n; ++j)
        for (int ii = 0; ii < n; ++ii)
            if (ii != j) K[j + j * n] = K[j + j * n] - K[ii + j * n];
    for (int j = 0; j < n; ++j) {
        float sum = 0.0f;
        for (int ii = 0; ii < n; ++ii) if (ii != j) sum = sum + K[ii + j * n];
        for (int ii = 0; ii < n; ++ii)
            P[ii + j * n] = (ii != j) ? K[ii + j * n] / sum : 0.0f;
    }
    for (int i = 0; i < n; ++i) {
        float s = 0.0f;
        for (int j = 0; j < n; ++j) s = s + K[i + j * n];
        s = s - K[i + i * n];
        pinit[i] = s;
    }
}
static void ref_tables_d(int n, const float *args, double *K, double *P, double *pinit) {
    const float *koff = args + n;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            K[i + j * n] = (i == j) ? 0.0 : (double)koff_at(koff, n, i, j);
    for (int j = 0; j < n; ++j)
        for (int ii = 0; ii < n; ++ii)
            if (ii != j) K[j + j * n] = K[j + j * n] - K[ii + j * n];
    for (int j = 0; j < n; ++j) {
        double sum = 0.0;
        for (int ii = 0; ii < n; ++ii) if (ii != j) sum = sum + K[ii + j * n];
        for (int ii = 0; ii < n; ++ii)
            P[ii + j * n] = (ii != j) ? K[ii + j * n] / sum : 0.0;
    }
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s = s + K[i + j * n];
        s = s - K[i + i * n];
        pinit[i] = s;
    }
}

static inline int pda_bin(int A, int N, int nbins) {
    if (N <= 0 || A < 0) return -1;
    long long v = (long long)A * nbins / N;
    if (v >= nbins) v = nbins - 1;
    return (int)v;
}

/* Boost.Histogram regular axis on [0,1): z in double; inner bins only. */
static inline int ref_bin_d(double z, int nbins) {
    if (z < 1.0) {
        if (z >= 0.0) return (int)(z * (double)nbins);
        return -1;
    }
    return -1;
}

/* reciprocal tables of the sequential-search loops: 1.0f/k and 1.0/k */
static float inv_tab_f[64];
static double inv_tab_d[64];

/* photon mode: Binomial(n, eps_s) with n <= ORC_TABLE_N (and V_s = 0) is
 * drawn by inverting a tabulated CDF (one uniform) */
#define ORC_TABLE_N 511
#define ORC_TABLE_ROWS ((ORC_TABLE_N + 1) * (ORC_TABLE_N + 2) / 2)

/* Double-float arithmetic (hi + lo in two floats; Dekker/Knuth error-free
 * transformations with fmaf), as the device builds its binomial tables. */
typedef struct { float hi, lo; } orc_df;
static inline orc_df df_fast_sum(float a, float b) {
    float s = a + b;
    orc_df r = {s, b - (s - a)};
    return r;
}
static inline orc_df df_mul(orc_df a, orc_df b) {
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_fast_sum(p, e);
}
static inline orc_df df_add(orc_df a, orc_df b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e = e + (a.lo + b.lo);
    return df_fast_sum(s, e);
}
static inline orc_df df_div(float x, orc_df y) {
    float q = x / y.hi;
    orc_df qf = {q, 0.0f};
    orc_df qy = df_mul(qf, y);
    float r = (x - qy.hi) - qy.lo;
    return df_fast_sum(q, r / y.hi);
}
static inline orc_df df_div2(orc_df x, orc_df y) {
    float q = x.hi / y.hi;
    orc_df qf = {q, 0.0f};
    orc_df qy = df_mul(qf, y);
    orc_df nqy = {-qy.hi, -qy.lo};
    orc_df rem = df_add(x, nqy);
    return df_fast_sum(q, rem.hi / y.hi);
}
static inline orc_df df_recip(int k) {
    float kf = (float)k;
    float ih = 1.0f / kf;
    return df_fast_sum(ih, fmaf(-ih, kf, 1.0f) / kf);
}

/* CDF row of Binomial(nn, pp), pp <= 1/2, in double-float around the mode
 * (relative probabilities from w(m) = 1 upward then downward, total, running
 * sum times 1/total), clamped to 1 with out[nn] = 1, as the device builds it. */
/* Row nn of the photon-mode table for pp <= 1/2, in the device's order
 * (binom_table_kernel, one warp of TAB_LANES lanes per row): products of the
 * ratios inside TAB_LANES contiguous chunks on each side of the mode, chunk
 * products folded left to right, w(k) rounded to float; cumulative sums in
 * TAB_LANES chunks over k = 0..nn, chunk sums folded left to right. */
#define TAB_LANES 32
static void binom_cdf_row_df(float pp, int nn, float *out) {
    orc_df qq = df_fast_sum(1.0f, -pp);
    orc_df up = df_div(pp, qq);
    orc_df ppd = {pp, 0.0f};
    orc_df down = df_div2(qq, ppd);
    int m = (int)floorf((float)(nn + 1) * pp);
    if (m > nn) m = nn;
    orc_df wl[ORC_TABLE_N + 1];
    orc_df P[TAB_LANES];
    /* upward, k = m+1 .. nn */
    {
        int len = nn - m, C = (len + TAB_LANES - 1) / TAB_LANES;
        for (int l = 0; l < TAB_LANES; ++l) {
            int k0 = m + 1 + l * C, k1 = k0 + C - 1 < nn ? k0 + C - 1 : nn;
            orc_df w = {1.0f, 0.0f};
            for (int k = k0; k <= k1; ++k) {
                orc_df a = {(float)(nn - k + 1), 0.0f};
                w = df_mul(w, df_mul(df_mul(a, df_recip(k)), up));
                wl[k] = w;
            }
            P[l] = w;
        }
        for (int l = 0; l < TAB_LANES; ++l) {
            orc_df Q = {1.0f, 0.0f};
            for (int i = 0; i < l; ++i) Q = df_mul(Q, P[i]);
            int k0 = m + 1 + l * C, k1 = k0 + C - 1 < nn ? k0 + C - 1 : nn;
            for (int k = k0; k <= k1; ++k) {
                orc_df v = df_mul(Q, wl[k]);
                out[k] = v.hi + v.lo;
            }
        }
    }
    /* downward, k = m-1 .. 0 */
    {
        int len = m, C = (len + TAB_LANES - 1) / TAB_LANES;
        for (int l = 0; l < TAB_LANES; ++l) {
            int k0 = m - 1 - l * C, k1 = k0 - C + 1 > 0 ? k0 - C + 1 : 0;
            orc_df w = {1.0f, 0.0f};
            for (int k = k0; k >= k1; --k) {
                orc_df a = {(float)(k + 1), 0.0f};
                w = df_mul(w, df_mul(df_mul(a, df_recip(nn - k)), down));
                wl[k] = w;
            }
            P[l] = w;
        }
        for (int l = 0; l < TAB_LANES; ++l) {
            orc_df Q = {1.0f, 0.0f};
            for (int i = 0; i < l; ++i) Q = df_mul(Q, P[i]);
            int k0 = m - 1 - l * C, k1 = k0 - C + 1 > 0 ? k0 - C + 1 : 0;
            for (int k = k0; k >= k1; --k) {
                orc_df v = df_mul(Q, wl[k]);
                out[k] = v.hi + v.lo;
            }
        }
    }
    out[m] = 1.0f;
    /* cumulative sums */
    int C2 = (nn + 1 + TAB_LANES - 1) / TAB_LANES;
    orc_df T[TAB_LANES];
    for (int l = 0; l < TAB_LANES; ++l) {
        int c0 = l * C2, c1 = c0 + C2 < nn + 1 ? c0 + C2 : nn + 1;
        orc_df t = {0.0f, 0.0f};
        for (int k = c0; k < c1; ++k) {
            orc_df x = {out[k], 0.0f};
            t = df_add(t, x);
        }
        T[l] = t;
    }
    orc_df W = {0.0f, 0.0f};
    for (int i = 0; i < TAB_LANES; ++i) W = df_add(W, T[i]);
    orc_df invW = df_div(1.0f, W);
    for (int l = 0; l < TAB_LANES; ++l) {
        orc_df cum = {0.0f, 0.0f};
        for (int i = 0; i < l; ++i) cum = df_add(cum, T[i]);
        int c0 = l * C2, c1 = c0 + C2 < nn + 1 ? c0 + C2 : nn + 1;
        for (int k = c0; k < c1; ++k) {
            orc_df x = {out[k], 0.0f};
            cum = df_add(cum, x);
            orc_df v = df_mul(cum, invW);
            float c = v.hi + v.lo;
            out[k] = (k == nn) ? 1.0f : (c < 1.0f ? c : 1.0f);
        }
    }
}

/* the FP64 transcription's rows: the same recurrence in double */
static void binom_cdf_row_d(double pp, int nn, double *out) {
    double qq = 1.0 - pp;
    double ratio = pp / qq;
    double f = 1.0, base = qq;
    for (int e = nn; e > 0; e >>= 1) {
        if (e & 1) f = f * base;
        base = base * base;
    }
    double cum = 0.0;
    for (int k = 0; k <= nn; ++k) {
        if (k > 0) f = f * (((double)(nn - k + 1) * (1.0 / (double)k)) * ratio);
        cum = cum + f;
        out[k] = cum;
    }
}

#define ORC_MAX_SEG 65536
#define ORC_MAX_RESTART 256

/* ------------------------------------------------------------------ */
/* FP32 instantiation: bit-exact mirror of the device kernels. */
#define REAL float
#define RL(x) x##f
#define LOGR orc_logf
#define EXPR orc_expf
#define SQRTR sqrtf
#define FLOORR floorf
#define FABSR fabsf
#define FMAR fmaf
#define COS2PIR orc_cos2pif
#define COPYSIGNR copysignf
#define INFR INFINITY
#define FC_T FC_TAB
#define LF_T LF_TAB
#define INV_T inv_tab_f
#define PFX(x) f32_##x
#include "gpda_oracle_core.inc"

static void init_lf_d(void);

/* ---------------- replay of the reference kernel's recorded draws ----------------
 * The reference-kernel harness (oracle/mcref_harness.cu, built from the
 * reference's own mc_kernel, gen_rand.cuh and binom.cuh) records, per thread,
 * every draw mc_kernel's helpers make: the Sobol uniforms, drawTau's value,
 * the Poisson variates with their means, the normal and drawE's value, and
 * rk_binomial's (n, p, result). orc_rc_replay runs the oracle's own
 * mc_kernel body (rc_unit_body.inc, the same text unit_rc runs on Philox
 * draws) on those records and compares its mcE with the reference's. */
typedef struct {
    const orc_tape_rec *rec;
    int64_t len, pos;
    int32_t off_path;           /* a record of the wrong kind, or none left */
    orc_replay_stats *st;
} tape_src;

static const orc_tape_rec *tape_next(tape_src *t, int kind) {
    static const orc_tape_rec none = {0, 0, 0.0};
    if (t->off_path || t->pos >= t->len || (t->rec[t->pos].tag & 0xff) != kind) {
        t->off_path = 1;
        return &none;
    }
    return &t->rec[t->pos++];
}

static float tape_u(tape_src *t) { return (float)tape_next(t, ORC_TAPE_U)->d; }

static uint32_t f32_bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}

/* drawTau: the reference's value is used; the oracle's log of the same
 * uniform is compared with it in ulps */
static float tape_tau(tape_src *t, float k) {
    const float u = tape_u(t);
    const float ours = orc_logf(u) / (-k);
    const float ref = (float)tape_next(t, ORC_TAPE_TAU)->d;
    if (t->off_path) return INFINITY;   /* ends the trajectory: the unit is reported off path */
    {
        int64_t d = (int64_t)f32_bits(ours) - (int64_t)f32_bits(ref);
        if (d < 0) d = -d;
        if (d > t->st->tau_max_ulp) t->st->tau_max_ulp = d;
    }
    return ref;
}

/* draw_P_B_Tr for one time bin: the clip rule on the reference's Poisson
 * variate; its mean must be the float tdiff * rate the body computed */
static float tape_bg(tape_src *t, float tot, float tdiff, float rate) {
    const orc_tape_rec *p = tape_next(t, ORC_TAPE_P);
    const float lam = tdiff * rate;
    if (!t->off_path && (double)lam != p->d) t->st->lambda_mismatch += 1;
    const int sv = p->i;
    if ((float)sv <= tot) return (float)sv;
    return floorf(tot * tape_u(t));
}

/* drawE: the reference's value is used; the oracle's formula on the same
 * normal is compared with it */
static float tape_e(tape_src *t, float e, float r0, float v) {
    const float z = (float)tape_next(t, ORC_TAPE_N)->d;
    const float ours = f32_broaden_z(z, e, r0, v);
    const float ref = (float)tape_next(t, ORC_TAPE_E)->d;
    if (!t->off_path) {
        double d = fabs((double)ours - (double)ref);
        if (d > t->st->e_max_abs) t->st->e_max_abs = d;
    }
    return ref;
}

/* rk_binomial: the reference's variate; its (n, p) must be the body's */
static int64_t tape_binom(tape_src *t, int n, float p) {
    const orc_tape_rec *b = tape_next(t, ORC_TAPE_B);
    if (!t->off_path && ((b->tag >> 8) != n || b->d != (double)p)) t->st->binom_arg_mismatch += 1;
    return b->i;
}

#define RC_U(src) tape_u(src)
#define RC_TAU(src, k) tape_tau(src, k)
#define RC_BG(src, tot, tdiff, rate) tape_bg(src, tot, tdiff, rate)
#define RC_E(src, e, r0, v) tape_e(src, e, r0, v)
#define RC_BINOM(src, n, p) tape_binom(src, n, p)
static float f32_unit_rc_tape(const f32_tab *tb, const orc_rc_bursts *bs, const orc_model *m,
                              int64_t b, tape_src *src) {
#include "rc_unit_body.inc"
}
#undef RC_U
#undef RC_TAU
#undef RC_BG
#undef RC_E
#undef RC_BINOM

/* The tape format's self-check: the oracle's own Philox draws written as the
 * harness writes the reference's (orc_rc_record), so that replaying them must
 * give unit_rc's values bit for bit. */
typedef struct {
    orc_rng r;
    orc_tape_rec *rec;
    int64_t len, cap;
} tape_sink;

static void sink_put(tape_sink *k, int32_t tag, int32_t i, double d) {
    if (k->len < k->cap) {
        k->rec[k->len].tag = tag;
        k->rec[k->len].i = i;
        k->rec[k->len].d = d;
    }
    k->len += 1;
}
static float sink_u(tape_sink *k) {
    const float u = f32_u01(&k->r);
    sink_put(k, ORC_TAPE_U, 0, (double)u);
    return u;
}
static float sink_tau(tape_sink *k, float kk) {
    const float v = orc_logf(sink_u(k)) / (-kk);
    sink_put(k, ORC_TAPE_TAU, 0, (double)v);
    return v;
}
static float sink_bg(tape_sink *k, float tot, float tdiff, float rate) {
    const float lam = tdiff * rate;
    const int sv = f32_poisson(&k->r, lam);
    sink_put(k, ORC_TAPE_P, sv, (double)lam);
    if ((float)sv <= tot) return (float)sv;
    return floorf(tot * sink_u(k));
}
static float sink_e(tape_sink *k, float e, float r0, float v) {
    const float z = f32_normal(&k->r);
    sink_put(k, ORC_TAPE_N, 0, (double)z);
    const float x = f32_broaden_z(z, e, r0, v);
    sink_put(k, ORC_TAPE_E, 0, (double)x);
    return x;
}
static int64_t sink_binom(tape_sink *k, int n, float p) {
    const int v = f32_binom(&k->r, n, p);
    sink_put(k, ORC_TAPE_B | (n << 8), v, (double)p);
    return v;
}
#define RC_U(src) sink_u(src)
#define RC_TAU(src, k) sink_tau(src, k)
#define RC_BG(src, tot, tdiff, rate) sink_bg(src, tot, tdiff, rate)
#define RC_E(src, e, r0, v) sink_e(src, e, r0, v)
#define RC_BINOM(src, n, p) sink_binom(src, n, p)
static float f32_unit_rc_record(const f32_tab *tb, const orc_rc_bursts *bs, const orc_model *m,
                                int64_t b, tape_sink *src) {
#include "rc_unit_body.inc"
}
#undef RC_U
#undef RC_TAU
#undef RC_BG
#undef RC_E
#undef RC_BINOM

int orc_rc_record(const orc_rc_bursts *bs, int32_t n, const float *args, const orc_model *m,
                  int32_t R, uint64_t seed, int32_t cap, orc_tape_rec *tape, int32_t *tape_len,
                  float *mcE_out) {
    if (!bs || !args || !m || !tape || !tape_len || !mcE_out || n < 2 || n > ORC_MAXS || R < 1 || cap < 0)
        return -1;
    init_lf_d();
    f32_tab tb;
    int rc = f32_build(n, args, m, &tb, 0);
    if (rc != 0) return rc;
    for (int64_t t = 0; t < bs->B * (int64_t)R; ++t) {
        tape_sink k;
        rng_init(&k.r, seed, 0u, (uint32_t)(t / R), (uint32_t)(t % R));
        k.rec = tape + t * (int64_t)cap;
        k.len = 0;
        k.cap = cap;
        mcE_out[t] = f32_unit_rc_record(&tb, bs, m, t / R, &k);
        tape_len[t] = (int32_t)k.len;
    }
    return 0;
}

int orc_rc_replay(const orc_rc_bursts *bs, int32_t n, const float *args, const orc_model *m,
                  int32_t R, const orc_tape_rec *tape, const int32_t *tape_len, int32_t cap,
                  const float *ref_mcE, float *mcE_out, int8_t *status_out,
                  orc_replay_stats *stats) {
    if (!bs || !args || !m || !tape || !tape_len || !ref_mcE || !stats || n < 2 || n > ORC_MAXS ||
        R < 1 || cap < 0)
        return -1;
    init_lf_d();
    f32_tab tb;
    int rc = f32_build(n, args, m, &tb, 0);
    if (rc != 0) return rc;
    memset(stats, 0, sizeof(*stats));
    const int64_t units = bs->B * (int64_t)R;
    stats->units = units;
    for (int64_t t = 0; t < units; ++t) {
        const int64_t b = t / R;
        int8_t status;
        float x = 0.0f;
        if (tape_len[t] > cap) {
            status = ORC_REPLAY_TRUNCATED;
        } else {
            tape_src src = {tape + t * (int64_t)cap, tape_len[t], 0, 0, stats};
            x = f32_unit_rc_tape(&tb, bs, m, b, &src);
            if (src.off_path || src.pos != src.len) status = ORC_REPLAY_OFF_PATH;
            else status = (f32_bits(x) == f32_bits(ref_mcE[t])) ? ORC_REPLAY_EXACT : ORC_REPLAY_DIFFERS;
        }
        if (mcE_out) mcE_out[t] = x;
        if (status_out) status_out[t] = status;
        if (status == ORC_REPLAY_EXACT) stats->exact += 1;
        else if (status == ORC_REPLAY_DIFFERS) stats->differs += 1;
        else if (status == ORC_REPLAY_TRUNCATED) stats->truncated += 1;
        else stats->off_path += 1;
    }
    return 0;
}
#undef REAL
#undef RL
#undef LOGR
#undef EXPR
#undef SQRTR
#undef FLOORR
#undef FABSR
#undef FMAR
#undef COS2PIR
#undef COPYSIGNR
#undef INFR
#undef FC_T
#undef LF_T
#undef INV_T
#undef PFX

/* FP64 transcription on the same counters. */
static double lf_tab_d[10];
static double cos2pi_d(double u) { return cos(6.283185307179586 * u); }
#define REAL double
#define RL(x) x
#define LOGR log
#define EXPR exp
#define SQRTR sqrt
#define FLOORR floor
#define FABSR fabs
#define FMAR fma
#define COS2PIR cos2pi_d
#define COPYSIGNR copysign
#define INFR ((double)INFINITY)
#define FC_T FC_TAB_D
#define LF_T lf_tab_d
#define INV_T inv_tab_d
#define PFX(x) f64_##x
#include "gpda_oracle_core.inc"

static void init_lf_d(void) {
    static int done = 0;
    if (done) return;
    for (int k = 0; k < 10; ++k) lf_tab_d[k] = lgamma((double)k + 1.0);
    for (int k = 0; k < 64; ++k) {
        inv_tab_f[k] = k > 0 ? 1.0f / (float)k : 0.0f;
        inv_tab_d[k] = k > 0 ? 1.0 / (double)k : 0.0;
    }
    done = 1;
}

/* ------------------------------------------------------------------ */
void orc_binom_cdf_row(float pp, int32_t nn, float *out) { binom_cdf_row_df(pp, nn, out); }

int orc_build_params(int32_t n, const float *args, const orc_model *m, orc_params *out) {
    (void)m;
    orc_derived d;
    memset(out, 0, sizeof(*out));
    int rc = derive_double(n, args, &d, 1);
    if (rc != 0) return rc;
    out->n = n;
    for (int i = 0; i < n; ++i) {
        out->E[i] = args[i];
        out->V[i] = args[n * n + i];
        out->kexit[i] = (float)d.kexit[i];
        out->inv_kexit[i] = d.kexit[i] > 0.0 ? (float)(1.0 / d.kexit[i]) : INFINITY;
        out->init_cdf[i] = (float)d.init_cdf[i];
        float e = args[i];
        float om = 1.0f - e;
        float num = m->gamma * e + m->crosstalk * om;
        out->eps[i] = num / (num + om);
        for (int j = 0; j < n; ++j) out->jump_cdf[i * ORC_MAXS + j] = (float)d.jump_cdf[i * ORC_MAXS + j];
    }
    ref_tables_f(n, args, out->K, out->Pi2j, out->pinit);
    return 0;
}

int orc_sample(int kind, uint64_t seed, int32_t n, float p, int64_t count, double *out) {
    init_lf_d();
    for (int64_t i = 0; i < count; ++i) {
        orc_rng r;
        rng_init(&r, seed, 0u, 0u, (uint32_t)i);
        switch (kind) {
        case 0: out[i] = (double)f32_binom(&r, n, p); break;
        case 1: out[i] = (double)f32_poisson(&r, p); break;
        case 2: out[i] = (double)(-orc_logf(f32_u01(&r)) * (1.0f / p)); break;
        case 3: out[i] = (double)f32_normal(&r); break;
        case 4: out[i] = (double)f32_u01(&r); break;
        case 5: out[i] = (double)f64_binom(&r, n, (double)p); break;
        case 6: out[i] = (double)f64_poisson(&r, (double)p); break;
        default: return -1;
        }
    }
    return 0;
}

/* the photon-mode background pair (background_pair) without clipping:
 * variate i = (A_i, D_i) on the unit stream of counter (0, 0, i), with the
 * kernel's constants for rates (bg_a, bg_d) over a segment of length dt */
int orc_sample_bgpair(uint64_t seed, float bg_a, float bg_d, float dt, int64_t count, int32_t *A,
                      int32_t *D) {
    if (!A || !D || !(bg_a > 0.0f) || !(bg_d > 0.0f) || !(dt >= 0.0f)) return -1;
    init_lf_d();
    const float bgs = bg_a + bg_d;
    const float pa = bg_a / bgs;
    const float bgc[4] = {bgs, pa, 1.0f / pa, 1.0f / (1.0f - pa)};
    for (int64_t i = 0; i < count; ++i) {
        orc_rng r;
        rng_init(&r, seed, 0u, 0u, (uint32_t)i);
        int rem = 0;
        A[i] = f32_background_pair(&r, 1 << 30, dt, bgc, &rem);
        D[i] = (1 << 30) - rem - A[i];
    }
    return 0;
}

/* categorical draws: mode 0 pda initial-state draw over a cumulative table
 * w[n]; mode 1 drawDisIdx over unnormalised weights w[n] (gen_rand.cuh:35-50);
 * mode 2 pda jump draw from `from` over the cumulative row w[n]; mode 3
 * drawJ_Si2Sj from `from` over the column-major n x n matrix w (:78-89). */
int orc_sample_cat(uint64_t seed, int32_t mode, int32_t n, const float *w, int32_t from,
                   int64_t count, int32_t *out) {
    if (n < 1 || n > ORC_MAXS || !w || !out || from < 0 || from >= n) return -1;
    for (int64_t i = 0; i < count; ++i) {
        orc_rng r;
        rng_init(&r, seed, 0u, 0u, (uint32_t)i);
        float u = f32_u01(&r);
        switch (mode) {
        case 0: out[i] = f32_cat(w, n, u); break;
        case 1: out[i] = f32_disidx(n, w, u); break;
        case 2: out[i] = f32_jump(w, n, from, u); break;
        case 3: {
            float col[ORC_MAXS];
            for (int ii = 0; ii < n - 1; ++ii)
                col[ii] = (ii >= from) ? w[from * n + ii + 1] : w[from * n + ii];
            int j = f32_disidx(n - 1, col, u);
            out[i] = (j >= from) ? j + 1 : j;
            break;
        }
        default: return -1;
        }
    }
    return 0;
}

static int check_model(const orc_model *m) {
    if (m->nbins < 1 || m->nbins > 4096) return -1;
    if (m->left_pad < 0 || m->left_pad > m->nbins) return -1;
    if (!(m->gamma > 0.0f && m->gamma < INFINITY)) return -1;
    if (!(m->crosstalk >= 0.0f && m->crosstalk < INFINITY)) return -1;
    if (!(m->bg_d >= 0.0f && m->bg_d < INFINITY)) return -1;
    if (!(m->bg_a >= 0.0f && m->bg_a < INFINITY)) return -1;
    if (!(m->r0 > 0.0f && m->rc_r0 > 0.0f)) return -1;
    return 0;
}

int orc_run_pda(const orc_bursts *bs, int32_t n, const float *args, int32_t P,
                const orc_model *m, int32_t mode, int32_t S, uint64_t seed,
                int64_t b0, int64_t b1, uint64_t *hist, int32_t *unit_out,
                int32_t nthreads, int32_t f64) {
    if (!bs || !args || !m || !hist) return -1;
    if (P < 1 || S < 1 || b0 < 0 || b1 < b0 || b1 > bs->B) return -1;
    if (mode != ORC_MODE_OCCUPANCY && mode != ORC_MODE_PHOTON) return -1;
    if (mode == ORC_MODE_PHOTON && (!bs->off_idx || !bs->offsets)) return -1;
    if (check_model(m)) return -1;
    init_lf_d();
    return f64 ? f64_run_pda(bs, n, args, P, m, mode, S, seed, b0, b1, hist, unit_out, nthreads)
               : f32_run_pda(bs, n, args, P, m, mode, S, seed, b0, b1, hist, unit_out, nthreads);
}

int orc_run_refcompat(const orc_rc_bursts *bs, int32_t n, const float *args,
                      const orc_model *m, int32_t S, uint64_t seed,
                      int64_t b0, int64_t b1, uint64_t *hist, float *mcE,
                      int32_t nthreads, int32_t f64) {
    if (!bs || !args || !m) return -1;
    if (n < 2 || n > ORC_MAXS) return -1;
    if (S < 1 || b0 < 0 || b1 < b0 || b1 > bs->B) return -1;
    if (check_model(m)) return -1;
    init_lf_d();
    return f64 ? f64_run_refcompat(bs, n, args, m, S, seed, b0, b1, hist, mcE, nthreads)
               : f32_run_refcompat(bs, n, args, m, S, seed, b0, b1, hist, mcE, nthreads);
}

double orc_chi2(const uint64_t *hist, const float *ohist, int32_t nbins,
                int32_t left_pad, int32_t S, int32_t n_states) {
    int effN = nbins - left_pad;
    double chi = 0.0;
    for (int i = left_pad; i < nbins; ++i) {
        if (hist[i] > 0) {
            double mi = (double)hist[i] / (double)S;
            double dlt = (double)ohist[i] - mi;
            chi = chi + dlt * dlt / mi;
        } else {
            effN -= 1;
        }
    }
    return chi / (double)(effN - n_states * (n_states + 1));
}

/* streamWorker.cpp:197-206, in its own float arithmetic */
float orc_chi2_f32(const float *mhist, const float *ohist, int32_t nbins,
                   int32_t left_pad, int32_t R, int32_t n_states) {
    int effN = nbins - left_pad;
    float chisqr = 0.0f;
    for (int i = left_pad; i < nbins; ++i) {
        if (mhist[i] > 0.0f) {
            /* pow(float, int) is a double; the += rounds back to float */
            float mr = mhist[i] / (float)R;
            float d = ohist[i] - mr;
            double term = pow((double)d, 2.0) / (double)mr;
            chisqr = (float)((double)chisqr + term);
        } else {
            effN--;
        }
    }
    return chisqr / (float)(effN - n_states * (n_states + 1));
}

void orc_bin_values(const float *x, int64_t n, int32_t nbins, float *hist_out) {
    for (int i = 0; i < nbins; ++i) hist_out[i] = 0.0f;
    for (int64_t k = 0; k < n; ++k) {
        int b = ref_bin_d((double)x[k], nbins);
        if (b >= 0) hist_out[b] += 1.0f;
    }
}

/* ------------------------------------------------------------------ */
/* Differentiable expected histogram (occupancy form), FP64 restatement of
 * gpda_expected_hist / gpda_expected_hist_adjoint.
 *
 * The state skeleton comes from the FP32 mirror (anchor tables, same Philox
 * counters and draw order as unit_occ); the background counts too, but from
 * counter block 2^31 on (independent of the trajectory's length). Both are the
 * device's integers. Everything continuous is FP64: dwells
 * -ln(u)/k_exit(theta), the likelihood-ratio weight, E_eff, the binomial
 * masses (exact over all x from a log-factorial table, no truncation), the
 * chi-square and the gradient. d ln pi / d ln K is a central difference of
 * the FP64 stationary solve (independent of the device's linear solve). */

#define XMAXS 4

typedef struct {
    int n;
    double E[XMAXS], kexit[XMAXS];
    double pi[XMAXS], pj[XMAXS][XMAXS];      /* theta */
    double lw_init[XMAXS], lw_jump[XMAXS][XMAXS];
    double dlnpi[XMAXS][XMAXS * (XMAXS - 1)];
} x_par;

/* K (column-major, K[j*n+i] = rate j->i) from a parameter vector, with the
 * off-diagonal `pidx` (parameter order) scaled by exp(h). */
static void x_rates(int n, const float *args, int pidx, double h, double *K, double *kexit) {
    const float *ko = args + n;
    for (int j = 0; j < n; ++j) {
        double cs = 0.0;
        for (int i = 0; i < n; ++i) {
            if (i == j) continue;
            int idx = i * (n - 1) + (j < i ? j : j - 1);
            double k = (double)koff_at(ko, n, i, j);
            if (idx == pidx) k *= exp(h);
            K[j * n + i] = k;
            cs += k;
        }
        K[j * n + j] = -cs;
        kexit[j] = cs;
    }
}

static int x_pi(int n, const double *K, double *pi) {
    double A[XMAXS][XMAXS + 1];
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) A[i][j] = (i == n - 1) ? 1.0 : K[j * n + i];
        A[i][n] = (i == n - 1) ? 1.0 : 0.0;
    }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r) if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        if (!(fabs(A[piv][c]) > 0.0)) return -2;
        if (piv != c) for (int k = 0; k <= n; ++k) { double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
        for (int r = c + 1; r < n; ++r) {
            double f = A[r][c] / A[c][c];
            for (int k = c; k <= n; ++k) A[r][k] -= f * A[c][k];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = A[r][n];
        for (int k = r + 1; k < n; ++k) s -= A[r][k] * pi[k];
        pi[r] = s / A[r][r];
    }
    for (int i = 0; i < n; ++i) if (!(pi[i] > 0.0)) return -2;
    return 0;
}

static int x_build(int n, const float *theta, const float *anchor, x_par *xp) {
    double Kt[16], K0[16], kt[4], k0[4], pi0[4];
    for (int i = 0; i < n; ++i)
        if (theta[n * n + i] != 0.0f || anchor[n * n + i] != 0.0f) return -1;
    x_rates(n, theta, -1, 0.0, Kt, kt);
    x_rates(n, anchor, -1, 0.0, K0, k0);
    if (x_pi(n, Kt, xp->pi) || x_pi(n, K0, pi0)) return -2;
    xp->n = n;
    for (int i = 0; i < n; ++i) {
        xp->E[i] = (double)theta[i];
        xp->kexit[i] = kt[i];
        xp->lw_init[i] = log(xp->pi[i]) - log(pi0[i]);
        for (int l = 0; l < n; ++l) {
            xp->pj[i][l] = 0.0;
            xp->lw_jump[i][l] = 0.0;
            if (l == i) continue;
            double pt = kt[i] > 0.0 ? Kt[i * n + l] / kt[i] : 0.0;
            double p0 = k0[i] > 0.0 ? K0[i * n + l] / k0[i] : 0.0;
            xp->pj[i][l] = pt;
            if (p0 > 0.0) xp->lw_jump[i][l] = pt > 0.0 ? log(pt) - log(p0) : -INFINITY;
        }
    }
    const double h = 1e-6;
    for (int idx = 0; idx < n * (n - 1); ++idx) {
        double Kp[16], Km[16], kk[4], pp[4], pm[4];
        x_rates(n, theta, idx, h, Kp, kk);
        x_rates(n, theta, idx, -h, Km, kk);
        if (x_pi(n, Kp, pp) || x_pi(n, Km, pm)) return -2;
        for (int s = 0; s < n; ++s) xp->dlnpi[s][idx] = (log(pp[s]) - log(pm[s])) / (2.0 * h);
    }
    return 0;
}

typedef struct {
    double eeff, W, dtl, D[XMAXS];
    int s0, sm, cnt[XMAXS][XMAXS], sig, ba, timed;
} x_unit;

/* one unit: skeleton from the FP32 anchor tables, FP64 dwells under theta */
static int x_walk(const f32_tab *sk, const x_par *xp, int Nb, float Tb, float bga, float bgd,
                  uint64_t seed, uint32_t pw, uint32_t b, uint32_t s, x_unit *U) {
    if (Nb <= 0) return 0;
    orc_rng r;
    rng_init(&r, seed, pw, b, s);
    int n = xp->n, st = 0;
    double t = 0.0, acc = 0.0, lw = 0.0, T = (double)Tb;
    memset(U, 0, sizeof(*U));
    U->timed = Tb > 0.0f;
    for (int seg = 0; seg < ORC_MAX_SEG; ++seg) {
        float us = f32_u01(&r);
        int ns;
        if (seg == 0) {
            ns = f32_cat(sk->init_cdf, n, us);
            U->s0 = ns;
            lw += xp->lw_init[ns];
        } else {
            ns = f32_jump(sk->jump_cdf + st * ORC_MAXS, n, st, us);
            lw += xp->lw_jump[st][ns];
            U->cnt[st][ns] += 1;
        }
        st = ns;
        if (!U->timed) break;
        float u = f32_u01(&r);
        double tau = xp->kexit[st] > 0.0 ? -log((double)u) / xp->kexit[st] : INFINITY;
        double tn = t + tau;
        int last = !(tn < T) || seg == ORC_MAX_SEG - 1;
        double dt = last ? T - t : tau;
        acc += dt * xp->E[st];
        if (last) { U->dtl = dt; break; }
        U->D[st] += dt;
        t = tn;
    }
    U->sm = st;
    U->eeff = U->timed ? acc / T : xp->E[st];
    U->W = exp(lw);
    r.ctr[0] = 0x80000000u;        /* background from a fixed counter block */
    rng_align(&r);
    int Ba = f32_poisson(&r, bga * Tb);
    if (Ba > Nb) Ba = (int)floorf((float)Nb * f32_u01(&r));
    int rem = Nb - Ba;
    int Bd = f32_poisson(&r, bgd * Tb);
    if (Bd > rem) Bd = (int)floorf((float)rem * f32_u01(&r));
    U->ba = Ba;
    U->sig = rem - Bd;
    return 1;
}

static inline double x_eps(double e, double g, double ct) {
    double om = 1.0 - e, num = g * e + ct * om;
    return num / (num + om);
}
static inline double x_deps(double e, double g, double ct) {
    double om = 1.0 - e, num = g * e + ct * om, den = num + om;
    return ((g - ct) * om + num) / (den * den);
}

/* visits every x of Binomial(sig, p): fn(bin, P(x), x) */
#define X_FOR_MASSES(U, Nb, nbins, p, lf, BODY)                                               \
    do {                                                                                       \
        int sig_ = (U).sig;                                                                    \
        if (sig_ <= 0 || !((p) > 0.0) || (p) >= 1.0) {                                        \
            int x = (sig_ > 0 && (p) >= 1.0) ? sig_ : 0;                                       \
            int bin = pda_bin((U).ba + x, Nb, nbins);                                          \
            double mass = 1.0;                                                                 \
            BODY;                                                                              \
        } else {                                                                               \
            double lp_ = log(p), lq_ = log1p(-(p));                                            \
            for (int x = 0; x <= sig_; ++x) {                                                  \
                double mass = exp(lf[sig_] - lf[x] - lf[sig_ - x] + x * lp_ + (sig_ - x) * lq_); \
                int bin = pda_bin((U).ba + x, Nb, nbins);                                      \
                BODY;                                                                          \
            }                                                                                  \
        }                                                                                      \
    } while (0)

int orc_expected(const orc_bursts *bs, int32_t n, const float *params, const float *anchor,
                 int32_t P, const orc_model *m, int32_t S, uint64_t seed, const float *obs,
                 double *hist, double *chi2, double *dE, double *dlogK, int32_t nthreads) {
    init_lf_d();
    if (n < 1 || n > XMAXS || P < 1 || S < 1 || !params || !obs || !hist || !chi2) return -1;
    const int nb = m->nbins, nk = n * (n - 1);
    int maxN = 0;
    for (int64_t b = 0; b < bs->B; ++b) if (bs->N[b] > maxN) maxN = bs->N[b];
    double *lf = (double *)malloc(sizeof(double) * (size_t)(maxN + 1));
    if (!lf) return -4;
    for (int k = 0; k <= maxN; ++k) lf[k] = lgamma((double)k + 1.0);
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const double g = m->gamma, ct = m->crosstalk;
    const float bga = m->bg_a, bgd = m->bg_d;
    int rc = 0;
    for (int p = 0; p < P && rc == 0; ++p) {
        const float *th = params + (size_t)p * n * (n + 1);
        const float *an = anchor ? anchor + (size_t)p * n * (n + 1) : th;
        f32_tab sk;
        x_par xp;
        if ((rc = f32_build(n, an, m, &sk, 1)) != 0) break;
        if ((rc = x_build(n, th, an, &xp)) != 0) break;
        double *H = hist + (size_t)p * nb;
        for (int i = 0; i < nb; ++i) H[i] = 0.0;
        /* forward */
#pragma omp parallel
        {
            double loc[64];
            for (int i = 0; i < nb; ++i) loc[i] = 0.0;
#pragma omp for schedule(dynamic, 64)
            for (int64_t b = 0; b < bs->B; ++b) {
                int Nb = bs->N[b];
                for (int s = 0; s < S; ++s) {
                    x_unit U;
                    if (!x_walk(&sk, &xp, Nb, bs->T[b], bga, bgd, seed, (uint32_t)p, (uint32_t)b, (uint32_t)s, &U)) continue;
                    double pe = x_eps(U.eeff, g, ct);
                    X_FOR_MASSES(U, Nb, nb, pe, lf, loc[bin] += U.W * mass);
                }
            }
#pragma omp critical
            for (int i = 0; i < nb; ++i) H[i] += loc[i];
        }
        /* chi-square and d chi2 / d hist */
        int effN = nb - m->left_pad;
        double chi = 0.0, gb[64];
        for (int i = m->left_pad; i < nb; ++i) {
            if (H[i] > 0.0) {
                double mi = H[i] / S, d = (double)obs[i] - mi;
                chi += d * d / mi;
            } else {
                effN -= 1;
            }
        }
        double den = (double)(effN - n * (n + 1));
        chi2[p] = chi / den;
        for (int i = 0; i < nb; ++i) {
            gb[i] = 0.0;
            if (i >= m->left_pad && H[i] > 0.0) {
                double mi = H[i] / S, o = (double)obs[i];
                gb[i] = (1.0 - o * o / (mi * mi)) / (S * den);
            }
        }
        if (!dE && !dlogK) continue;
        /* adjoint */
        double gE[XMAXS] = {0}, gK[XMAXS * (XMAXS - 1)] = {0};
#pragma omp parallel
        {
            double lE[XMAXS] = {0}, lK[XMAXS * (XMAXS - 1)] = {0};
#pragma omp for schedule(dynamic, 64)
            for (int64_t b = 0; b < bs->B; ++b) {
                int Nb = bs->N[b];
                for (int s = 0; s < S; ++s) {
                    x_unit U;
                    if (!x_walk(&sk, &xp, Nb, bs->T[b], bga, bgd, seed, (uint32_t)p, (uint32_t)b, (uint32_t)s, &U)) continue;
                    double pe = x_eps(U.eeff, g, ct);
                    double G = 0.0, GX = 0.0;
                    X_FOR_MASSES(U, Nb, nb, pe, lf, { G += gb[bin] * mass; GX += gb[bin] * mass * x; });
                    double Hd = 0.0;
                    if (U.sig > 0 && pe > 0.0 && pe < 1.0) Hd = (GX - U.sig * pe * G) / (pe * (1.0 - pe));
                    double HE = U.W * Hd * x_deps(U.eeff, g, ct), WG = U.W * G;
                    double invT = U.timed ? 1.0 / (double)bs->T[b] : 0.0;
                    for (int i = 0; i < n; ++i) {
                        double occ = U.timed ? (U.D[i] + (i == U.sm ? U.dtl : 0.0)) * invT : (i == U.sm ? 1.0 : 0.0);
                        lE[i] += HE * occ;
                    }
                    for (int l = 0; l < n; ++l)
                        for (int i = 0; i < n; ++i) {
                            if (i == l) continue;
                            int idx = l * (n - 1) + (i < l ? i : i - 1);
                            int nout = 0;
                            for (int j = 0; j < n; ++j) nout += U.cnt[i][j];
                            double score = xp.dlnpi[U.s0][idx] + U.cnt[i][l] - nout * xp.pj[i][l];
                            double path = -xp.pj[i][l] * U.D[i] * (xp.E[i] - xp.E[U.sm]) * invT;
                            lK[idx] += WG * score + HE * path;
                        }
                }
            }
#pragma omp critical
            {
                for (int i = 0; i < n; ++i) gE[i] += lE[i];
                for (int k = 0; k < nk; ++k) gK[k] += lK[k];
            }
        }
        if (dE) for (int i = 0; i < n; ++i) dE[(size_t)p * n + i] = gE[i];
        if (dlogK) for (int k = 0; k < nk; ++k) dlogK[(size_t)p * nk + k] = gK[k];
    }
    free(lf);
    return rc;
}
