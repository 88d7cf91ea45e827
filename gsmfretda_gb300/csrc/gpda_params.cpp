// gpda_params.cpp — host-side derivation of the per-parameter-set tables.
//
// Input: the reference's parameter vector (src/mc.cu:792-800)
//   args = [E(n), K off-diagonals (n*n-n, row-major over i skipping i==j,
//           K(i,j) = rate j->i), V(n)].
// Output (DevParams):
//   pda tables  — exit rates, 1/exit rates, cumulative jump probabilities per
//                 source state, cumulative stationary distribution (solved in
//                 FP64, K pi = 0, sum pi = 1), apparent acceptor probability
//                 eps(E) = (g E + ct (1-E)) / (g E + (1+ct)(1-E)).
//   rc tables   — genMatK (src/eigenhelper.cpp:4-22), genP_i2j (:24-38),
//                 genMatP (:39-53) in the reference's float operation order.
// All FP64 work is rounded once to FP32. Compiled with -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "gpda_internal.h"

namespace gpda {

namespace {

// The device's logf_ (gpda_device.cuh), evaluated on the host with the same
// operation order so that precomputed constants are the device's bits.
float dev_logf(float x) {
    if (x != x) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return x;
    uint32_t bits;
    std::memcpy(&bits, &x, 4);
    int e = 0;
    if ((bits >> 23) == 0u) {
        x = x * 0x1p24f;
        std::memcpy(&bits, &x, 4);
        e = -24;
    }
    e += (int)(bits >> 23) - 127;
    uint32_t mb = (bits & 0x007FFFFFu) | 0x3F800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float poly = std::fmaf(z, std::fmaf(z, std::fmaf(z, 0x1.c71c72p-3f, 0x1.24924ap-2f), 0x1.99999ap-2f), 0x1.555556p-1f);
    float lm = std::fmaf(s * z, poly, 2.0f * s);
    float ef = (float)e;
    return std::fmaf(ef, 0x1.62e430p-1f, std::fmaf(ef, -0x1.05c610p-29f, lm));
}

inline float koff(const float *k, int n, int i, int j) {
    return (i < j) ? k[i * (n - 1) + j - 1] : k[i * (n - 1) + j];
}

}  // namespace

int build_params(int n, const float *args, float gamma, float ct, bool need_pi, DevParams *out) {
    std::memset(out, 0, sizeof(*out));
    if (n < 1 || n > 8 || args == nullptr) return -1;
    const float *ko = args + n;
    const float *V = args + n * n;
    for (int i = 0; i < n; ++i) {
        float e = args[i], v = V[i];
        if (!(e >= 0.0f && e <= 1.0f)) return -1;
        if (!(v >= 0.0f && v < INFINITY)) return -1;
    }
    double Kd[64];
    double kexit[8];
    double jcdf[64];
    double kmax = 1.0;
    for (int j = 0; j < n; ++j) {
        double colsum = 0.0;
        for (int i = 0; i < n; ++i) {
            if (i == j) continue;
            float k = koff(ko, n, i, j);
            if (!(k >= 0.0f && k < INFINITY)) return -1;
            Kd[j * n + i] = (double)k;
            colsum += (double)k;
            if ((double)k > kmax) kmax = (double)k;
        }
        Kd[j * n + j] = -colsum;
        kexit[j] = colsum;
        double acc = 0.0;
        for (int i = 0; i < n; ++i) {
            if (colsum > 0.0) {
                if (i != j) acc += Kd[j * n + i];
                jcdf[j * 8 + i] = acc / colsum;
            } else {
                jcdf[j * 8 + i] = 1.0;
            }
        }
    }
    double icdf[8];
    if (need_pi) {
        double A[8][9];
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j < n; ++j) A[i][j] = Kd[j * n + i];
            A[i][n] = 0.0;
        }
        for (int j = 0; j < n; ++j) A[n - 1][j] = 1.0;
        A[n - 1][n] = 1.0;
        for (int c = 0; c < n; ++c) {
            int piv = c;
            for (int r = c + 1; r < n; ++r)
                if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
            if (!(std::fabs(A[piv][c]) > 1e-13 * kmax)) return -2;
            if (piv != c)
                for (int k = 0; k <= n; ++k) { double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
            for (int r = c + 1; r < n; ++r) {
                double f = A[r][c] / A[c][c];
                for (int k = c; k <= n; ++k) A[r][k] = A[r][k] - f * A[c][k];
            }
        }
        double pi[8];
        for (int r = n - 1; r >= 0; --r) {
            double s = A[r][n];
            for (int k = r + 1; k < n; ++k) s = s - A[r][k] * pi[k];
            pi[r] = s / A[r][r];
        }
        double sum = 0.0;
        for (int i = 0; i < n; ++i) { if (!(pi[i] > 0.0)) pi[i] = 0.0; sum += pi[i]; }
        if (!(sum > 0.0)) return -2;
        double acc = 0.0;
        for (int i = 0; i < n; ++i) { acc += pi[i] / sum; icdf[i] = acc; }
    } else {
        for (int i = 0; i < n; ++i) icdf[i] = (double)(i + 1) / (double)n;
    }
    out->n = n;
    out->anyV = 0;
    for (int i = 0; i < n; ++i) {
        out->E[i] = args[i];
        out->V[i] = V[i];
        if (V[i] > 0.0f) out->anyV = 1;
        out->kexit[i] = (float)kexit[i];
        out->inv_kexit[i] = kexit[i] > 0.0 ? (float)(1.0 / kexit[i]) : INFINITY;
        out->init_cdf[i] = (float)icdf[i];
        float e = args[i];
        float om = 1.0f - e;
        float num = gamma * e + ct * om;
        out->eps[i] = num / (num + om);
        float p = out->eps[i];
        float pp = (p > 0.5f) ? 1.0f - p : p;
        float q = 1.0f - pp;
        out->bpp[i] = pp;
        out->blogq[i] = dev_logf(q);
        out->brr[i] = pp / q;
        for (int j = 0; j < n; ++j) out->jump_cdf[i * 8 + j] = (float)jcdf[i * 8 + j];
    }
    // reference float tables (leading dimension n)
    float *K = out->K, *P = out->Pi2j, *pinit = out->pinit;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) K[i + j * n] = (i == j) ? 0.0f : koff(ko, n, i, j);
    for (int j = 0; j < n; ++j)
        for (int ii = 0; ii < n; ++ii)
            if (ii != j) K[j + j * n] = K[j + j * n] - K[ii + j * n];
    for (int j = 0; j < n; ++j) {
        float sum = 0.0f;
        for (int ii = 0; ii < n; ++ii)
            if (ii != j) sum = sum + K[ii + j * n];
        for (int ii = 0; ii < n; ++ii) P[ii + j * n] = (ii != j) ? K[ii + j * n] / sum : 0.0f;
    }
    for (int i = 0; i < n; ++i) {
        float s = 0.0f;
        for (int j = 0; j < n; ++j) s = s + K[i + j * n];
        s = s - K[i + i * n];
        pinit[i] = s;
    }
    return 0;
}

// ---------------------------------------------------------------- expected histogram

namespace {

// Rate matrix of a parameter vector in FP64, column-major K[j*n + i] = rate j->i,
// diagonal = -exit rate.
void rate_matrix(int n, const float *args, double *K, double *kexit, double *kmax) {
    const float *ko = args + n;
    *kmax = 1.0;
    for (int j = 0; j < n; ++j) {
        double colsum = 0.0;
        for (int i = 0; i < n; ++i) {
            if (i == j) continue;
            double k = (double)koff(ko, n, i, j);
            K[j * n + i] = k;
            colsum += k;
            if (k > *kmax) *kmax = k;
        }
        K[j * n + j] = -colsum;
        kexit[j] = colsum;
    }
}

// Solves rows 0..n-2 of K x = r together with sum(x) = r[n-1] (the balance
// equations with the last one replaced by the normalisation), Gaussian
// elimination with partial pivoting. Returns -2 when the system is singular.
int solve_balance(int n, const double *K, const double *r, double kmax, double *x) {
    double A[kExpMaxStates][kExpMaxStates + 1];
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) A[i][j] = (i == n - 1) ? 1.0 : K[j * n + i];
        A[i][n] = r[i];
    }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int q = c + 1; q < n; ++q)
            if (std::fabs(A[q][c]) > std::fabs(A[piv][c])) piv = q;
        if (!(std::fabs(A[piv][c]) > 1e-13 * kmax)) return -2;
        if (piv != c)
            for (int k = 0; k <= n; ++k) { double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
        for (int q = c + 1; q < n; ++q) {
            double f = A[q][c] / A[c][c];
            for (int k = c; k <= n; ++k) A[q][k] = A[q][k] - f * A[c][k];
        }
    }
    for (int q = n - 1; q >= 0; --q) {
        double v = A[q][n];
        for (int k = q + 1; k < n; ++k) v = v - A[q][k] * x[k];
        x[q] = v / A[q][q];
    }
    return 0;
}

int stationary(int n, const double *K, double kmax, double *pi) {
    double r[kExpMaxStates] = {0.0, 0.0, 0.0, 0.0};
    r[n - 1] = 1.0;
    if (solve_balance(n, K, r, kmax, pi)) return -2;
    for (int i = 0; i < n; ++i)
        if (!(pi[i] > 0.0)) return -2;
    return 0;
}

}  // namespace

int build_exp_params(int n, const float *theta, const float *anchor, float gamma, float ct,
                     ExpParams *out) {
    std::memset(out, 0, sizeof(*out));
    if (n < 1 || n > kExpMaxStates || theta == nullptr || anchor == nullptr) return -1;
    DevParams dt, d0;
    int rc = build_params(n, theta, gamma, ct, true, &dt);
    if (rc) return rc;
    rc = build_params(n, anchor, gamma, ct, true, &d0);
    if (rc) return rc;
    if (dt.anyV || d0.anyV) return -1;      // no distance broadening in this form
    double Kt[16], K0[16], kt[4], k0[4], kmt, km0, pit[4], pi0[4];
    rate_matrix(n, theta, Kt, kt, &kmt);
    rate_matrix(n, anchor, K0, k0, &km0);
    if (stationary(n, Kt, kmt, pit) || stationary(n, K0, km0, pi0)) return -2;
    out->n = n;
    const float ninf = -INFINITY;
    for (int i = 0; i < n; ++i) {
        out->E[i] = dt.E[i];
        out->kexit[i] = dt.kexit[i];
        out->inv_kexit[i] = dt.inv_kexit[i];
        out->init_cdf[i] = d0.init_cdf[i];
        out->lw_init[i] = (float)(std::log(pit[i]) - std::log(pi0[i]));
        for (int l = 0; l < n; ++l) {
            out->jump_cdf[i * 4 + l] = d0.jump_cdf[i * 8 + l];
            if (l == i) continue;
            double pt = kt[i] > 0.0 ? Kt[i * n + l] / kt[i] : 0.0;
            double p0 = k0[i] > 0.0 ? K0[i * n + l] / k0[i] : 0.0;
            out->pj[i * 4 + l] = (float)pt;
            out->lw_jump[i * 4 + l] = (p0 > 0.0) ? (pt > 0.0 ? (float)(std::log(pt) - std::log(p0)) : ninf) : 0.0f;
        }
    }
    // d pi / d ln K(i,j) (rate j->i): K dpi = -dK pi with dK = K(i,j) (e_i - e_j) e_j^T,
    // sum(dpi) = 0.
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            const int idx = i * (n - 1) + (j < i ? j : j - 1);
            double r[kExpMaxStates] = {0.0, 0.0, 0.0, 0.0};
            const double f = Kt[j * n + i] * pit[j];
            r[i] -= f;
            r[j] += f;
            r[n - 1] = 0.0;
            double dpi[kExpMaxStates];
            if (solve_balance(n, Kt, r, kmt, dpi)) return -2;
            for (int s2 = 0; s2 < n; ++s2) out->dlnpi[s2 * 12 + idx] = (float)(dpi[s2] / pit[s2]);
        }
    }
    return 0;
}

}  // namespace gpda
