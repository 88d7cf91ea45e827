"""Pins of the oracle's primitives: Philox known answers, FP32 elementary
functions against libm, and the reference's statistical sampler tests
(tests/GenRandTest.cu, tests/gen_rand_tests.cpp) restated with fixed seeds.
The reference's r^2 thresholds stay as minimum bars; a chi-square
goodness-of-fit test against the exact law is added on top."""
import math

import numpy as np
import pytest
from scipy import stats


def r_squared(a, b):
    """dlib::r_squared: squared Pearson correlation of two sequences."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    c = np.corrcoef(a, b)[0, 1]
    return c * c


def gof_pvalue(x, pmf, lo, hi, min_expected=5.0):
    ks = np.arange(lo, hi + 1)
    cnt = np.array([(x == k).sum() for k in ks], dtype=np.float64)
    exp = pmf(ks) * x.size
    m = exp > min_expected
    # lump the tails into one cell so that no mass is dropped
    tail_obs = x.size - cnt[m].sum()
    tail_exp = x.size - exp[m].sum()
    obs = np.append(cnt[m], tail_obs)
    ex = np.append(exp[m], tail_exp)
    keep = ex > 0
    c2 = ((obs[keep] - ex[keep]) ** 2 / ex[keep]).sum()
    return stats.chi2.sf(c2, keep.sum() - 1)


# ------------------------------------------------------------------ Philox

# Known-answer vectors of Philox4x32-10 published with Random123 (Salmon et al. 2011)
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(orc, ctr, key, expect):
    assert [int(x) for x in orc.philox(ctr, key)] == expect


def test_u01_range_and_grid(orc):
    u = orc.sample("u01", 5, 0, 0.0, 200_000)
    assert u.min() > 0.0 and u.max() <= 1.0
    k = u * 2 ** 24
    np.testing.assert_array_equal(k, np.round(k))      # exact multiples of 2^-24
    assert stats.kstest(u, "uniform").pvalue > 1e-3


# ------------------------------------------------------------------ FP32 math

def _ulps(got, ref):
    ref32 = np.abs(ref).astype(np.float32)
    return np.abs(got - ref) / np.spacing(ref32).astype(np.float64)


def test_logf_within_2ulp(orc):
    L = orc.lib()
    rs = np.random.RandomState(0)
    xs = np.concatenate([rs.uniform(0, 1, 20000), rs.uniform(0.5, 2.0, 20000),
                         np.exp(rs.uniform(-80, 80, 20000)), [1.0, 2.0, 0.5, 1e-38, 3e-45]])
    xs = xs.astype(np.float32)
    got = np.array([L.orc_logf(float(x)) for x in xs], dtype=np.float64)
    ref = np.log(xs.astype(np.float64))
    nz = np.abs(ref) > 1e-3
    assert _ulps(got[nz], ref[nz]).max() < 2.0
    assert np.abs(got[~nz] - ref[~nz]).max() < 1e-9
    assert L.orc_logf(0.0) == -math.inf
    assert math.isnan(L.orc_logf(-1.0))


def test_expf_within_1ulp(orc):
    L = orc.lib()
    xs = np.random.RandomState(1).uniform(-87, 88, 20000).astype(np.float32)
    got = np.array([L.orc_expf(float(x)) for x in xs])
    assert _ulps(got, np.exp(xs.astype(np.float64))).max() < 1.0
    assert L.orc_expf(-200.0) == 0.0 and L.orc_expf(100.0) == math.inf


def test_cos2pi(orc):
    L = orc.lib()
    us = np.random.RandomState(2).uniform(0, 1, 20000).astype(np.float32)
    got = np.array([L.orc_cos2pif(float(u)) for u in us])
    assert np.abs(got - np.cos(2 * np.pi * us.astype(np.float64))).max() < 2e-7


# ------------------------------------------------------------------ samplers

# reference grid: N draws in {1000,10000,20000,30000}, n in 3..6, p in
# {0.41, 0.54, 1/2.1, 1/3.3} (p > 1 -> 1/p, p < 0.2 skipped), r^2 >= 0.711
@pytest.mark.parametrize("N", [1000, 10000, 20000, 30000])
@pytest.mark.parametrize("n", [3, 4, 5, 6])
@pytest.mark.parametrize("p", [0.41, 0.54, 1 / 2.1, 1 / 3.3])
def test_binomial_reference_grid(orc, N, n, p):
    x = orc.sample("binomial", 1000 + n, n, p, N)
    sp = np.bincount(x.astype(np.int64), minlength=n + 1)[:n] / N
    tp = stats.binom.pmf(np.arange(n), n, np.float32(p))
    assert r_squared(sp, tp) >= 0.711


@pytest.mark.parametrize("n,p", [(5, 0.3), (30, 0.2), (50, 0.19), (100, 0.5), (1000, 0.3),
                                 (3000, 0.85), (40, 0.9), (2000, 0.01), (60, 0.2), (12, 0.02),
                                 (400, 0.47), (21, 0.5)])
def test_binomial_goodness_of_fit(orc, n, p):
    x = orc.sample("binomial", 77, n, p, 200_000)
    assert gof_pvalue(x, lambda k: stats.binom.pmf(k, n, np.float32(p)), 0, n) > 1e-4


@pytest.mark.parametrize("lam", [0.05, 0.6, 2.5, 9.99, 10.0, 15.0, 50.0, 400.0])
def test_poisson_goodness_of_fit(orc, lam):
    x = orc.sample("poisson", 78, 0, lam, 200_000)
    hi = int(lam + 12 * math.sqrt(lam) + 12)
    assert gof_pvalue(x, lambda k: stats.poisson.pmf(k, np.float32(lam)), 0, hi) > 1e-4


@pytest.mark.parametrize("k", [0.41, 2.1, 334.3, 4343.0, 72343.0])
def test_exponential_dwell(orc, k):
    # drawTau (GenRandTest.cu:228-270): 100-bin histogram vs the exact law, r^2 >= 0.711
    x = orc.sample("exponential", 79, 0, k, 30000)
    edges = np.linspace(0, np.quantile(x, 0.99), 101)
    sp = np.histogram(x, edges)[0] / x.size
    tp = np.diff(1 - np.exp(-k * edges))
    assert r_squared(sp, tp) >= 0.711
    assert stats.kstest(x * k, "expon").pvalue > 1e-4


def test_normal(orc):
    x = orc.sample("normal", 80, 0, 0.0, 200_000)
    assert stats.kstest(x, "norm").pvalue > 1e-4


@pytest.mark.parametrize("n", [3, 4, 5, 6])
def test_drawdisidx_reference_semantics(orc, n):
    # drawDisIdx (GenRandTest.cu:189-225): weights normalised to 1 -> frequencies, r^2 >= 0.6
    w = np.random.RandomState(n).uniform(0, 1, n).astype(np.float32)
    w /= w.sum()
    x = orc.sample_cat(3, 1, w, 30000)
    sp = np.bincount(x, minlength=n) / x.size
    assert r_squared(sp, w) >= 0.6
    exp = w.astype(np.float64) / w.astype(np.float64).sum() * x.size
    assert stats.chisquare(np.bincount(x, minlength=n), exp).pvalue > 1e-4


def test_drawdisidx_unnormalised_weights_pick_first(orc):
    # Q1: genMatP gives in-rates >> 1, so drawDisIdx almost always returns 0
    x = orc.sample_cat(3, 1, [500.0, 700.0, 900.0], 10000)
    assert (x == 0).all()


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6])
def test_jump_draws_follow_k_columns(orc, n):
    # drawJ_Si2Sj (GenRandTest.cu:137-182): frequencies of j from column i vs P_i2j, r^2 >= 0.711
    rs = np.random.RandomState(10 + n)
    from gsmfretda_gb300.synth import pack_args
    K = rs.uniform(0, 1000, (n, n))
    np.fill_diagonal(K, 0)
    args = pack_args(rs.uniform(0, 1, n), K, rs.uniform(0, 10, n))
    prm = orc.build_params(n, args, orc.model())
    P = np.frombuffer(prm.Pi2j, dtype=np.float32)[:n * n].reshape(n, n).T  # [row i, col j]
    Pm = np.frombuffer(prm.Pi2j, dtype=np.float32)[:n * n]
    jc = np.frombuffer(prm.jump_cdf, dtype=np.float32).reshape(8, 8)
    for i in range(n):
        x_ref = orc.sample_cat(5 + i, 3, Pm, 30000, frm=i, n=n)
        x_pda = orc.sample_cat(5 + i, 2, jc[i, :n], 30000, frm=i, n=n)
        tp = P[:, i]
        for x in (x_ref, x_pda):
            assert not (x == i).any()
            sp = np.bincount(x, minlength=n) / x.size
            assert r_squared(sp, tp) >= 0.711
            assert np.abs(sp - tp).max() < 0.02


def test_fp32_and_fp64_samplers_make_the_same_decisions(orc):
    for kind32, kind64, n, p in [("binomial", "binomial64", 800, 0.37), ("poisson", "poisson64", 0, 23.0)]:
        a = orc.sample(kind32, 81, n, p, 50_000)
        b = orc.sample(kind64, 81, n, p, 50_000)
        assert (a != b).mean() < 1e-3


@pytest.mark.parametrize("pp", [0.5, 0.49, 0.24, 0.15, 0.05, 0.013, 1e-4])
def test_binomial_table_rows_match_exact_cdf(orc, pp):
    """Photon-mode binomial tables (double-float rows around the mode) against
    the exact CDF, for every n up to the table bound."""
    worst = 0.0
    for nn in list(range(0, 40)) + [63, 100, 127, 128, 255, 256, 300, 511]:
        row = orc.binom_cdf_row(pp, nn)
        exact = stats.binom.cdf(np.arange(nn + 1), nn, np.float64(np.float32(pp)))
        assert row[-1] == 1.0 and np.all(np.diff(row) >= 0)
        worst = max(worst, np.abs(row - exact).max())
    assert worst < 5e-7
