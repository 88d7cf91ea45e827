"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py).

ref_binomial.npz holds histograms of the reference's own rk_binomial
(src/binom.cuh) over a grid of (n, p). The oracle's binomial sampler must be
statistically indistinguishable from it (two-sample chi-square homogeneity
test) and both must fit the exact law. Where the reference tree is mounted
the fixture itself is re-derived from the reference sampler and compared.
oracle_small.npz pins the oracle's own per-unit outputs (regression)."""
import ctypes as C
import os

import numpy as np
import pytest
from scipy import stats

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def homogeneity_p(h1, h2, min_cell=10):
    """Two-sample chi-square test on count vectors (cells with few counts lumped)."""
    h1 = np.asarray(h1, dtype=np.float64)
    h2 = np.asarray(h2, dtype=np.float64)
    tot = h1 + h2
    keep = tot >= min_cell
    a = np.append(h1[keep], h1[~keep].sum())
    b = np.append(h2[keep], h2[~keep].sum())
    cols = (a + b) > 0
    table = np.vstack([a[cols], b[cols]])
    if table.shape[1] < 2:
        return 1.0
    return stats.chi2_contingency(table, correction=False)[1]


def gof_p(h, pmf, min_exp=10):
    h = np.asarray(h, dtype=np.float64)
    exp = pmf * h.sum()
    keep = exp >= min_exp
    o = np.append(h[keep], h[~keep].sum())
    e = np.append(exp[keep], exp[~keep].sum())
    ok = e > 0
    return stats.chisquare(o[ok], e[ok] * o[ok].sum() / e[ok].sum()).pvalue


@pytest.fixture(scope="module")
def ref_binom():
    d = np.load(os.path.join(HERE, "ref_binomial.npz"))
    return d["grid"], d["hist"], int(d["draws"])


def test_fixture_shape(ref_binom):
    grid, H, draws = ref_binom
    assert grid.shape[0] == H.shape[0] >= 26
    assert (H.sum(axis=1) == draws).all()


def test_oracle_binomial_matches_reference_sampler(orc, ref_binom):
    grid, H, draws = ref_binom
    worst = 1.0
    for i, (n, p) in enumerate(grid):
        n = int(n)
        x = orc.sample("binomial", 555 + i, n, float(p), draws).astype(np.int64)
        h_orc = np.bincount(x, minlength=n + 1)
        h_ref = H[i, :n + 1]
        worst = min(worst, homogeneity_p(h_orc, h_ref))
        pmf = stats.binom.pmf(np.arange(n + 1), n, np.float32(p))
        assert gof_p(h_ref, pmf) > 1e-5, ("reference sampler vs exact law", n, p)
        assert gof_p(h_orc, pmf) > 1e-5, ("oracle vs exact law", n, p)
    # 26 tests: a family-wise floor
    assert worst > 1e-5


def test_reference_thresholds_on_reference_grid(ref_binom):
    """r^2 >= 0.711 between the reference sampler's histogram and the exact law
    (tests/GenRandTest.cu:347-350) holds for the fixture itself."""
    grid, H, draws = ref_binom
    for i, (n, p) in enumerate(grid[:16]):
        n = int(n)
        sp = H[i, :n] / draws
        tp = stats.binom.pmf(np.arange(n), n, np.float32(p))
        assert np.corrcoef(sp, tp)[0, 1] ** 2 >= 0.711


def test_fixture_rederived_from_reference():
    import build_ref
    if not build_ref.available() and not os.path.exists(build_ref.LIB):
        pytest.skip("reference tree not mounted here")
    lib = C.CDLL(build_ref.build())
    lib.ref_binomial_many.argtypes = [C.c_ulonglong, C.c_int, C.c_double, C.c_long, C.c_void_p]
    d = np.load(os.path.join(HERE, "ref_binomial.npz"))
    for i in (0, 17, 20, 25):
        n, p = int(d["grid"][i, 0]), float(d["grid"][i, 1])
        out = np.zeros(int(d["draws"]), dtype=np.int64)
        lib.ref_binomial_many(1000003 + 7919 * i, n, float(np.float32(p)), out.size, out.ctypes.data)
        np.testing.assert_array_equal(np.bincount(out, minlength=n + 1), d["hist"][i, :n + 1])


def test_oracle_regression_vectors(orc):
    from gsmfretda_gb300 import synth
    g = np.load(os.path.join(HERE, "oracle_small.npz"))
    bs, n, args, md, S = synth.occupancy_2state(B=200, seed=101)
    m = orc.model(**md)
    _, u = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 2718, unit_out=True)
    np.testing.assert_array_equal(u, g["occ_units"])
    bs, n, args, md, S = synth.photon_3state(B=200, seed=102)
    _, u = orc.run_pda(bs.N, bs.T, n, args, m, 1, 8, 3141, off_idx=bs.off_idx,
                       offsets=bs.offsets, unit_out=True)
    np.testing.assert_array_equal(u, g["pho_units"])
    d = synth.photon_stream(B=100, seed=103)
    args3 = synth.random_3state_args(np.random.default_rng(104))
    _, e = orc.run_refcompat(d, 3, args3, m, 4, 1618)
    np.testing.assert_array_equal(e.view(np.uint32), g["rc_mcE"].view(np.uint32))
