"""The oracle's models against exact analytic limits and its own invariants
(CPU only).

- Static states (rates << 1/T): the proximity-ratio histogram is the
  pi-weighted mixture over bursts of Binomial(N_b, E_s) binned by A*nbins/N.
- ref-compat static limit: one dwell window covers the burst, so mc_kernel's
  photon-counting rule (src/mc.cu:140-181) gives (f_id, f_ia) per burst and
  mcE = Binomial(round(f_if), E)/f_if; the rule is restated here in Python.
- The FP64 transcription agrees with the FP32 path unit by unit except where
  rounding moves a decision, and in bin mass within 1e-3.
- Linearity over burst sub-ranges, determinism over thread counts.
"""
import numpy as np
import pytest
from scipy import stats

from gsmfretda_gb300 import synth

NB = 21


def static_args(E, rates):
    n = len(E)
    K = np.zeros((n, n))
    k = iter(rates)
    for i in range(n):
        for j in range(n):
            if i != j:
                K[i, j] = next(k)
    return synth.pack_args(E, K), K


def stationary(K):
    n = K.shape[0]
    Q = K - np.diag(K.sum(axis=0))
    A = Q.copy()
    A[-1, :] = 1.0
    b = np.zeros(n)
    b[-1] = 1.0
    return np.linalg.solve(A, b)


def mixture_masses(N, E, pi, nbins=NB):
    masses = np.zeros(nbins)
    for Nb in np.unique(N):
        cnt = (N == Nb).sum()
        A = np.arange(Nb + 1)
        bins = np.minimum(A * nbins // Nb, nbins - 1)
        for e, w in zip(E, pi):
            pmf = stats.binom.pmf(A, Nb, e)
            masses += cnt * w * np.bincount(bins, weights=pmf, minlength=nbins)
    return masses / N.size


@pytest.mark.parametrize("mode", [0, 1])
def test_static_limit_is_binomial_mixture(orc, mode):
    bs, _, _, _, _ = synth.photon_3state(B=20000, seed=31)
    E = [0.25, 0.8]
    args, K = static_args(E, [1e-3, 3e-3])          # rate 1->0 = 1e-3, rate 0->1 = 3e-3
    pi = stationary(K)
    m = orc.model(bg_d=0.0, bg_a=0.0, crosstalk=0.0, gamma=1.0)
    S = 100
    h, _ = orc.run_pda(bs.N, bs.T, 2, args, m, mode, S, 17, off_idx=bs.off_idx, offsets=bs.offsets)
    got = h[0] / (bs.B * S)
    want = mixture_masses(bs.N, E, pi)
    assert np.abs(got - want).max() < 1e-3
    sigma = np.sqrt(np.maximum(want * (1 - want), 1e-12) / (bs.B * S))
    # samples within a burst are not independent draws of the mixture weight
    assert (np.abs(got - want) / sigma).max() < 12


def test_crosstalk_and_gamma_shift_the_mean(orc):
    bs, _, _, _, _ = synth.occupancy_2state(B=4000, seed=32)
    args, _ = static_args([0.5, 0.5], [1e-3, 1e-3])
    for g, ct in [(1.0, 0.0), (0.5, 0.0), (1.0, 0.2), (2.0, 0.1)]:
        m = orc.model(bg_d=0.0, bg_a=0.0, crosstalk=ct, gamma=g)
        _, u = orc.run_pda(bs.N, bs.T, 2, args, m, 0, 50, 3, unit_out=True)
        pr = (u[0] / bs.N[:, None]).mean()
        eps = (g * 0.5 + ct * 0.5) / (g * 0.5 + (1 + ct) * 0.5)
        assert abs(pr - eps) < 3e-3


def test_background_mean(orc):
    bs, _, _, _, _ = synth.occupancy_2state(B=4000, seed=33)
    args, _ = static_args([0.4, 0.4], [1e-3, 1e-3])
    m = orc.model(bg_d=3000.0, bg_a=2000.0, crosstalk=0.0, gamma=1.0)
    _, u = orc.run_pda(bs.N, bs.T, 2, args, m, 0, 50, 4, unit_out=True)
    A = u[0].astype(np.float64)
    lam_a = 2000.0 * bs.T.astype(np.float64)
    lam_d = 3000.0 * bs.T.astype(np.float64)
    # E[A] = E[Ba] + 0.4 E[N - Ba - Bd]; lam_a + lam_d ~ 9 << N >= 31, clipping negligible
    want = lam_a + 0.4 * (bs.N - lam_a - lam_d)
    assert abs(A.mean() - want.mean()) < 0.005 * want.mean()


def ref_window_counts(d, b, gam=0.34, ct=0.07, de=0.08):
    """mc_kernel's photon scan for one window [start, stop] (src/mc.cu:140-181)."""
    s, n = int(d["istart"][b]), int(d["phCount"][b])
    bad = d["burst_ad"][s:s + n]
    bdd = d["burst_dd"][s:s + n]
    stop = d["stop"][b]
    sdd = sad = False
    f_id = f_ia = 0
    for i in range(n):
        ddx, adx = bdd[i], bad[i]
        if ddx >= stop or adx >= stop or i == n - 1:
            break
        if ddx > 0:
            sdd = True
        if adx > 0:
            sad = True
        if sad and sdd:
            continue
        if sad:
            f_ia += 1
        if sdd:
            f_id += 1
    f_if = np.float32(np.float32(gam - ct) * np.float32(f_id)) + \
        np.float32(np.float32(1.0 - de) * np.float32(f_ia))
    return f_id, f_ia, np.float32(f_if)


def test_refcompat_static_limit(orc):
    d = synth.photon_stream(B=600, seed=41, bg_ad_rate=0.0, bg_dd_rate=0.0)
    E = [0.3, 0.65]
    args, _ = static_args(E, [1e-3, 1e-3])
    m = orc.model()
    R = 400
    _, e = orc.run_refcompat(d, 2, args, m, R, 9)
    chi2, dof = 0.0, 0
    for b in range(600):
        f_id, f_ia, f_if = ref_window_counts(d, b)
        x = e[b]
        if f_if <= 0:
            assert (x == 0).all()
            continue
        f_i = int(np.floor(np.float64(f_if) + 0.5))
        ai = np.rint(x.astype(np.float64) * np.float64(f_if)).astype(np.int64)
        assert (ai >= 0).all() and (ai <= f_i).all()
        # tiny rates make genMatP's weights ~1e-3, so drawDisIdx returns the last state
        pmf = stats.binom.pmf(np.arange(f_i + 1), f_i, E[1])
        obs = np.bincount(ai, minlength=f_i + 1)
        keep = pmf * R >= 5
        if keep.sum() >= 2:
            o = np.append(obs[keep], obs[~keep].sum())
            ex = np.append(pmf[keep], pmf[~keep].sum()) * R
            ok = ex > 0
            chi2 += (((o[ok] - ex[ok]) ** 2) / ex[ok]).sum()
            dof += ok.sum() - 1
    assert dof > 100
    assert stats.chi2.sf(chi2, dof) > 1e-4


def test_fp64_transcription_agrees(orc):
    bs, n, args, md, _ = synth.photon_3state(B=5000, seed=34)
    m = orc.model(**md)
    for mode in (0, 1):
        h32, u32 = orc.run_pda(bs.N, bs.T, n, args, m, mode, 20, 8, off_idx=bs.off_idx,
                               offsets=bs.offsets, unit_out=True)
        h64, u64 = orc.run_pda(bs.N, bs.T, n, args, m, mode, 20, 8, off_idx=bs.off_idx,
                               offsets=bs.offsets, unit_out=True, f64=True)
        assert (u32 != u64).mean() < 1e-3
        tot = u32.size
        assert np.abs(h32.astype(np.float64) - h64.astype(np.float64)).max() / tot <= 1e-3


def test_subrange_additivity_and_thread_independence(orc):
    bs, n, args, md, S = synth.photon_3state(B=3000, seed=35)
    m = orc.model(**md)
    kw = dict(off_idx=bs.off_idx, offsets=bs.offsets)
    full, uf = orc.run_pda(bs.N, bs.T, n, args, m, 1, 10, 5, unit_out=True, nthreads=1, **kw)
    a, ua = orc.run_pda(bs.N, bs.T, n, args, m, 1, 10, 5, b0=0, b1=1234, unit_out=True, nthreads=3, **kw)
    b, ub = orc.run_pda(bs.N, bs.T, n, args, m, 1, 10, 5, b0=1234, b1=3000, unit_out=True, **kw)
    np.testing.assert_array_equal(full, a + b)
    np.testing.assert_array_equal(uf, np.concatenate([ua, ub], axis=1))
    other, _ = orc.run_pda(bs.N, bs.T, n, args, m, 1, 10, 6, **kw)
    assert not np.array_equal(full, other)


def test_edge_cases(orc):
    N = np.array([0, 1, 5, 30, 2000], dtype=np.int32)
    T = np.array([1e-3, 0.0, 2e-3, 1e-3, 5e-3], dtype=np.float32)
    off_idx = np.concatenate([[0], np.cumsum(N)]).astype(np.int64)
    rng = np.random.default_rng(0)
    offs = np.concatenate([np.sort(rng.uniform(0, t, k)).astype(np.float32) for k, t in zip(N, T)])
    args, _ = static_args([0.2, 0.7], [300.0, 800.0])
    m = orc.model()
    for mode in (0, 1):
        h, u = orc.run_pda(N, T, 2, args, m, mode, 16, 1, off_idx=off_idx, offsets=offs, unit_out=True)
        assert (u[0, 0] == -1).all()                         # N = 0: no PR, not counted
        assert ((u[0, 1:] >= 0) & (u[0, 1:] <= N[1:, None])).all()
        assert h.sum() == 4 * 16
    # absorbing state: 0 -> 1 never happens, stationary mass all in state 0
    args_abs, _ = static_args([0.1, 0.9], [100.0, 0.0])   # rate 1->0 = 100, rate 0->1 = 0
    h, u = orc.run_pda(N, T, 2, args_abs, orc.model(bg_d=0, bg_a=0, crosstalk=0), 0, 64, 2,
                       unit_out=True)
    pr = u[0, 4] / N[4]
    assert abs(pr.mean() - 0.1) < 0.01
    # singular chain is rejected
    args_sing, _ = static_args([0.1, 0.9], [0.0, 0.0])
    with pytest.raises(ValueError):
        orc.run_pda(N, T, 2, args_sing, m, 0, 4, 1)


@pytest.mark.parametrize("lam", [0.5, 5.0, 9.9])
@pytest.mark.parametrize("pa", [800.0 / 2300.0, 0.1])
def test_background_pair_joint_law_is_two_independent_poissons(orc, lam, pa):
    """The photon step's background pair (A, D) drawn from one uniform (the
    total by inversion, then Bernoulli splits on the uniform's rescaled
    residual; the GPU matches this mirror bit for bit) against independent
    Poisson(lam pa) x Poisson(lam (1 - pa)): chi-square goodness of fit over
    the joint table (cells with expectation below 5 lumped), 2e6 variates."""
    from scipy import stats
    la, ld = lam * pa, lam * (1.0 - pa)
    A, D = orc.sample_bgpair(11, np.float32(la), np.float32(ld), 1.0, 2_000_000)
    K = 40
    obs = np.zeros((K, K))
    np.add.at(obs, (np.minimum(A, K - 1), np.minimum(D, K - 1)), 1)
    pmf_a = stats.poisson.pmf(np.arange(K), la)
    pmf_a[-1] = stats.poisson.sf(K - 2, la)
    pmf_d = stats.poisson.pmf(np.arange(K), ld)
    pmf_d[-1] = stats.poisson.sf(K - 2, ld)
    exp = np.outer(pmf_a, pmf_d) * A.size
    keep = exp >= 5.0
    o = np.append(obs[keep], obs[~keep].sum())
    e = np.append(exp[keep], exp[~keep].sum())
    chi = float(((o - e) ** 2 / e).sum())
    p = stats.chi2.sf(chi, o.size - 1)
    assert p > 1e-4, (chi, o.size - 1, p)
    assert abs(np.corrcoef(A, D)[0, 1]) < 5e-3
