"""The FP64 expected-histogram oracle (checker of gpda_expected_hist and its
adjoint): its gradient against common-random-number central differences of
its own forward, its forward against the sampled occupancy model, and the
invariants of the likelihood-ratio form."""
import numpy as np
import pytest

from gsmfretda_gb300 import synth


def _vec(args, n):
    a = np.asarray(args, dtype=np.float64)
    return np.concatenate([a[:n], np.log(a[n:n * n])])


def _args(v, n, base):
    a = np.array(base, dtype=np.float64).copy()
    a[:n] = v[:n]
    a[n:n * n] = np.exp(v[n:])
    return a.astype(np.float32)


def _setup(orc, n, B=400):
    bs, n, truth, md, _ = synth.expected_bursts(B=B, n=n, seed=4)
    m = orc.model(**md)
    h_obs, _ = orc.run_pda(bs.N, bs.T, n, truth, m, 0, 1, 999)
    return bs, n, truth, m, h_obs[0].astype(np.float32)


@pytest.mark.parametrize("n", [2, 3])
def test_gradient_matches_central_differences(orc, n):
    bs, n, truth, m, obs = _setup(orc, n)
    th0 = synth.perturb_args(truth, n, seed=1)
    S, seed, h = 16, 7, 1e-4
    _, chi, dE, dK = orc.expected(bs.N, bs.T, n, th0, m, S, seed, obs)
    g = np.concatenate([dE[0], dK[0]])
    v0 = _vec(th0, n)
    fd = np.zeros_like(g)
    for k in range(v0.size):
        ap = _args(v0 + h * np.eye(v0.size)[k], n, th0)
        am = _args(v0 - h * np.eye(v0.size)[k], n, th0)
        # the step actually taken after rounding the parameters to float32
        step = (_vec(ap, n) - _vec(am, n))[k]
        _, cp, _, _ = orc.expected(bs.N, bs.T, n, ap, m, S, seed, obs, anchor=th0, grad=False)
        _, cm, _, _ = orc.expected(bs.N, bs.T, n, am, m, S, seed, obs, anchor=th0, grad=False)
        fd[k] = (cp[0] - cm[0]) / step
    scale = np.abs(fd).max()
    assert np.abs(g - fd).max() <= 1e-4 * scale, (g, fd)
    # component by component: 1e-3 relative above a floor of 1e-3 of the largest
    big = np.abs(fd) >= 1e-3 * scale
    rel = np.abs(g - fd)[big] / np.abs(fd)[big]
    assert np.all(rel <= 1e-3), (rel, g, fd)


def test_anchor_equal_to_params_is_the_plain_form(orc):
    bs, n, truth, m, obs = _setup(orc, 3)
    th = synth.perturb_args(truth, n, seed=2)
    h1, c1, e1, k1 = orc.expected(bs.N, bs.T, n, th, m, 8, 3, obs)
    h2, c2, e2, k2 = orc.expected(bs.N, bs.T, n, th, m, 8, 3, obs, anchor=th)
    # (the oracle's threads add their partial sums in a varying order)
    np.testing.assert_allclose(h1, h2, rtol=1e-12)
    np.testing.assert_allclose(c1, c2, rtol=1e-12)
    np.testing.assert_allclose(k1, k2, rtol=1e-10, atol=1e-12 * np.abs(k1).max())


def test_mass_sums_to_units(orc):
    """At the anchor every unit with photons spreads exactly one unit of mass."""
    bs, n, truth, m, obs = _setup(orc, 3, B=300)
    S = 8
    H, _, _, _ = orc.expected(bs.N, bs.T, n, truth, m, S, 5, obs, grad=False)
    units = int((bs.N > 0).sum()) * S
    assert abs(H.sum() - units) < 1e-9 * units


def test_matches_the_sampled_model_in_distribution(orc):
    """The expected histogram and the sampled occupancy model's histogram
    estimate the same distribution (different uniforms: a z-test per bin)."""
    bs, n, truth, m, obs = _setup(orc, 3, B=3000)
    S = 32
    H, _, _, _ = orc.expected(bs.N, bs.T, n, truth, m, S, 11, obs, grad=False)
    hs, _ = orc.run_pda(bs.N, bs.T, n, truth, m, 0, S, 12)
    hs = hs[0].astype(np.float64)
    # variance of a sampled bin count plus the trajectory noise of the expected one
    z = (hs - H[0]) / np.sqrt(2.0 * np.maximum(H[0], 1.0))
    assert np.abs(z).max() < 5.0, z


def test_static_limit_is_a_binomial_mixture(orc):
    """Rates far below 1/T: no jumps inside a burst, so each unit is
    Binomial(sig, eps(E_s0)); summed over units and states with pi weights the
    mass of state s is proportional to pi_s."""
    bs, n, truth, m, obs = _setup(orc, 2, B=500)
    args = synth.pack_args([0.25, 0.8], np.array([[0.0, 1e-3], [3e-3, 0.0]]))
    H, _, dE, dK = orc.expected(bs.N, bs.T, n, args, m, 64, 9, obs)
    lo = H[0][: m.nbins // 2].sum()
    hi = H[0][m.nbins // 2:].sum()
    # K(i,j) = rate j->i: rate 0->1 = 3e-3, rate 1->0 = 1e-3, so pi_1 = 0.75
    assert abs(hi / (lo + hi) - 0.75) < 0.02
    assert np.all(np.isfinite(dE)) and np.all(np.isfinite(dK))


def test_rejects_broadening_and_large_n(orc):
    bs, n, truth, m, obs = _setup(orc, 2, B=50)
    a = np.array(truth, dtype=np.float32).copy()
    a[n * n] = 1.0
    with pytest.raises(ValueError):
        orc.expected(bs.N, bs.T, n, a, m, 4, 1, obs)
    with pytest.raises(ValueError):
        orc.expected(bs.N, bs.T, 5, np.full(30, 100.0, dtype=np.float32), m, 4, 1, obs)
