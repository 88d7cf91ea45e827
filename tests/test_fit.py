"""Fit drivers (gsmfretda_gb300.fit) on the host: coordinates, Adam and the
separable CMA-ES against objectives with a known minimum; on the GPU, both
fits on a small two-state problem recover the generating parameters."""
import numpy as np
import pytest

from gsmfretda_gb300 import fit, synth


class Quadratic(fit.FitProblem):
    """f(z) = sum c_i (z_i - t_i)^2 with the FitProblem coordinates."""

    def __init__(self, n, template, target, scales):
        super().__init__(None, n, template)
        self.t = np.asarray(target, dtype=np.float64)
        self.c = np.asarray(scales, dtype=np.float64)

    def expected(self, Z, samples, seed, grad=True):
        Z = np.atleast_2d(Z)
        d = Z - self.t
        return (self.c * d * d).sum(1), 2.0 * self.c * d

    def noisy(self, Z, samples, seed):
        f, _ = self.expected(Z, samples, seed)
        return f + np.random.default_rng(seed).normal(0.0, 1e-3, f.shape)


def test_coordinates_round_trip_and_free_rates():
    args = synth.cyclic_4state_args()
    prob = fit.FitProblem(None, 4, args)
    assert prob.free.size == 8 and prob.D == 12
    z = prob.from_args(args)
    back = prob.to_args(z)[0]
    np.testing.assert_allclose(back[:16], args[:16], rtol=2e-6)
    assert np.all(back[16:] == 0.0)
    # zero rates stay zero whatever z is
    zz = z + 0.3
    a2 = prob.to_args(zz)[0]
    assert np.array_equal(a2[4:16] == 0.0, args[4:16] == 0.0)


def test_chain_rule_of_the_coordinates():
    """d chi2 / d z from (dE, dlnK) by the chain rule equals finite
    differences of the composed map on a smooth stand-in objective."""
    args = synth.cyclic_4state_args()
    prob = fit.FitProblem(None, 4, args)

    class Eng:
        def expected_grad(self, n, a, samples, seed):
            a = np.asarray(a, dtype=np.float64)
            E = a[:, :n]
            lk = np.log(np.where(a[:, n:n * n] > 0, a[:, n:n * n], 1.0))
            f = (np.sin(3 * E).sum(1) + (0.1 * lk ** 2).sum(1))
            return None, f, 3 * np.cos(3 * E), 0.2 * lk

    prob.eng = Eng()
    z = prob.from_args(args)[0] + 0.1
    _, g = prob.expected(z, 1, 1)
    h = 1e-5
    for k in range(prob.D):
        e = np.zeros(prob.D)
        e[k] = h
        fp, _ = prob.expected(z + e, 1, 1)
        fm, _ = prob.expected(z - e, 1, 1)
        # the float32 parameter vector limits the agreement
        assert abs((fp[0] - fm[0]) / (2 * h) - g[0, k]) < 2e-2 * max(1.0, abs(g[0, k]))


def test_adam_converges_on_a_quadratic():
    args = synth.cyclic_4state_args()
    q = Quadratic(4, args, target=np.linspace(-1, 1, 12), scales=np.linspace(1, 5, 12))
    res = fit.adam(q, np.zeros(12), steps=800, lr=0.05)
    np.testing.assert_allclose(res.z, q.t, atol=2e-2)
    assert res.values[-1] < 1e-3


def test_adam_runs_parallel_starts_and_stops_early():
    args = synth.cyclic_4state_args()
    q = Quadratic(4, args, target=np.zeros(12), scales=np.ones(12))
    z0 = np.stack([np.full(12, 2.0), np.full(12, 0.1)])
    res = fit.adam(q, z0, steps=500, lr=0.05, stop=lambda t, z: np.abs(z).max() < 0.05)
    assert len(res.times) < 500
    assert res.evals == 2 * len(res.times)


def test_sep_cma_es_converges_on_a_noisy_quadratic():
    args = synth.cyclic_4state_args()
    q = Quadratic(4, args, target=np.linspace(-1, 1, 12), scales=np.linspace(1, 5, 12))
    res = fit.sep_cma_es(q, np.zeros(12), sigma0=0.5, popsize=32, evaluate=q.noisy, samples=1,
                         generations=250)
    np.testing.assert_allclose(res.z, q.t, atol=0.05)
    assert res.evals == 32 * len(res.times)


@pytest.mark.gpu
def test_gpu_fits_recover_a_two_state_system(orc, gpda_lib):
    from gsmfretda_gb300.api import MODE_OCCUPANCY, Engine
    bs, n, truth, md, _ = synth.expected_bursts(B=20000, n=2, seed=8)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        ohist, _ = eng.run_plain(MODE_OCCUPANCY, n, truth, 1, 4321)
        eng.set_observed(ohist.astype(np.float32))
        prob = fit.FitProblem(eng, n, truth)
        z_true = prob.from_args(truth)[0]
        z0 = z_true + np.array([0.4, -0.4, 0.5, -0.5])
        ra = fit.adam(prob, z0, steps=250, lr=0.05, samples=16, seed=3)
        rs = fit.sep_cma_es(prob, z0, sigma0=0.3, popsize=32, evaluate=prob.sampled_batched,
                            samples=10, generations=60)
        # yardstick: expected chi-square with many samples at an unrelated seed
        yard = lambda z: prob.expected(z, 64, 777, grad=False)[0][0]  # noqa: E731
        y_true, y_adam, y_es, y0 = yard(z_true), yard(ra.z), yard(rs.z), yard(z0)
    assert y_adam < 0.2 * y0 and y_es < 0.2 * y0
    assert y_adam < 1.5 * y_true + 0.5
    Ea = prob.to_args(ra.z)[0][:n]
    np.testing.assert_allclose(np.sort(Ea), np.sort(truth[:n]), atol=0.03)
