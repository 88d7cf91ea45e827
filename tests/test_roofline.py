"""The ALU cost model the bench reports its roofline fraction against: the rate
matrix layout, the stationary jump flux, and the mean segments per unit
against a direct simulation of the same chain."""
import numpy as np

from gsmfretda_gb300 import roofline as rl
from gsmfretda_gb300 import synth


def test_rate_matrix_matches_the_parameter_layout():
    rng = np.random.default_rng(3)
    args = synth.random_3state_args(rng)
    _, K, _ = synth.unpack_args(args, 3)
    np.testing.assert_allclose(rl.rate_matrix(3, args), K)


def test_two_state_segments_are_one_plus_rate_times_duration():
    args = synth.pack_args([0.3, 0.72], [[0, 500.0], [500.0, 0]])
    T = np.array([1e-3, 2e-3])
    assert abs(rl.mean_segments(2, args, T) - (1.0 + 500.0 * 1.5e-3)) < 1e-9


def _simulated_segments(K, T, rng):
    n = K.shape[0]
    kexit = K.sum(axis=0)
    pi = rl.stationary(K)
    total = 0
    for Tb in T:
        s = rng.choice(n, p=pi)
        t, seg = 0.0, 1
        while True:
            t += rng.exponential(1.0 / kexit[s])
            if t >= Tb:
                break
            seg += 1
            s = rng.choice(n, p=K[:, s] / kexit[s])
        total += seg
    return total / len(T)


def test_mean_segments_match_a_direct_simulation():
    bs, n, args, md, S = synth.photon_3state(B=20000, seed=2)
    K = rl.rate_matrix(n, args)
    rng = np.random.default_rng(11)
    sim = _simulated_segments(K, bs.T.astype(np.float64), rng)
    D = rl.mean_segments(n, args, bs.T)
    assert abs(sim - D) < 0.02 * D, (sim, D)


def test_photon_ops_per_unit_formula():
    bs, n, args, md, S = synth.photon_3state(B=2000, seed=2)
    ops, D = rl.photon_ops_per_unit(n, args, bs.N, bs.T)
    Nbar = float(np.mean(bs.N))
    expect = 25 * (5 + 3 * D) + 56 * D + 4 * (D - 1) * np.log2(Nbar + 1)
    assert abs(ops - expect) < 1e-9
    b = rl.photon_ops_breakdown(n, args, bs.N, bs.T)
    assert abs(b["draws"] + b["search"] - ops) < 1e-9
    assert abs(b["linear_scan"] - 2 * Nbar) < 1e-9



def test_background_term_counts_the_poisson_pairs():
    """bg_a + bg_d = 2,300 /s over the photon_3state bursts: an exponential
    and (lam + 1) inversion steps per segment, a split trial per background
    photon; no term without background."""
    bs, n, args, md, S = synth.photon_3state(B=2000, seed=2)
    bg = md["bg_a"] + md["bg_d"]
    b = rl.photon_ops_breakdown(n, args, bs.N, bs.T, bg)
    D, lam = b["segments"], bg * float(np.mean(bs.T.astype(np.float64)))
    assert abs(b["background_photons"] - lam) < 1e-9
    assert abs(b["background"] - (16 * D + 4 * (lam + D) + 3 * lam)) < 1e-9
    assert abs(b["ops"] - (b["draws"] + b["search"] + b["background"])) < 1e-9
    assert rl.photon_ops_breakdown(n, args, bs.N, bs.T)["background"] == 0.0
