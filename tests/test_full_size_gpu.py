"""GPU parity at the full sizes of the benchmark workloads: every histogram
count and every FP64 reduced chi-square equal to the CPU oracle's on the same
Philox counters (the oracle runs on all host cores; the largest case is
6.4e8 units).

  occupancy_2state  4,000 bursts x 10 samples, 2 states           units + hist + chi2
  photon_3state     100,000 bursts x 100 samples, photon by photon units + hist + chi2
  population_256    256 sets x 50,000 bursts x 50 samples, through the
                    captured graph after the tile autotuner      hist + chi2
  fit_4state        64 sets x 1,000,000 bursts x 10 samples, 4 states, 41 bins
                                                                  hist + chi2
  photon heavy tail Pareto(1.8) photon counts up to 3,000 with slow rates, so
                    segments hold more photons than the tabulated binomial CDFs
                    cover (n > 511: BINV / BTRD in the photon step)  units
"""
import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300.api import MODE_OCCUPANCY, MODE_PHOTON, Engine

pytestmark = pytest.mark.gpu


def _observed(orc, bs, n, args, m, mode, seed=99):
    kw = dict(off_idx=bs.off_idx, offsets=bs.offsets) if mode == MODE_PHOTON else {}
    h, _ = orc.run_pda(bs.N, bs.T, n, args, m, mode, 1, seed, **kw)
    return h[0].astype(np.float32)


def _chi2_ref(orc, h_ref, ohist, md, S, n):
    return np.array([orc.chi2(h, ohist, md["nbins"], md["left_pad"], S, n) for h in h_ref])


def test_occupancy_2state_full(orc, gpda_lib):
    bs, n, args, md, S = synth.occupancy_2state(B=4000, seed=1)
    m = orc.model(**md)
    ohist = _observed(orc, bs, n, args, m, MODE_OCCUPANCY)
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 2024, unit_out=True)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        units, hist_u = eng.run_units(MODE_OCCUPANCY, n, args, S, 2024)
        hist, chi2 = eng.run_plain(MODE_OCCUPANCY, n, args, S, 2024)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist_u, h_ref)
    np.testing.assert_array_equal(hist, h_ref[0])
    assert chi2 == _chi2_ref(orc, h_ref, ohist, md, S, n)[0]


def test_photon_3state_full(orc, gpda_lib):
    bs, n, args, md, S = synth.photon_3state(B=100000, seed=2)
    m = orc.model(**md)
    ohist = _observed(orc, bs, n, args, m, MODE_PHOTON)
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, 1, S, 2024, off_idx=bs.off_idx,
                               offsets=bs.offsets, unit_out=True)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        units, _ = eng.run_units(MODE_PHOTON, n, args, S, 2024)
        hist, chi2 = eng.run_batched(MODE_PHOTON, n, args, S, 2024)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist, h_ref)
    np.testing.assert_array_equal(chi2, _chi2_ref(orc, h_ref, ohist, md, S, n))


def test_population_256_graph_full(orc, gpda_lib):
    bs, n, args, md, S = synth.population_256(B=50000, P=256, seed=3)
    m = orc.model(**md)
    ohist = _observed(orc, bs, n, args[0], m, MODE_OCCUPANCY)
    h_ref, _ = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 31)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        tile = eng.autotune(MODE_OCCUPANCY, n, args, S)
        eng.graph_create(MODE_OCCUPANCY, n, 256, S)
        hist, chi2 = eng.graph_run(args, 31)
    assert 1 <= tile <= 256
    np.testing.assert_array_equal(hist, h_ref)
    np.testing.assert_array_equal(chi2, _chi2_ref(orc, h_ref, ohist, md, S, n))


def test_fit_4state_population_full(orc, gpda_lib):
    bs, n, truth, md, P = synth.fit_4state(B=1000000, seed=5)
    md = dict(md, nbins=41)
    S = 10
    args = np.stack([truth] + [synth.perturb_args(truth, n, seed=i) for i in range(1, P)])
    m = orc.model(**md)
    ohist = _observed(orc, bs, n, truth, m, MODE_OCCUPANCY)
    h_ref, _ = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 77)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        hist, chi2 = eng.run_batched(MODE_OCCUPANCY, n, args, S, 77)
    np.testing.assert_array_equal(hist, h_ref)
    np.testing.assert_array_equal(chi2, _chi2_ref(orc, h_ref, ohist, md, S, n))


def test_photon_heavy_tail_beyond_tables(orc, gpda_lib):
    rng = np.random.default_rng(41)
    B = 30000
    N = synth._pareto_N(rng, B, 1.8, 30, 3000)
    T = synth._lognormal_T(rng, B, 2e-3, 0.6)
    bs = synth.BurstSet(N, T, *synth.make_offsets(rng, N, T))
    n = 2
    # slow exchange: most bursts are one or two segments, so segments carry
    # up to 3,000 photons
    args = synth.pack_args([0.35, 0.8], np.array([[0.0, 60.0], [90.0, 0.0]]))
    md = dict(synth.MODEL_DEFAULTS)
    m = orc.model(**md)
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, 1, 8, 5150, off_idx=bs.off_idx,
                               offsets=bs.offsets, unit_out=True)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        units, hist = eng.run_units(MODE_PHOTON, n, args, 8, 5150)
    assert int(N.max()) > 2000 and int((N > 511).sum()) > 100, int((N > 511).sum())
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist, h_ref)
