"""GPU parity: every kernel against the CPU oracle on the same Philox
counters. Integer outputs (per-unit acceptor counts, histogram counts) must be
bit-exact; the FP64 reduced chi-square is compared exactly too (same
sequential operation order on both sides)."""
import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300.api import MODE_OCCUPANCY, MODE_PHOTON, Engine

pytestmark = pytest.mark.gpu


def _engine(model):
    return Engine(0, **model)


def test_occupancy_units_bit_exact(orc, gpda_lib):
    bs, n, args, md, S = synth.occupancy_2state(B=3000, seed=11)
    m = orc.model(**md)
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 777, unit_out=True)
    with _engine(md) as eng:
        eng.upload(bs)
        units, hist = eng.run_units(MODE_OCCUPANCY, n, args, S, 777)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist, h_ref)


def test_photon_units_bit_exact(orc, gpda_lib):
    bs, n, args, md, S = synth.photon_3state(B=2000, seed=12)
    m = orc.model(**md)
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, 1, 20, 4242, off_idx=bs.off_idx,
                               offsets=bs.offsets, unit_out=True)
    with _engine(md) as eng:
        eng.upload(bs)
        units, hist = eng.run_units(MODE_PHOTON, n, args, 20, 4242)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist, h_ref)


def test_plain_hist_and_chi2_exact(orc, gpda_lib):
    bs, n, args, md, S = synth.occupancy_2state(B=4000, seed=13)
    m = orc.model(**md)
    obs_h, _ = orc.run_pda(bs.N, bs.T, n, args, m, 0, 1, 99)   # observed set at a held-out seed
    ohist = obs_h[0].astype(np.float32)
    h_ref, _ = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 5)
    chi_ref = orc.chi2(h_ref[0], ohist, md["nbins"], md["left_pad"], S, n)
    with _engine(md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        hist, chi2 = eng.run_plain(MODE_OCCUPANCY, n, args, S, 5)
    np.testing.assert_array_equal(hist, h_ref[0])
    assert chi2 == chi_ref


def test_batched_population_exact(orc, gpda_lib):
    bs, n, _, md, S = synth.population_256(B=1500, P=6, seed=14)
    args = synth.population_args(6, 77)
    m = orc.model(**md)
    h_ref, _ = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 31)
    with _engine(md) as eng:
        eng.upload(bs)
        hist, _ = eng.run_batched(MODE_OCCUPANCY, n, args, S, 31)
    np.testing.assert_array_equal(hist, h_ref)


def test_refcompat_mc_dropin_bit_exact(orc, gpda_lib):
    from gsmfretda_gb300.mc import mc
    d = synth.photon_stream(B=1500, seed=21)
    n = 3
    args = synth.random_3state_args(np.random.default_rng(5))
    md = synth.MODEL_DEFAULTS
    m = orc.model(**md)
    R = 4
    nbins = 50
    pdamc = mc(0, 2)
    pdamc.set_seed(1000)
    pdamc.set_hist_bins(nbins)
    pdamc.init_data_gpu(d["istart"], d["start"], d["stop"], d["phCount"], d["times"].size,
                        d["burst_ad"], d["burst_dd"], d["T"], synth.sgdivsr(d), d["clk_p"],
                        d["bg_ad_rate"], d["bg_dd_rate"])
    sid = 1
    old = pdamc.set_nstates(n, sid)
    assert pdamc.set_params(n, sid, args)
    N = pdamc.setBurstBd(0, 1500, sid)
    assert N == 1500
    pdamc.init_randstate(N, sid)
    pdamc.set_params_buff(old, N, sid)
    pdamc.run_kernel(N, sid)
    while not pdamc.streamQuery(sid):
        pass
    got = pdamc.hmcE(sid).reshape(N, R)
    ghist = pdamc.hist(sid, nbins)
    pdamc.close()
    m.nbins = nbins
    h_ref, e_ref = orc.run_refcompat(d, n, args, m, R, 1000 + sid)
    np.testing.assert_array_equal(got.view(np.uint32), e_ref.view(np.uint32))
    np.testing.assert_array_equal(ghist, h_ref.astype(np.float32))
