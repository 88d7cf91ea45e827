"""GPU parity on the edge cases of the path, unit by unit against the oracle
(bit-exact): empty and one-photon bursts, zero durations, bursts whose
segments exceed the 511-photon table bound (BINV/BTRD fallback in photon
mode), distance broadening, an absorbing state, 8 states at high rates, the
largest and smallest histograms, burst sub-ranges, batched photon mode, and
upload validation."""
import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300._lib import GpdaError
from gsmfretda_gb300.api import MODE_OCCUPANCY, MODE_PHOTON, Engine

pytestmark = pytest.mark.gpu


def _bursts(N, T, seed):
    rng = np.random.default_rng(seed)
    N = np.asarray(N, dtype=np.int32)
    T = np.asarray(T, dtype=np.float32)
    bs = synth.BurstSet(N, T)
    bs.off_idx, bs.offsets = synth.make_offsets(rng, N, T)
    return bs


def _compare(orc, bs, n, args, md, mode, S, seed, b0=0, b1=None):
    b1 = bs.B if b1 is None else b1
    m = orc.model(**md)
    kw = dict(off_idx=bs.off_idx, offsets=bs.offsets) if mode == MODE_PHOTON else {}
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, mode, S, seed, b0=b0, b1=b1, unit_out=True, **kw)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        units, hist = eng.run_units(mode, n, args, S, seed, b0, b1)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist, h_ref)
    return units


def _odd_bursts(seed=1):
    rng = np.random.default_rng(seed)
    N = np.concatenate([[0, 1, 2, 3000, 0, 700], 30 + rng.geometric(1 / 120, 200)])
    T = np.concatenate([[1e-3, 1e-3, 0.0, 8e-3, 0.0, 2e-3], rng.lognormal(np.log(1.5e-3), 0.5, 200)])
    return _bursts(N, T, seed)


@pytest.mark.parametrize("mode", [MODE_OCCUPANCY, MODE_PHOTON])
def test_odd_bursts(orc, gpda_lib, mode):
    bs = _odd_bursts()
    args = synth.random_3state_args(np.random.default_rng(2))
    u = _compare(orc, bs, 3, args, dict(synth.MODEL_DEFAULTS), mode, 12, 77)
    assert np.all(u[0, 0] == -1) and np.all(u[0, 4] == -1)        # N = 0: no value
    assert np.all((u[0, 1] >= 0) & (u[0, 1] <= 1))


@pytest.mark.parametrize("mode", [MODE_OCCUPANCY, MODE_PHOTON])
def test_distance_broadening(orc, gpda_lib, mode):
    bs = _odd_bursts(3)
    E, K, _ = synth.unpack_args(synth.random_3state_args(np.random.default_rng(4)), 3)
    args = synth.pack_args(E, K, V=[2.0, 0.0, 5.0])
    _compare(orc, bs, 3, args, dict(synth.MODEL_DEFAULTS), mode, 8, 91)


@pytest.mark.parametrize("mode", [MODE_OCCUPANCY, MODE_PHOTON])
def test_absorbing_state(orc, gpda_lib, mode):
    bs = _odd_bursts(5)
    # state 1 never leaves (K(0,1) = rate 1->0 = 0): all stationary mass there
    args = synth.pack_args([0.25, 0.75], np.array([[0.0, 0.0], [800.0, 0.0]]))
    u = _compare(orc, bs, 2, args, dict(synth.MODEL_DEFAULTS), mode, 8, 5)
    ok = bs.N > 20
    pr = u[0][ok] / bs.N[ok][:, None]
    assert pr.mean() > 0.6


@pytest.mark.parametrize("mode", [MODE_OCCUPANCY, MODE_PHOTON])
def test_eight_states_fast_rates(orc, gpda_lib, mode):
    rng = np.random.default_rng(6)
    bs = _bursts(30 + rng.geometric(1 / 80, 300), rng.lognormal(np.log(3e-3), 0.4, 300), 6)
    K = np.exp(rng.uniform(np.log(1e4), np.log(2e5), (8, 8)))
    np.fill_diagonal(K, 0.0)
    args = synth.pack_args(np.linspace(0.05, 0.95, 8), K)
    _compare(orc, bs, 8, args, dict(synth.MODEL_DEFAULTS), mode, 4, 8)


@pytest.mark.parametrize("nbins", [1, 1024])
def test_extreme_bin_counts(orc, gpda_lib, nbins):
    bs, n, args, md, _ = synth.occupancy_2state(B=500, seed=9)
    md = dict(md, nbins=nbins, left_pad=0)
    _compare(orc, bs, n, args, md, MODE_OCCUPANCY, 10, 10)


def test_burst_subrange_and_photon_batch(orc, gpda_lib):
    bs, n, args, md, _ = synth.photon_3state(B=900, seed=12)
    _compare(orc, bs, n, args, md, MODE_PHOTON, 6, 13, b0=217, b1=731)
    rng = np.random.default_rng(14)
    argsP = np.stack([synth.random_3state_args(rng) for _ in range(3)])
    _compare(orc, bs, n, argsP, md, MODE_PHOTON, 5, 15)


def test_upload_validation_rejects_bad_stores(gpda_lib):
    bs = _odd_bursts(7)
    with Engine(0) as eng:
        bad = bs.offsets.copy()
        i = int(bs.off_idx[3]) + 10                   # inside the 3000-photon burst
        bad[i], bad[i + 1] = bad[i + 1] + 1e-4, bad[i]  # out of order
        with pytest.raises(GpdaError):
            eng.upload(N=bs.N, T=bs.T, off_idx=bs.off_idx, offsets=bad)
        T = bs.T.copy()
        T[5] = np.nan
        with pytest.raises(GpdaError):
            eng.upload(N=bs.N, T=T, off_idx=bs.off_idx, offsets=bs.offsets)
        eng.upload(bs)                                 # a valid store still uploads
