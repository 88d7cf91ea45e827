"""Captured batched launches (gpda_graph_create / gpda_graph_run) and tile
autotuning: replays equal gpda_run_batched bit for bit whatever the seed and
parameters of each replay, the tile chosen by the autotuner changes no result,
and uploading bursts drops the captured graph."""
import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300._lib import GpdaError
from gsmfretda_gb300.api import MODE_OCCUPANCY, MODE_PHOTON, Engine

pytestmark = pytest.mark.gpu


def _population(P, seed):
    return synth.population_args(P, seed)


def test_graph_replays_match_batched_occupancy(gpda_lib):
    bs, n, _, md, S = synth.population_256(B=3000, P=8, seed=31)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        ref_h, _ = eng.run_plain(MODE_OCCUPANCY, n, _population(1, 1)[0], 1, 5)
        eng.set_observed(ref_h.astype(np.float32))
        eng.graph_create(MODE_OCCUPANCY, n, 8, S)
        for r in range(3):
            args = _population(8, 100 + r)
            hg, cg = eng.graph_run(args, 1000 + r)
            hb, cb = eng.run_batched(MODE_OCCUPANCY, n, args, S, 1000 + r)
            np.testing.assert_array_equal(hg, hb)
            np.testing.assert_array_equal(cg, cb)
        # a different seed changes the result
        h2, _ = eng.graph_run(_population(8, 100), 5555)
        assert not np.array_equal(h2, eng.run_batched(MODE_OCCUPANCY, n, _population(8, 100), S, 1000)[0])


def test_graph_replays_match_batched_photon(gpda_lib):
    bs, n, args, md, S = synth.photon_3state(B=1500, seed=32)
    rng = np.random.default_rng(3)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.graph_create(MODE_PHOTON, n, 2, 20)
        for r in range(2):
            a2 = np.stack([synth.random_3state_args(rng) for _ in range(2)])
            hg, cg = eng.graph_run(a2, 77 + r)
            hb, cb = eng.run_batched(MODE_PHOTON, n, a2, 20, 77 + r)
            np.testing.assert_array_equal(hg, hb)
            assert np.all(np.isnan(cg))          # no observed histogram: no chi-square


def test_autotune_changes_no_result_and_upload_drops_the_graph(gpda_lib):
    bs, n, _, md, S = synth.population_256(B=4000, P=4, seed=33)
    args = _population(4, 9)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        h0, _ = eng.run_batched(MODE_OCCUPANCY, n, args, S, 42)
        tile = eng.autotune(MODE_OCCUPANCY, n, args, S)
        assert 1 <= tile <= 256
        h1, _ = eng.run_batched(MODE_OCCUPANCY, n, args, S, 42)
        np.testing.assert_array_equal(h0, h1)
        eng.graph_create(MODE_OCCUPANCY, n, 4, S)
        hg, _ = eng.graph_run(args, 42)
        np.testing.assert_array_equal(hg, h0)
        eng.upload(bs)
        with pytest.raises(GpdaError):
            eng.graph_run(args, 42)


@pytest.mark.parametrize("ranges", [1, 4, 7])
def test_run_host_equals_upload_and_batched(gpda_lib, ranges):
    """Upload overlapped with the simulation: same results as uploading first."""
    bs, n, args, md, S = synth.photon_3state(B=2500, seed=41)
    rng = np.random.default_rng(42)
    argsP = np.stack([synth.random_3state_args(rng) for _ in range(2)])
    with Engine(0, **md) as eng:
        eng.upload(bs)
        obs, _ = eng.run_plain(MODE_PHOTON, n, args, 1, 9)
        eng.set_observed(obs.astype(np.float32))
        hb, cb = eng.run_batched(MODE_PHOTON, n, argsP, 10, 77)
        hh, ch = eng.run_host(MODE_PHOTON, n, argsP, 10, 77, bs=bs, ranges=ranges)
        np.testing.assert_array_equal(hh, hb)
        np.testing.assert_array_equal(ch, cb)
        # the store stays uploaded
        h2, c2 = eng.run_batched(MODE_PHOTON, n, argsP, 10, 77)
        np.testing.assert_array_equal(h2, hb)
    bo, no, ao, mo, So = synth.occupancy_2state(B=3000, seed=43)
    with Engine(0, **mo) as eng:
        eng.upload(bo)
        hb, _ = eng.run_batched(MODE_OCCUPANCY, no, ao, So, 5)
        hh, _ = eng.run_host(MODE_OCCUPANCY, no, ao, So, 5, N=bo.N, T=bo.T, ranges=ranges)
        np.testing.assert_array_equal(hh, hb)


def test_run_host_rejects_a_bad_range(gpda_lib):
    bs, n, args, md, S = synth.photon_3state(B=2000, seed=44)
    bad = bs.offsets.copy()
    i = int(bs.off_idx[1500]) + 3                     # in the last of 4 ranges
    bad[i], bad[i + 1] = bad[i + 1] + 1e-4, bad[i]
    with Engine(0, **md) as eng:
        with pytest.raises(GpdaError):
            eng.run_host(MODE_PHOTON, n, args, 4, 1, N=bs.N, T=bs.T, off_idx=bs.off_idx,
                         offsets=bad, ranges=4)
        with pytest.raises(GpdaError):                # no store is left behind
            eng.run_plain(MODE_PHOTON, n, args, 4, 1)
        hh, _ = eng.run_host(MODE_PHOTON, n, args, 4, 1, bs=bs, ranges=4)
        hp, _ = eng.run_plain(MODE_PHOTON, n, args, 4, 1)
        np.testing.assert_array_equal(hh[0], hp)


def test_run_host_tiny_store_with_empty_ranges(gpda_lib):
    """Doubling ranges over 5 bursts leave the first ranges empty."""
    bs, n, args, md, S = synth.photon_3state(B=5, seed=45)
    a1 = np.asarray(args, dtype=np.float32).reshape(1, -1)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        obs, _ = eng.run_plain(MODE_PHOTON, n, args, 3, 2)
        eng.set_observed(obs.astype(np.float32) + 1.0)
        hb, cb = eng.run_batched(MODE_PHOTON, n, a1, 7, 3)
        for ranges in (3, 8, 64):
            hh, ch = eng.run_host(MODE_PHOTON, n, a1, 7, 3, bs=bs, ranges=ranges)
            np.testing.assert_array_equal(hh, hb)
            np.testing.assert_array_equal(ch, cb)


@pytest.mark.parametrize("P", [1, 6])
def test_run_host_reports_each_store_error(gpda_lib, P):
    """The store checks of gpda_run_host (made by the kernel's CTAs for photon
    mode with few parameter sets, by validate_kernel otherwise) name the
    same errors as gpda_upload_bursts."""
    bs, n, args, md, S = synth.photon_3state(B=3000, seed=46)
    rng = np.random.default_rng(47)
    argsP = np.stack([synth.random_3state_args(rng) for _ in range(P)])
    i = int(bs.off_idx[2500]) + 5
    cases = []
    T = bs.T.copy()
    T[1700] = np.nan
    cases.append((dict(T=T), "T not finite"))
    off = bs.offsets.copy()
    off[i] = np.inf
    cases.append((dict(offsets=off), "offset not finite"))
    off = bs.offsets.copy()
    off[i], off[i + 1] = off[i + 1] + 1e-4, off[i]
    cases.append((dict(offsets=off), "not sorted"))
    with Engine(0, **md) as eng:
        for over, why in cases:
            kw = dict(N=bs.N, T=bs.T, off_idx=bs.off_idx, offsets=bs.offsets)
            kw.update(over)
            with pytest.raises(GpdaError, match=why):
                eng.run_host(MODE_PHOTON, n, argsP, 4, 1, ranges=3, **kw)
            with pytest.raises(GpdaError, match=why):
                eng.upload(**kw)
        hh, _ = eng.run_host(MODE_PHOTON, n, argsP, 4, 1, bs=bs, ranges=3)
        hb, _ = eng.run_batched(MODE_PHOTON, n, argsP, 4, 1)
        np.testing.assert_array_equal(hh, hb)
