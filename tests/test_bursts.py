"""gSMFRETda's HDF5 burst layout (src/loadHdf5.cpp:17-128) in .npz form:
round trip, the drop-in's arrays as burst_data builds them, the fused
engine's store and the observed histograms; on the GPU, a store built from
the layout runs bit-exact against the oracle."""
import numpy as np
import pytest

from gsmfretda_gb300 import bursts, synth


@pytest.fixture(scope="module")
def layout():
    return bursts.from_photon_stream(synth.photon_stream(B=400, seed=41))


def test_npz_round_trip(tmp_path, layout):
    p = str(tmp_path / "run.npz")
    bursts.save_npz(p, layout)
    back = bursts.load(p)
    assert set(back) == set(bursts.DATASETS)
    for k in bursts.DATASETS:
        np.testing.assert_array_equal(np.asarray(back[k]), np.asarray(layout[k]))
        assert np.asarray(back[k]).dtype == np.dtype(bursts.DATASETS[k])


def test_missing_or_inconsistent_datasets_are_rejected(tmp_path, layout):
    d = dict(layout)
    del d["mask_dd"]
    p = str(tmp_path / "bad.npz")
    np.savez(p, **d)
    with pytest.raises(KeyError):
        bursts.load(p)
    d = dict(layout)
    d["sub_bursts_l/istop"] = d["sub_bursts_l/istop"].copy()
    d["sub_bursts_l/istop"][-1] = d["times"].size
    with pytest.raises(ValueError):
        bursts.validate(d)


def test_mc_arrays_follow_burst_data(layout):
    s = synth.photon_stream(B=400, seed=41)
    a = bursts.mc_arrays(layout)
    np.testing.assert_array_equal(a["phCount"], s["phCount"])
    np.testing.assert_array_equal(a["burst_ad"], s["burst_ad"])
    np.testing.assert_array_equal(a["burst_dd"], s["burst_dd"])
    np.testing.assert_array_equal(a["istart"], s["istart"])
    assert a["sz_tag"] == s["times"].size


def test_burst_set_counts_fret_photons_and_sorted_offsets(layout):
    bs = bursts.burst_set(layout)
    ist, isp = layout["sub_bursts_l/istart"], layout["sub_bursts_l/istop"]
    for b in range(0, bs.B, 37):
        sl = slice(ist[b], isp[b] + 1)
        fret = (layout["mask_ad"][sl] != 0) | (layout["mask_dd"][sl] != 0)
        assert bs.N[b] == fret.sum()
        off = bs.offsets[bs.off_idx[b]:bs.off_idx[b + 1]]
        want = ((layout["times"][sl][fret] - layout["sub_bursts_l/start"][b]) * float(layout["clk_p"]))
        np.testing.assert_allclose(off, want.astype(np.float32), rtol=1e-6)
        assert np.all(np.diff(off) >= 0) and off.min() >= 0
    assert bs.off_idx[-1] == bs.offsets.size


def test_observed_histograms(layout):
    h = bursts.observed_counts(layout, 21)
    bs = bursts.burst_set(layout)
    assert h.sum() == (bs.N > 0).sum()
    # the reference's rule bins SgDivSr = A/(A+D) on [0,1): value 1.0 falls out
    r = bursts.observed_reference(layout, 21)
    s = layout["SgDivSr"]
    assert r.sum() == ((s >= 0) & (s < 1)).sum()


def test_hdf5_reader_needs_h5py(tmp_path):
    try:
        import h5py  # noqa: F401
    except ImportError:
        with pytest.raises(ImportError):
            bursts.load(str(tmp_path / "run.hdf5"))
        return
    layout = bursts.from_photon_stream(synth.photon_stream(B=50, seed=2))
    p = str(tmp_path / "run.hdf5")
    with h5py.File(p, "w") as f:
        for k in bursts.DATASETS:
            f[k] = np.asarray(layout[k])
    back = bursts.load(p)
    np.testing.assert_array_equal(back["times"], layout["times"])


@pytest.mark.gpu
def test_layout_store_bit_exact_on_the_gpu(orc, gpda_lib, layout):
    from gsmfretda_gb300.api import MODE_PHOTON, Engine
    bs = bursts.burst_set(layout)
    args = synth.random_3state_args(np.random.default_rng(5))
    md = synth.MODEL_DEFAULTS
    m = orc.model(**md)
    h_ref, u_ref = orc.run_pda(bs.N, bs.T, 3, args, m, 1, 16, 321, off_idx=bs.off_idx,
                               offsets=bs.offsets, unit_out=True)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(bursts.observed_counts(layout, md["nbins"]))
        units, hist = eng.run_units(MODE_PHOTON, 3, args, 16, 321)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hist, h_ref)
