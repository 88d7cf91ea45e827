"""Burst data in gSMFRETda's HDF5 layout (src/loadHdf5.cpp:17-128), and its
conversion to the two device stores.

Datasets, under the names loadhdf5 reads:
  sub_bursts_l/start, sub_bursts_l/stop     int64[B]  first / last photon clock tick
  sub_bursts_l/istart, sub_bursts_l/istop   int64[B]  first / last photon index (inclusive)
  times                                     int64[M]  photon clock ticks
  mask_ad, mask_dd                          uint8[M]  acceptor / donor detection channel
  T_burst_duration                          float32[B] burst duration (s)
  SgDivSr                                   float32[B] observed proximity ratio per burst
  clk_p, bg_ad_rate, bg_dd_rate             float32 scalars

libhdf5 is not needed: `load` reads the same datasets from an .npz archive
with the same names (and an HDF5 file through h5py where that is installed);
`save_npz` writes one.

  d = bursts.load("run.npz")
  mc.init_data_gpu(**bursts.mc_arrays(d))          # the drop-in (burst_data's arrays)
  engine.upload(bursts.burst_set(d))               # the fused engine (N, T, offsets)
  engine.set_observed(bursts.observed_counts(d, 21))
"""
import numpy as np

from .synth import BurstSet

__all__ = ["DATASETS", "load", "save_npz", "validate", "from_photon_stream", "mc_arrays",
           "burst_set", "observed_counts", "observed_reference"]

DATASETS = {
    "sub_bursts_l/start": np.int64, "sub_bursts_l/stop": np.int64,
    "sub_bursts_l/istart": np.int64, "sub_bursts_l/istop": np.int64,
    "times": np.int64, "mask_ad": np.uint8, "mask_dd": np.uint8,
    "T_burst_duration": np.float32, "SgDivSr": np.float32,
    "clk_p": np.float32, "bg_ad_rate": np.float32, "bg_dd_rate": np.float32,
}
_SCALARS = ("clk_p", "bg_ad_rate", "bg_dd_rate")


def _coerce(raw):
    d = {}
    for k, t in DATASETS.items():
        if k not in raw:
            raise KeyError(f"dataset {k} missing")
        a = np.asarray(raw[k])
        d[k] = t(a.reshape(-1)[0]) if k in _SCALARS else np.ascontiguousarray(a, dtype=t).reshape(-1)
    validate(d)
    return d


def load(path):
    """The datasets of one file, as numpy arrays (scalars as numpy floats)."""
    if str(path).endswith(".npz"):
        with np.load(path) as z:
            return _coerce({k: z[k] for k in z.files})
    try:
        import h5py
    except ImportError as e:
        raise ImportError("reading HDF5 needs h5py; convert the file to .npz with the same "
                          "dataset names instead") from e
    with h5py.File(path, "r") as f:
        return _coerce({k: f[k][()] for k in DATASETS})


def save_npz(path, d):
    np.savez(path, **{k: np.asarray(d[k]) for k in DATASETS})


def validate(d):
    B = d["sub_bursts_l/start"].size
    M = d["times"].size
    for k in ("sub_bursts_l/stop", "sub_bursts_l/istart", "sub_bursts_l/istop", "T_burst_duration",
              "SgDivSr"):
        if d[k].size != B:
            raise ValueError(f"{k} has {d[k].size} entries, expected {B}")
    for k in ("mask_ad", "mask_dd"):
        if d[k].size != M:
            raise ValueError(f"{k} has {d[k].size} entries, expected {M}")
    ist, isp = d["sub_bursts_l/istart"], d["sub_bursts_l/istop"]
    if B and (ist.min() < 0 or isp.max() >= M or np.any(isp < ist - 1)):
        raise ValueError("istart/istop out of range")
    if not (d["clk_p"] > 0):
        raise ValueError("clk_p must be positive")


def from_photon_stream(s):
    """The layout of a synth.photon_stream data set (SgDivSr from the masks)."""
    from .synth import sgdivsr
    ist = np.asarray(s["istart"], dtype=np.int64)
    return _coerce({
        "sub_bursts_l/start": s["start"], "sub_bursts_l/stop": s["stop"],
        "sub_bursts_l/istart": ist, "sub_bursts_l/istop": ist + np.asarray(s["phCount"]) - 1,
        "times": s["times"], "mask_ad": s["mask_ad"], "mask_dd": s["mask_dd"],
        "T_burst_duration": s["T"], "SgDivSr": sgdivsr(s),
        "clk_p": s["clk_p"], "bg_ad_rate": s["bg_ad_rate"], "bg_dd_rate": s["bg_dd_rate"],
    })


def mc_arrays(d):
    """Keyword arguments of mc.init_data_gpu as burst_data builds them
    (src/loadHdf5.cpp:101-128): phCount = istop - istart + 1, per-photon
    masked ticks burst_ad = mask_ad * times and burst_dd = mask_dd * times."""
    ist = d["sub_bursts_l/istart"]
    ph = (d["sub_bursts_l/istop"] - ist + 1).astype(np.int32)
    t = d["times"]
    return dict(istart=ist, start=d["sub_bursts_l/start"], stop=d["sub_bursts_l/stop"],
                phCount=ph, sz_tag=t.size, burst_ad=d["mask_ad"].astype(np.int64) * t,
                burst_dd=d["mask_dd"].astype(np.int64) * t, T_burst_duration=d["T_burst_duration"],
                SgDivSr=d["SgDivSr"], clk_p=float(d["clk_p"]), bg_ad_rate=float(d["bg_ad_rate"]),
                bg_dd_rate=float(d["bg_dd_rate"]))


def _counted(d):
    """Per burst: the indices of its photons that are in the donor or the
    acceptor channel (the photons the FRET model splits)."""
    ist, isp = d["sub_bursts_l/istart"], d["sub_bursts_l/istop"]
    fret = (d["mask_ad"] != 0) | (d["mask_dd"] != 0)
    M = d["times"].size
    # a photon belongs to burst b when istart[b] <= i <= istop[b]
    owner = np.full(M, -1, dtype=np.int64)
    lengths = np.maximum(isp - ist + 1, 0)
    if lengths.sum():
        bids = np.repeat(np.arange(ist.size), lengths)
        first = np.repeat(np.cumsum(lengths) - lengths, lengths)
        owner[np.arange(bids.size) - first + np.repeat(ist, lengths)] = bids
    keep = fret & (owner >= 0)
    return owner, keep


def burst_set(d):
    """The fused engine's store: N = donor + acceptor photons per burst, T =
    T_burst_duration, and each counted photon's arrival offset
    (times - start) * clk_p (s), sorted within its burst."""
    B = d["sub_bursts_l/start"].size
    owner, keep = _counted(d)
    idx = np.nonzero(keep)[0]
    ob = owner[idx]
    order = np.lexsort((d["times"][idx], ob))      # by burst, then by time
    idx, ob = idx[order], ob[order]
    N = np.bincount(ob, minlength=B).astype(np.int32)
    off_idx = np.zeros(B + 1, dtype=np.int64)
    np.cumsum(N, out=off_idx[1:])
    rel = (d["times"][idx] - d["sub_bursts_l/start"][ob]).astype(np.float64) * float(d["clk_p"])
    offsets = np.maximum(rel, 0.0).astype(np.float32)
    bs = BurstSet(N, np.ascontiguousarray(d["T_burst_duration"], dtype=np.float32))
    bs.off_idx, bs.offsets = off_idx, offsets
    return bs


def observed_counts(d, nbins):
    """Observed histogram under the fused engine's binning: acceptor photons A
    of the N counted ones, bin = min(A * nbins / N, nbins - 1); bursts with
    N = 0 are not counted."""
    B = d["sub_bursts_l/start"].size
    owner, keep = _counted(d)
    N = np.bincount(owner[keep], minlength=B)
    A = np.bincount(owner[keep & (d["mask_ad"] != 0)], minlength=B)
    ok = N > 0
    b = np.minimum(A[ok] * nbins // N[ok], nbins - 1)
    return np.bincount(b, minlength=nbins).astype(np.float32)


def observed_reference(d, nbins):
    """The reference's observed histogram: mkhist of SgDivSr on a regular axis
    over [0, 1), inner bins only (src/streamWorker.cpp:33-38, 62-67)."""
    from .api import bin_values
    return bin_values(d["SgDivSr"], nbins)
