"""Seeded synthetic burst sets with the shapes and distributions of the five
benchmark workloads, and synthetic photon streams in the reference's
HDF5-derived layout.

The reference ships no public dataset (its only fixture, tests/data/sample.hdf5,
is a Git-LFS pointer), so every workload here is generated from a seed:

  occupancy_2state  4,000 bursts, N = 30 + Geometric(mean 80), T ~ LogNormal(ln 1.5 ms, 0.5),
                    2 states E=(0.30,0.72), k12=k21=500/s, 10 samples/burst
  photon_3state     100,000 bursts, N = 30 + Geometric(mean 120), T as above, arrival offsets
                    uniform in [0,T] sorted (fp32), 3 states E=(0.2,0.5,0.85), off-diagonal
                    rates log-uniform in [50,5000]/s, 100 samples/burst
  population_256    50,000 bursts, N ~ Pareto(1.8, 30) clipped to [30,2000], T as above,
                    256 two-state parameter sets (E uniform [0.05,0.95], rates log-uniform
                    [10,1e4]/s), 50 samples/burst
  expected_hist     20,000 bursts drawn as photon_3state, 64 fixed-uniform dwell samples
  fit_4state        1,000,000 bursts, N ~ Pareto(1.8, 30) clipped to [30,3000],
                    T ~ LogNormal(ln 2 ms, 0.6), 4-state cyclic K (8 rates in [100,2e4]/s),
                    E=(0.15,0.4,0.6,0.9)

Shared model constants: background 1.5 kHz (donor) / 0.8 kHz (acceptor),
crosstalk 0.05, gamma 1, 21 bins on [0,1].
"""
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

MODEL_DEFAULTS = dict(nbins=21, left_pad=2, gamma=1.0, crosstalk=0.05, bg_d=1500.0, bg_a=800.0,
                      r0=52.0)


@dataclass
class BurstSet:
    """Bursts in the layout the engine stores in HBM."""
    N: np.ndarray                       # int32[B] photons per burst
    T: np.ndarray                       # float32[B] duration (s)
    off_idx: Optional[np.ndarray] = None  # int64[B+1] prefix offsets into offsets
    offsets: Optional[np.ndarray] = None  # float32[sum N] sorted arrival offsets (s)

    @property
    def B(self):
        return int(self.N.size)


def pack_args(E, K, V=None):
    """Parameter vector in the reference layout (src/mc.cu:792-800):
    [E(n), K off-diagonals row-major skipping the diagonal (K[i,j] = rate j->i), V(n)]."""
    E = np.asarray(E, dtype=np.float64)
    K = np.asarray(K, dtype=np.float64)
    n = E.size
    V = np.zeros(n) if V is None else np.asarray(V, dtype=np.float64)
    koff = [K[i, j] for i in range(n) for j in range(n) if i != j]
    return np.concatenate([E, np.asarray(koff), V]).astype(np.float32)


def unpack_args(args, n):
    args = np.asarray(args, dtype=np.float64)
    E = args[:n]
    koff = args[n:n * n]
    V = args[n * n:n * n + n]
    K = np.zeros((n, n))
    it = iter(koff)
    for i in range(n):
        for j in range(n):
            if i != j:
                K[i, j] = next(it)
    return E, K, V


def _lognormal_T(rng, B, median_s, sigma):
    return rng.lognormal(np.log(median_s), sigma, size=B).astype(np.float32)


def _pareto_N(rng, B, alpha, xm, hi):
    n = np.floor(xm * (1.0 + rng.pareto(alpha, size=B)))
    return np.clip(n, xm, hi).astype(np.int32)


def make_offsets(rng, N, T):
    """Sorted uniform arrival offsets in [0,T] per burst (fp32)."""
    N = np.asarray(N, dtype=np.int64)
    off_idx = np.zeros(N.size + 1, dtype=np.int64)
    np.cumsum(N, out=off_idx[1:])
    tot = int(off_idx[-1])
    bid = np.repeat(np.arange(N.size), N)
    u = rng.random(tot)
    vals = (u * np.repeat(T.astype(np.float64), N)).astype(np.float32)
    # sort within bursts: key = burst id then value
    order = np.lexsort((vals, bid))
    offsets = vals[order]
    return off_idx, offsets


def occupancy_2state(B=4000, seed=1):
    rng = np.random.default_rng(seed)
    N = (30 + rng.geometric(1.0 / 80.0, size=B)).astype(np.int32)
    T = _lognormal_T(rng, B, 1.5e-3, 0.5)
    args = pack_args([0.30, 0.72], [[0, 500.0], [500.0, 0]])
    return BurstSet(N, T), 2, args, dict(MODEL_DEFAULTS), 10


def random_3state_args(rng):
    K = np.exp(rng.uniform(np.log(50.0), np.log(5000.0), size=(3, 3)))
    np.fill_diagonal(K, 0.0)
    return pack_args([0.2, 0.5, 0.85], K)


def photon_3state(B=100000, seed=2, with_offsets=True):
    rng = np.random.default_rng(seed)
    N = (30 + rng.geometric(1.0 / 120.0, size=B)).astype(np.int32)
    T = _lognormal_T(rng, B, 1.5e-3, 0.5)
    args = random_3state_args(np.random.default_rng(seed + 1000))
    bs = BurstSet(N, T)
    if with_offsets:
        bs.off_idx, bs.offsets = make_offsets(rng, N, T)
    return bs, 3, args, dict(MODEL_DEFAULTS), 100


def expected_bursts(B=20000, n=3, seed=4):
    """Differentiable expected-histogram workload: bursts as photon_3state
    (N = 30 + Geometric(mean 120), T lognormal around 1.5 ms) without offsets,
    64 fixed-uniform dwell samples per burst; n = 2 uses occupancy_2state's
    parameters, n = 3 random_3state_args."""
    bs, _, args3, md, _ = photon_3state(B=B, seed=seed, with_offsets=False)
    if n == 2:
        args = pack_args([0.30, 0.72], np.array([[0.0, 500.0], [500.0, 0.0]]))
    elif n == 3:
        args = args3
    else:
        raise ValueError("expected_bursts: n is 2 or 3")
    return bs, n, args, md, 64


def perturb_args(args, n, dE=0.05, dlogk=0.3, seed=0):
    """A nearby parameter vector: E shifted (clipped to [0.02, 0.98]) and the
    off-diagonal rates scaled by exp(+-dlogk)."""
    rng = np.random.default_rng(seed)
    a = np.array(args, dtype=np.float64).copy()
    a[:n] = np.clip(a[:n] + rng.uniform(-dE, dE, n), 0.02, 0.98)
    a[n:n * n] = a[n:n * n] * np.exp(rng.uniform(-dlogk, dlogk, n * n - n))
    return a.astype(np.float32)


def population_args(P, seed, n=2):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(P):
        E = rng.uniform(0.05, 0.95, size=n)
        K = np.exp(rng.uniform(np.log(10.0), np.log(1e4), size=(n, n)))
        np.fill_diagonal(K, 0.0)
        out.append(pack_args(E, K))
    return np.stack(out)


def population_256(B=50000, P=256, seed=3):
    rng = np.random.default_rng(seed)
    N = _pareto_N(rng, B, 1.8, 30, 2000)
    T = _lognormal_T(rng, B, 1.5e-3, 0.5)
    return BurstSet(N, T), 2, population_args(P, seed + 1000), dict(MODEL_DEFAULTS), 50


def cyclic_4state_args(rates=None):
    if rates is None:
        rates = [400.0, 1200.0, 3000.0, 800.0, 2500.0, 6000.0, 150.0, 15000.0]
    K = np.zeros((4, 4))
    # forward ring 0->1->2->3->0 and backward ring (K[i,j] = rate j->i)
    for s in range(4):
        K[(s + 1) % 4, s] = rates[s]
        K[(s - 1) % 4, s] = rates[4 + s]
    return pack_args([0.15, 0.4, 0.6, 0.9], K)


def fit_4state(B=1000000, seed=5):
    rng = np.random.default_rng(seed)
    N = _pareto_N(rng, B, 1.8, 30, 3000)
    T = _lognormal_T(rng, B, 2e-3, 0.6)
    return BurstSet(N, T), 4, cyclic_4state_args(), dict(MODEL_DEFAULTS), 64


# ---------------------------------------------------------------- ref-compat data

def photon_stream(B=2000, seed=7, clk_p=12.5e-9, mean_n=60, p_dd=0.55, p_ad=0.35,
                  t0=3.0e9, bg_ad_rate=800.0, bg_dd_rate=1500.0):
    """Bursts in the reference's HDF5-derived layout (loadHdf5.cpp:101-128):
    per-photon int64 clock ticks masked by channel (burst_ad = mask_ad*times,
    burst_dd = mask_dd*times), start/stop ticks, istart, phCount, T (s).
    Photons that are in neither channel (acceptor-excitation) have both masks 0."""
    rng = np.random.default_rng(seed)
    ph = (2 + rng.geometric(1.0 / mean_n, size=B)).astype(np.int32)
    istart = np.zeros(B, dtype=np.int64)
    np.cumsum(ph[:-1], out=istart[1:])
    tot = int(ph.sum())
    times = np.empty(tot, dtype=np.int64)
    start = np.empty(B, dtype=np.int64)
    stop = np.empty(B, dtype=np.int64)
    t = int(t0)
    for b in range(B):
        gaps = rng.geometric(1.0 / 2000.0, size=int(ph[b]))  # ~25 us mean inter-photon gap
        tt = t + np.cumsum(gaps)
        times[istart[b]:istart[b] + ph[b]] = tt
        start[b] = tt[0]
        stop[b] = tt[-1]
        t = int(tt[-1]) + int(rng.integers(10**5, 10**7))
    ch = rng.random(tot)
    mask_dd = (ch < p_dd).astype(np.int64)
    mask_ad = ((ch >= p_dd) & (ch < p_dd + p_ad)).astype(np.int64)
    T = ((stop - start).astype(np.float64) * clk_p).astype(np.float32)
    return dict(start=start, stop=stop, istart=istart, phCount=ph,
                burst_ad=mask_ad * times, burst_dd=mask_dd * times, T=T,
                clk_p=float(np.float32(clk_p)), bg_ad_rate=float(bg_ad_rate),
                bg_dd_rate=float(bg_dd_rate), times=times, mask_ad=mask_ad, mask_dd=mask_dd)


def sgdivsr(d):
    """Observed proximity ratio per burst, A/(A+D) from the channel masks."""
    out = np.zeros(d["start"].size, dtype=np.float32)
    for b in range(out.size):
        s, n = int(d["istart"][b]), int(d["phCount"][b])
        a = int(d["mask_ad"][s:s + n].sum())
        dd = int(d["mask_dd"][s:s + n].sum())
        out[b] = a / (a + dd) if a + dd > 0 else 0.0
    return out
