"""gpda_run_host over page-locked host arrays in photon mode with one
parameter set: the kernel reads the caller's arrays itself (each CTA stages
its tile from host memory and writes it through to the device store). The
results equal the oracle and uploading first; the store ends up uploaded;
tiles too large for shared memory, a photon total that is not a multiple of
four, empty bursts and every store error behave as on the copy path."""
import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300._lib import GpdaError
from gsmfretda_gb300.api import MODE_PHOTON, Engine

pytestmark = pytest.mark.gpu


def _pinned(x, dtype):
    import torch
    x = np.ascontiguousarray(x, dtype=dtype)
    t = torch.empty(x.shape, dtype=getattr(torch, np.dtype(dtype).name), pin_memory=True)
    t.numpy()[...] = x
    return t.numpy(), t          # keep the tensor alive with the view


def _pinned_store(bs):
    keep = []
    out = {}
    for k, dt in (("N", np.int32), ("T", np.float32), ("off_idx", np.int64), ("offsets", np.float32)):
        a, t = _pinned(getattr(bs, k), dt)
        out[k] = a
        keep.append(t)
    return out, keep


def _odd_store(seed):
    """Bursts of the photon workload plus a few of 9,000-10,000 photons (their
    tiles exceed the 8,192-float staging), empty bursts, and a photon total
    that is not a multiple of four."""
    bs, n, args, md, S = synth.photon_3state(B=700, seed=seed)
    rng = np.random.default_rng(seed + 1)
    N = bs.N.copy()
    T = bs.T.copy()
    N[[13, 350]] = [9001, 9999]
    T[[13, 350]] = [4e-3, 5e-3]
    N[[5, 6, 600]] = 0
    if int(N.sum()) % 4 == 0:
        N[7] += 1
    big = synth.BurstSet(N, T)
    big.off_idx, big.offsets = synth.make_offsets(rng, N, T)
    assert int(big.off_idx[-1]) % 4 != 0
    return big, n, args, md


def test_direct_reads_equal_the_oracle_and_upload_first(gpda_lib, orc):
    bs, n, args, md = _odd_store(51)
    S = 6
    a1 = np.asarray(args, dtype=np.float32).reshape(1, -1)
    m = orc.model(**md)
    h_ref, _ = orc.run_pda(bs.N, bs.T, n, args, m, MODE_PHOTON, S, 99, off_idx=bs.off_idx,
                           offsets=bs.offsets)
    host, keep = _pinned_store(bs)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        obs, _ = eng.run_plain(MODE_PHOTON, n, args, 1, 3)
        eng.set_observed(obs.astype(np.float32))
        hb, cb = eng.run_batched(MODE_PHOTON, n, a1, S, 99)
        np.testing.assert_array_equal(hb, h_ref)
    with Engine(0, **md) as eng:
        eng.set_observed(obs.astype(np.float32))
        l0 = eng.launch_count
        hh, ch = eng.run_host(MODE_PHOTON, n, a1, S, 99, ranges=3, **host)
        # one binomial-table launch and one Monte-Carlo launch: no range kernels
        assert eng.launch_count - l0 == 2
        np.testing.assert_array_equal(hh, h_ref)
        np.testing.assert_array_equal(ch, cb)
        # the kernel wrote the store through: resident runs see the same bursts
        h2, c2 = eng.run_batched(MODE_PHOTON, n, a1, S, 99)
        np.testing.assert_array_equal(h2, h_ref)
        units, hu = eng.run_units(MODE_PHOTON, n, args, S, 123)
    h_u, u_ref = orc.run_pda(bs.N, bs.T, n, args, m, MODE_PHOTON, S, 123, off_idx=bs.off_idx,
                             offsets=bs.offsets, unit_out=True)
    np.testing.assert_array_equal(units, u_ref)
    np.testing.assert_array_equal(hu, h_u)
    del keep


def test_direct_reads_replace_a_larger_store(gpda_lib):
    """Two calls in a row, the second with fewer bursts: the second result
    equals a fresh upload of its own store."""
    big, n, args, md, S = synth.photon_3state(B=3000, seed=52)
    small, _, _, _, _ = synth.photon_3state(B=900, seed=53)
    a1 = np.asarray(args, dtype=np.float32).reshape(1, -1)
    hb_big, hb_small = None, None
    with Engine(0, **md) as eng:
        eng.upload(big)
        hb_big, _ = eng.run_batched(MODE_PHOTON, n, a1, 8, 5)
        eng.upload(small)
        hb_small, _ = eng.run_batched(MODE_PHOTON, n, a1, 8, 5)
    hbig, k1 = _pinned_store(big)
    hsmall, k2 = _pinned_store(small)
    with Engine(0, **md) as eng:
        hh, _ = eng.run_host(MODE_PHOTON, n, a1, 8, 5, **hbig)
        np.testing.assert_array_equal(hh, hb_big)
        hh, _ = eng.run_host(MODE_PHOTON, n, a1, 8, 5, **hsmall)
        np.testing.assert_array_equal(hh, hb_small)
        h2, _ = eng.run_batched(MODE_PHOTON, n, a1, 8, 5)
        np.testing.assert_array_equal(h2, hb_small)
    del k1, k2


def test_direct_reads_report_each_store_error(gpda_lib):
    bs, n, args, md, S = synth.photon_3state(B=3000, seed=54)
    a1 = np.asarray(args, dtype=np.float32).reshape(1, -1)
    i = int(bs.off_idx[2500]) + 5
    cases = []
    T = bs.T.copy()
    T[1700] = np.nan
    cases.append(("T", T, "T not finite"))
    N = bs.N.copy()
    N[10] += 1
    cases.append(("N", N, "off_idx inconsistent"))
    off = bs.offsets.copy()
    off[i] = np.inf
    cases.append(("offsets", off, "offset not finite"))
    off = bs.offsets.copy()
    off[i], off[i + 1] = off[i + 1] + 1e-4, off[i]
    cases.append(("offsets", off, "not sorted"))
    with Engine(0, **md) as eng:
        for key, bad, why in cases:
            host, keep = _pinned_store(bs)
            host[key][...] = bad
            l0 = eng.launch_count
            with pytest.raises(GpdaError, match=why):
                eng.run_host(MODE_PHOTON, n, a1, 4, 1, **host)
            assert eng.launch_count - l0 == 2          # the direct path made the check
            with pytest.raises(GpdaError):             # no store is left behind
                eng.run_plain(MODE_PHOTON, n, args, 4, 1)
            del keep
        host, keep = _pinned_store(bs)
        hh, _ = eng.run_host(MODE_PHOTON, n, a1, 4, 1, **host)
        hp, _ = eng.run_plain(MODE_PHOTON, n, args, 4, 1)
        np.testing.assert_array_equal(hh[0], hp)
        del keep
