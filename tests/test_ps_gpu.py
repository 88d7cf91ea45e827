"""The parameter-server protocol end to end on the GPU: chi-square values and
histograms that reach the server through the wire equal those of direct
engine calls with the same seeds (and, for the mc drop-in, the oracle's)."""
import threading

import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300.api import MODE_OCCUPANCY, Engine
from gsmfretda_gb300.ps import server as psrv
from gsmfretda_gb300.ps import worker as pw

pytestmark = pytest.mark.gpu


def _start(srv, evaluator, ohist, nworkers=1, sz_burst=1000):
    ths = []
    for i in range(nworkers):
        w = pw.StreamWorker(srv.url, evaluator, ohist, len(ohist))
        t = threading.Thread(target=w.run, args=(i, sz_burst), daemon=True)
        t.start()
        ths.append(t)
    return ths


def _stop(srv, ths):
    srv.finish()
    for t in ths:
        t.join(timeout=60)
        assert not t.is_alive()
    srv.close()


def _sets(n, k, seed):
    return [synth.population_args(1, seed + i).reshape(-1)[: n * (n + 1)] for i in range(k)]


def test_pda_evaluator_over_the_wire(gpda_lib):
    bs, n, args, md, S = synth.occupancy_2state(B=3000, seed=31)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        ohist, _ = eng.run_plain(MODE_OCCUPANCY, n, args, 1, 5)
        ohist = ohist.astype(np.float32)
        eng.set_observed(ohist)
        sets = _sets(n, 4, 40)
        srv = psrv.ParamServer(n)
        ths = _start(srv, pw.PdaEvaluator(eng, MODE_OCCUPANCY, S, seed=10), ohist)
        idxs = srv.submit(sets)
        got = srv.wait(idxs, timeout=120)
        _stop(srv, ths)
        best = np.inf
        for k, (i, p) in enumerate(zip(idxs, sets), start=1):
            hist, chi2 = eng.run_plain(MODE_OCCUPANCY, n, p, S, 10 + 7919 * k)
            assert np.float32(got[k - 1]) == np.float32(chi2)
            r = srv.results[i]
            if chi2 < best:
                np.testing.assert_array_equal(r["shist"], hist.astype(np.float32) / np.float32(S))
                best = np.float32(chi2)
            else:
                assert r["shist"] is None
        np.testing.assert_array_equal(srv.observed, ohist)


def test_gpu_worker_batches_streams(gpda_lib):
    bs, n, args, md, S = synth.occupancy_2state(B=3000, seed=32)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        ohist, _ = eng.run_plain(MODE_OCCUPANCY, n, args, 1, 6)
        eng.set_observed(ohist.astype(np.float32))
        gw = pw.GpuWorker(eng, MODE_OCCUPANCY, S, seed=3, linger_s=0.02, record=True)
        srv = psrv.ParamServer(n)
        ths = _start(srv, gw, ohist.astype(np.float32), nworkers=4)
        sets = _sets(n, 12, 70)
        idxs = srv.submit(sets)
        got = dict(zip(idxs, srv.wait(idxs, timeout=120)))
        _stop(srv, ths)
        gw.close()
        # replay every recorded launch; each row's chi-square is the one a
        # worker reported for that parameter set
        by_params = {tuple(np.float32(p)): i for i, p in zip(idxs, sets)}
        seen = set()
        for seed, nn, a in gw.history:
            _, chi2 = eng.run_batched(MODE_OCCUPANCY, nn, a, S, seed)
            for row, c in zip(a, chi2):
                i = by_params[tuple(np.float32(row))]
                assert np.float32(got[i]) == np.float32(c)
                seen.add(i)
        assert seen == set(idxs)
        assert gw.launches < len(sets)          # streams shared launches


def test_mc_evaluator_over_the_wire(orc, gpda_lib):
    from gsmfretda_gb300.mc import mc
    d = synth.photon_stream(B=1200, seed=33)
    n, nbins, seed = 3, 40, 500
    args = synth.random_3state_args(np.random.default_rng(34))
    m = orc.model(**synth.MODEL_DEFAULTS)
    m.nbins = nbins
    pdamc = mc(0, 2)
    try:
        pdamc.set_seed(seed)
        pdamc.init_data_gpu(d["istart"], d["start"], d["stop"], d["phCount"], d["times"].size,
                            d["burst_ad"], d["burst_dd"], d["T"], synth.sgdivsr(d), d["clk_p"],
                            d["bg_ad_rate"], d["bg_dd_rate"])
        R = pdamc.reSampleTimes
        h_obs, _ = orc.run_refcompat(d, n, args, m, 1, 99, want_mcE=False)
        ohist = h_obs.astype(np.float32)
        srv = psrv.ParamServer(n)
        ev = pw.McEvaluator(pdamc, ohist, nbins)
        ths = _start(srv, ev, ohist)
        (chi,) = srv.evaluate([args], timeout=120)
        res = srv.results[0]
        _stop(srv, ths)
    finally:
        pdamc.close()
    h_ref, _ = orc.run_refcompat(d, n, args, m, R, seed + 0, want_mcE=False)
    want = pw.chi2_reference_f32(h_ref.astype(np.float32), ohist, 2, R, n)
    assert np.float32(chi) == np.float32(want)
    np.testing.assert_array_equal(res["shist"], h_ref.astype(np.float32) / np.float32(R))
