"""gpda_run_pda_noalloc, the entry point for callers that cannot allocate
device memory where they evaluate parameter sets: through the C ABI, its
histograms and chi-square on caller-owned device buffers must equal those of
the context-based entry point (gpda_run_batched) on the same inputs and
seeds, bit for bit, on two calls in a row (the second call reuses the
library's fixed scratch left by the first)."""
import ctypes as C

import numpy as np
import pytest


@pytest.mark.gpu
def test_noalloc_matches_batched_on_two_calls(gpda_lib):
    import torch

    from gsmfretda_gb300 import synth
    from gsmfretda_gb300._lib import GPDA_OK, default_model
    from gsmfretda_gb300.api import MODE_PHOTON, Engine

    bs, n, args1, md, _ = synth.photon_3state(B=3000, seed=71)
    S = 16
    P = 2                       # photon mode: P * n_states <= 8 binomial tables
    rng = np.random.default_rng(72)
    params = np.concatenate([synth.random_3state_args(rng) for _ in range(P)]).astype(np.float32)
    nb = md["nbins"]
    ohist = np.zeros(nb, dtype=np.float32)
    ohist[3:18] = np.linspace(5, 60, 15, dtype=np.float32)

    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        want = [eng.run_batched(MODE_PHOTON, n, params, S, seed) for seed in (101, 202)]

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    dN = torch.from_numpy(bs.N).to(dev)
    dT = torch.from_numpy(bs.T).to(dev)
    dOI = torch.from_numpy(bs.off_idx).to(dev)
    # padded like the engine's store so a tile's 16-byte span can be read whole
    dOF = torch.zeros(bs.offsets.size + 8, dtype=torch.float32, device=dev)
    dOF[:bs.offsets.size] = torch.from_numpy(bs.offsets).to(dev)
    dObs = torch.from_numpy(ohist).to(dev)
    m = default_model(**md)
    stream = torch.cuda.current_stream(dev)
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for (h_want, c_want), seed in zip(want, (101, 202)):
        dHist = torch.full((P, nb), -1, dtype=torch.int64, device=dev)   # stale contents
        dChi = torch.zeros(P, dtype=torch.float64, device=dev)
        rc = gpda_lib.gpda_run_pda_noalloc(C.byref(m), MODE_PHOTON, P, n,
                                           params.ctypes.data_as(C.c_void_p), vp(dN), vp(dT),
                                           vp(dOI), vp(dOF), bs.B, S, seed, vp(dHist), vp(dObs),
                                           vp(dChi), C.c_void_p(stream.cuda_stream))
        assert rc == GPDA_OK
        torch.cuda.synchronize(dev)
        got = dHist.cpu().numpy().view(np.uint64)
        np.testing.assert_array_equal(got, h_want)
        np.testing.assert_array_equal(dChi.cpu().numpy(), c_want)


def test_noalloc_rejects_more_parameter_sets_than_its_scratch_holds(gpda_lib):
    # argument checks run before any CUDA call, so this needs no GPU
    from gsmfretda_gb300._lib import GPDA_OK, default_model
    m = default_model()
    params = np.zeros(65 * 6, dtype=np.float32)
    rc = gpda_lib.gpda_run_pda_noalloc(C.byref(m), 0, 65, 2, params.ctypes.data_as(C.c_void_p),
                                       C.c_void_p(1), C.c_void_p(1), None, None, 10, 4, 1,
                                       C.c_void_p(1), None, None, None)
    assert rc != GPDA_OK
