"""gpda_run_pda_noalloc, the entry point for callers that cannot allocate
device memory where they evaluate parameter sets (a framework whose caching
allocator owns the device, or a loop that must not pay cudaMalloc's implicit
synchronisation): through the C ABI, its histograms and chi-square on
caller-owned device buffers must equal those of the context-based entry point
(gpda_run_batched) on the same inputs and seeds, bit for bit, on two calls in
a row (the second call reuses the library's fixed scratch left by the first).

The caller's offsets buffer is exactly off_idx[B] floats long (no padding),
and the photon-mode cases include the scratch limits (P * n_states = 8
binomial tables) next to the occupancy limit (P = 64).
"""
import ctypes as C

import numpy as np
import pytest

from gsmfretda_gb300._lib import GPDA_OK


def _cases():
    # (mode, P, n_states, bursts, samples, label)
    return [(1, 2, 3, 3000, 16, "photon"),
            (1, 2, 4, 2000, 8, "photon-limit"),        # 8 (set, state) tables
            (0, 8, 2, 3000, 16, "occupancy"),
            (0, 64, 2, 1500, 4, "occupancy-limit")]    # 64 parameter sets


def _params(rng, P, n):
    from gsmfretda_gb300 import synth
    if n == 3:
        return np.concatenate([synth.random_3state_args(rng) for _ in range(P)]).astype(np.float32)
    if n == 4:
        out = []
        for _ in range(P):
            a = synth.cyclic_4state_args().copy()
            a[:4] = rng.uniform(0.1, 0.9, 4)
            out.append(a)
        return np.concatenate(out).astype(np.float32)
    return synth.population_args(P, seed=int(rng.integers(1 << 30)), n=n).reshape(-1).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,P,n,B,S,label", _cases(), ids=[c[-1] for c in _cases()])
def test_noalloc_matches_batched_on_two_calls(gpda_lib, mode, P, n, B, S, label):
    import torch

    from gsmfretda_gb300 import synth
    from gsmfretda_gb300._lib import default_model
    from gsmfretda_gb300.api import Engine

    bs, _, _, md, _ = synth.photon_3state(B=B, seed=71)
    rng = np.random.default_rng(72 + P + n)
    params = _params(rng, P, n)
    nb = md["nbins"]
    ohist = np.zeros(nb, dtype=np.float32)
    ohist[3:18] = np.linspace(5, 60, 15, dtype=np.float32)
    seeds = (101, 202)

    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(ohist)
        want = [eng.run_batched(mode, n, params, S, seed) for seed in seeds]

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    dN = torch.from_numpy(bs.N).to(dev)
    dT = torch.from_numpy(bs.T).to(dev)
    dOI = torch.from_numpy(bs.off_idx).to(dev)
    dOF = torch.from_numpy(bs.offsets).to(dev)           # exactly sum(N) floats
    assert dOF.numel() == int(bs.off_idx[-1]) and dOF.data_ptr() % 16 == 0
    dObs = torch.from_numpy(ohist).to(dev)
    m = default_model(**md)
    stream = torch.cuda.Stream(dev)                       # not the default stream
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for (h_want, c_want), seed in zip(want, seeds):
        with torch.cuda.stream(stream):
            dHist = torch.full((P, nb), -1, dtype=torch.int64, device=dev)   # stale contents
            dChi = torch.zeros(P, dtype=torch.float64, device=dev)
        rc = gpda_lib.gpda_run_pda_noalloc(C.byref(m), mode, P, n,
                                           params.ctypes.data_as(C.c_void_p), vp(dN), vp(dT),
                                           vp(dOI), vp(dOF), bs.B, S, seed, vp(dHist), vp(dObs),
                                           vp(dChi), C.c_void_p(stream.cuda_stream))
        assert rc == GPDA_OK
        stream.synchronize()
        got = dHist.cpu().numpy().view(np.uint64)
        np.testing.assert_array_equal(got, h_want)
        np.testing.assert_array_equal(dChi.cpu().numpy(), c_want)


def test_noalloc_rejects_more_parameter_sets_than_its_scratch_holds(gpda_lib):
    # argument checks run before any CUDA call, so this needs no GPU
    from gsmfretda_gb300._lib import default_model
    m = default_model()
    params = np.zeros(65 * 6, dtype=np.float32)
    rc = gpda_lib.gpda_run_pda_noalloc(C.byref(m), 0, 65, 2, params.ctypes.data_as(C.c_void_p),
                                       C.c_void_p(256), C.c_void_p(256), None, None, 10, 4, 1,
                                       C.c_void_p(256), None, None, None)
    assert rc != GPDA_OK
    params = np.zeros(3 * 12, dtype=np.float32)          # photon: 3 sets x 3 states > 8 tables
    rc = gpda_lib.gpda_run_pda_noalloc(C.byref(m), 1, 3, 3, params.ctypes.data_as(C.c_void_p),
                                       C.c_void_p(256), C.c_void_p(256), C.c_void_p(256),
                                       C.c_void_p(256), 10, 4, 1, C.c_void_p(256), None, None, None)
    assert rc != GPDA_OK


def test_noalloc_rejects_misaligned_offsets(gpda_lib):
    # the photon staging reads offsets as 16-byte vectors; checked on the host
    from gsmfretda_gb300._lib import default_model
    m = default_model()
    params = np.zeros(12, dtype=np.float32)
    rc = gpda_lib.gpda_run_pda_noalloc(C.byref(m), 1, 1, 3, params.ctypes.data_as(C.c_void_p),
                                       C.c_void_p(256), C.c_void_p(256), C.c_void_p(256),
                                       C.c_void_p(256 + 4), 10, 4, 1, C.c_void_p(256), None, None,
                                       None)
    assert rc != GPDA_OK
