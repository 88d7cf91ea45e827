"""Generate the golden fixtures in tests/golden/.

ref_binomial.npz — histograms of the REFERENCE's own binomial sampler
    (src/binom.cuh rk_binomial, compiled for the host by oracle/build_ref.py
    from the reference tree) over a grid of (n, p): the reference test grid
    (tests/gen_rand_tests.cpp:79-93: n in 3..6, p in {0.41, 0.54, 1/2.1,
    1/3.3}) plus the kernel's operating range (inversion and BTPE/BTRD
    regimes, p on both sides of 1/2). 200,000 draws per point, fixed seeds.
    These pin the oracle's binomial sampler against the reference's.

oracle_small.npz — per-unit outputs of the oracle on three small seeded cases
    (occupancy, photon, ref-compat), a regression pin for the oracle itself.

Run (where the reference tree is mounted):  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

BINOM_GRID = ([(n, p) for n in (3, 4, 5, 6) for p in (0.41, 0.54, 1 / 2.1, 1 / 3.3)] +
              [(30, 0.2), (60, 0.3), (150, 0.18), (150, 0.85), (400, 0.5), (1000, 0.07),
               (2000, 0.9), (3000, 0.25), (45, 0.95), (12, 0.02)])
DRAWS = 200_000


def ref_binomial_hists():
    import build_ref
    lib = C.CDLL(build_ref.build())
    lib.ref_binomial_many.argtypes = [C.c_ulonglong, C.c_int, C.c_double, C.c_long, C.c_void_p]
    hists = []
    for i, (n, p) in enumerate(BINOM_GRID):
        out = np.zeros(DRAWS, dtype=np.int64)
        lib.ref_binomial_many(1000003 + 7919 * i, n, float(np.float32(p)), DRAWS, out.ctypes.data)
        hists.append(np.bincount(out, minlength=n + 1).astype(np.int64))
    grid = np.array(BINOM_GRID, dtype=np.float64)
    maxlen = max(h.size for h in hists)
    H = np.zeros((len(hists), maxlen), dtype=np.int64)
    for i, h in enumerate(hists):
        H[i, :h.size] = h
    return grid, H


def oracle_small():
    import build_oracle
    build_oracle.build()
    import orc

    from gsmfretda_gb300 import synth
    out = {}
    bs, n, args, md, S = synth.occupancy_2state(B=200, seed=101)
    m = orc.model(**md)
    _, u = orc.run_pda(bs.N, bs.T, n, args, m, 0, S, 2718, unit_out=True)
    out["occ_units"] = u
    bs, n, args, md, S = synth.photon_3state(B=200, seed=102)
    _, u = orc.run_pda(bs.N, bs.T, n, args, m, 1, 8, 3141, off_idx=bs.off_idx, offsets=bs.offsets,
                       unit_out=True)
    out["pho_units"] = u
    d = synth.photon_stream(B=100, seed=103)
    args3 = synth.random_3state_args(np.random.default_rng(104))
    _, e = orc.run_refcompat(d, 3, args3, m, 4, 1618)
    out["rc_mcE"] = e
    return out


if __name__ == "__main__":
    grid, H = ref_binomial_hists()
    np.savez_compressed(os.path.join(HERE, "ref_binomial.npz"), grid=grid, hist=H, draws=DRAWS)
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **oracle_small())
    print("wrote", os.listdir(HERE))
