"""ctypes binding of the reference-kernel harness (oracle/_ref/libmcref.so,
built by oracle/build_mcref.py from the reference's own mc_kernel,
gen_rand.cuh and binom.cuh).

TEST INFRASTRUCTURE ONLY: the reference's kernel, run as the reference runs it,
so that the oracle (and through it the GPU path) can be compared with the
reference's own output.
"""
import ctypes as C
import os

import numpy as np

import orc

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def load(path=None):
    """Builds the harness where its extracted sources exist and loads it
    (path: another build of it); raises FileNotFoundError where they do not."""
    global _lib
    if _lib is None:
        import build_mcref
        path = path or build_mcref.build()
        lib = C.CDLL(path)
        vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
        lib.mcref_run.restype = C.c_int
        lib.mcref_run.argtypes = [vp, vp, vp, vp, i64, vp, vp, i64, vp, f32, f32, f32, i32,
                                  vp, vp, vp, vp, vp, i32, i32, vp, vp, vp, i32, vp]
        lib.mcref_shift.restype = C.c_int
        lib.mcref_shift.argtypes = [i32]
        _lib = lib
    return _lib


def tables(n, args, m):
    """(gpe, gpv, gpk, gpp_i2j, gpp) as mc::set_params builds them (genMatK,
    genP_i2j, genMatP, src/eigenhelper.cpp:4-53), from the oracle's
    restatement."""
    p = orc.build_params(n, args, m)
    return (np.array(p.E[:n], dtype=np.float32), np.array(p.V[:n], dtype=np.float32),
            np.array(p.K[:n * n], dtype=np.float32), np.array(p.Pi2j[:n * n], dtype=np.float32),
            np.array(p.pinit[:n], dtype=np.float32))


def shift(R):
    """The thread-to-burst shift mc_kernel computes on this device for
    reSampleTimes = R, (int)log2((double)R) (src/mc.cu:101)."""
    return load().mcref_shift(R)


def run(d, n, args, m, R, tape_cap=0, debug=False):
    """mc_kernel with reSampleTimes = R (a power of two) over all bursts of
    the reference-layout burst data d, launched so that its threads map onto
    exactly these bursts (see mcref_shift). Returns (mcE[B*Reff], tape, tape
    lengths, Reff): Reff = 2^shift samples per burst, the values
    (burst, sample)-major; with tape_cap, the per-thread draw tapes
    (orc.TAPE_DTYPE[B*Reff, tape_cap])."""
    lib = load()
    arr = {k: np.ascontiguousarray(d[k], dtype=t) for k, t in
           [("start", np.int64), ("stop", np.int64), ("istart", np.int64), ("phCount", np.int32),
            ("burst_ad", np.int64), ("burst_dd", np.int64), ("T", np.float32)]}
    B = arr["start"].size
    gpe, gpv, gpk, gpij, gpp = tables(n, args, m)
    reff = 1 << shift(R)
    units = B * reff
    mcE = np.zeros(units, dtype=np.float32)
    tape = np.zeros((units, max(tape_cap, 1)), dtype=orc.TAPE_DTYPE) if tape_cap else None
    tlen = np.zeros(units, dtype=np.int32) if tape_cap else None
    p = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    r_eff = C.c_int32(0)
    rc = lib.mcref_run(p(arr["start"]), p(arr["stop"]), p(arr["istart"]), p(arr["phCount"]), B,
                       p(arr["burst_ad"]), p(arr["burst_dd"]), arr["burst_ad"].size, p(arr["T"]),
                       d["clk_p"], d["bg_ad_rate"], d["bg_dd_rate"], n, p(gpe), p(gpv), p(gpk),
                       p(gpij), p(gpp), R, tape_cap, p(mcE), p(tape), p(tlen), 1 if debug else 0,
                       C.byref(r_eff))
    if rc != 0:
        raise RuntimeError(f"mcref_run rc={rc}")
    assert r_eff.value == reff
    return mcE, tape, tlen, reff
