"""ctypes binding of the CPU oracle (oracle/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, always as the checker, never as the product.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAXS = 8


class OrcModel(C.Structure):
    _fields_ = [("nbins", C.c_int32), ("left_pad", C.c_int32), ("gamma", C.c_float),
                ("crosstalk", C.c_float), ("bg_d", C.c_float), ("bg_a", C.c_float),
                ("r0", C.c_float), ("rc_gamma", C.c_float), ("rc_de", C.c_float),
                ("rc_ct", C.c_float), ("rc_r0", C.c_float)]


class OrcParams(C.Structure):
    _fields_ = [("n", C.c_int32), ("pad_", C.c_int32 * 3),
                ("E", C.c_float * MAXS), ("V", C.c_float * MAXS), ("eps", C.c_float * MAXS),
                ("kexit", C.c_float * MAXS), ("inv_kexit", C.c_float * MAXS),
                ("init_cdf", C.c_float * MAXS), ("jump_cdf", C.c_float * (MAXS * MAXS)),
                ("K", C.c_float * (MAXS * MAXS)), ("Pi2j", C.c_float * (MAXS * MAXS)),
                ("pinit", C.c_float * MAXS)]


class OrcBursts(C.Structure):
    _fields_ = [("B", C.c_int64), ("N", C.c_void_p), ("T", C.c_void_p),
                ("off_idx", C.c_void_p), ("offsets", C.c_void_p)]


class OrcRcBursts(C.Structure):
    _fields_ = [("B", C.c_int64), ("start", C.c_void_p), ("stop", C.c_void_p),
                ("istart", C.c_void_p), ("phCount", C.c_void_p), ("burst_ad", C.c_void_p),
                ("burst_dd", C.c_void_p), ("T", C.c_void_p), ("clk_p", C.c_float),
                ("bg_ad_rate", C.c_float), ("bg_dd_rate", C.c_float)]


class OrcReplayStats(C.Structure):
    _fields_ = [("units", C.c_int64), ("exact", C.c_int64), ("differs", C.c_int64),
                ("truncated", C.c_int64), ("off_path", C.c_int64), ("lambda_mismatch", C.c_int64),
                ("binom_arg_mismatch", C.c_int64), ("tau_max_ulp", C.c_int64),
                ("e_max_abs", C.c_double)]


# one draw record of the tape format (orc_tape_rec): kind | n << 8, integer, double
TAPE_DTYPE = np.dtype([("tag", np.int32), ("i", np.int32), ("d", np.float64)])
TAPE_U, TAPE_TAU, TAPE_N, TAPE_E, TAPE_P, TAPE_B = 1, 2, 3, 4, 5, 6

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            from . import build_oracle  # noqa: F401  (only when imported as a package)
        _lib = C.CDLL(path)
        _lib.orc_logf.restype = C.c_float
        _lib.orc_logf.argtypes = [C.c_float]
        _lib.orc_expf.restype = C.c_float
        _lib.orc_expf.argtypes = [C.c_float]
        _lib.orc_cos2pif.restype = C.c_float
        _lib.orc_cos2pif.argtypes = [C.c_float]
        _lib.orc_chi2.restype = C.c_double
        _lib.orc_chi2.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        _lib.orc_chi2_f32.restype = C.c_float
        _lib.orc_chi2_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        _lib.orc_sample.argtypes = [C.c_int, C.c_uint64, C.c_int32, C.c_float, C.c_int64, C.c_void_p]
        _lib.orc_sample_cat.argtypes = [C.c_uint64, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                        C.c_int64, C.c_void_p]
        _lib.orc_binom_cdf_row.argtypes = [C.c_float, C.c_int32, C.c_void_p]
        _lib.orc_build_params.argtypes = [C.c_int32, C.c_void_p, C.POINTER(OrcModel), C.POINTER(OrcParams)]
        _lib.orc_run_pda.argtypes = [C.POINTER(OrcBursts), C.c_int32, C.c_void_p, C.c_int32,
                                     C.POINTER(OrcModel), C.c_int32, C.c_int32, C.c_uint64,
                                     C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
        _lib.orc_run_refcompat.argtypes = [C.POINTER(OrcRcBursts), C.c_int32, C.c_void_p,
                                           C.POINTER(OrcModel), C.c_int32, C.c_uint64, C.c_int64,
                                           C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
        _lib.orc_expected.argtypes = [C.POINTER(OrcBursts), C.c_int32, C.c_void_p, C.c_void_p,
                                      C.c_int32, C.POINTER(OrcModel), C.c_int32, C.c_uint64,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_int32]
        _lib.orc_bin_values.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]
        _lib.orc_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_sample_bgpair.argtypes = [C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_int64,
                                           C.c_void_p, C.c_void_p]
        _lib.orc_rc_replay.argtypes = [C.POINTER(OrcRcBursts), C.c_int32, C.c_void_p,
                                       C.POINTER(OrcModel), C.c_int32, C.c_void_p, C.c_void_p,
                                       C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(OrcReplayStats)]
        _lib.orc_rc_record.argtypes = [C.POINTER(OrcRcBursts), C.c_int32, C.c_void_p,
                                       C.POINTER(OrcModel), C.c_int32, C.c_uint64, C.c_int32,
                                       C.c_void_p, C.c_void_p, C.c_void_p]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def model(nbins=21, left_pad=2, gamma=1.0, crosstalk=0.05, bg_d=1500.0, bg_a=800.0, r0=52.0,
          rc_gamma=0.34, rc_de=0.08, rc_ct=0.07, rc_r0=52.0):
    return OrcModel(nbins, left_pad, gamma, crosstalk, bg_d, bg_a, r0, rc_gamma, rc_de, rc_ct, rc_r0)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def sample(kind, seed, n, p, count):
    """kind: binomial, poisson, exponential, normal, u01, binomial64, poisson64"""
    kinds = {"binomial": 0, "poisson": 1, "exponential": 2, "normal": 3, "u01": 4,
             "binomial64": 5, "poisson64": 6}
    out = np.zeros(count, dtype=np.float64)
    rc = lib().orc_sample(kinds[kind], seed, n, p, count, _ptr(out))
    if rc != 0:
        raise ValueError(rc)
    return out


def sample_cat(seed, mode, w, count, frm=0, n=None):
    w = np.ascontiguousarray(w, dtype=np.float32).reshape(-1)
    n = w.size if n is None else n
    out = np.zeros(count, dtype=np.int32)
    rc = lib().orc_sample_cat(seed, mode, n, _ptr(w), frm, count, _ptr(out))
    if rc != 0:
        raise ValueError(rc)
    return out


def binom_cdf_row(pp, nn):
    out = np.zeros(nn + 1, dtype=np.float32)
    lib().orc_binom_cdf_row(pp, nn, _ptr(out))
    return out


def build_params(n, args, m):
    a = np.ascontiguousarray(args, dtype=np.float32)
    out = OrcParams()
    rc = lib().orc_build_params(n, _ptr(a), C.byref(m), C.byref(out))
    if rc != 0:
        raise ValueError(f"orc_build_params rc={rc}")
    return out


def run_pda(N, T, n, args, m, mode, S, seed, b0=0, b1=None, off_idx=None, offsets=None,
            unit_out=False, nthreads=0, f64=False):
    N = np.ascontiguousarray(N, dtype=np.int32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    args = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
    P = args.size // (n * (n + 1))
    if b1 is None:
        b1 = N.size
    oi = None if off_idx is None else np.ascontiguousarray(off_idx, dtype=np.int64)
    of = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.float32)
    bs = OrcBursts(N.size, _ptr(N), _ptr(T), _ptr(oi), _ptr(of))
    hist = np.zeros((P, m.nbins), dtype=np.uint64)
    uo = np.zeros((P, b1 - b0, S), dtype=np.int32) if unit_out else None
    rc = lib().orc_run_pda(C.byref(bs), n, _ptr(args), P, C.byref(m), mode, S, seed, b0, b1,
                           _ptr(hist), _ptr(uo), nthreads, 1 if f64 else 0)
    if rc != 0:
        raise ValueError(f"orc_run_pda rc={rc}")
    return hist, uo


def run_refcompat(rc_data, n, args, m, S, seed, b0=0, b1=None, want_mcE=True, nthreads=0, f64=False):
    d = rc_data
    B = d["start"].size
    if b1 is None:
        b1 = B
    arrs = {k: np.ascontiguousarray(d[k], dtype=t) for k, t in
            [("start", np.int64), ("stop", np.int64), ("istart", np.int64), ("phCount", np.int32),
             ("burst_ad", np.int64), ("burst_dd", np.int64), ("T", np.float32)]}
    bs = OrcRcBursts(B, _ptr(arrs["start"]), _ptr(arrs["stop"]), _ptr(arrs["istart"]),
                     _ptr(arrs["phCount"]), _ptr(arrs["burst_ad"]), _ptr(arrs["burst_dd"]),
                     _ptr(arrs["T"]), d["clk_p"], d["bg_ad_rate"], d["bg_dd_rate"])
    a = np.ascontiguousarray(args, dtype=np.float32)
    hist = np.zeros(m.nbins, dtype=np.uint64)
    mcE = np.zeros((b1 - b0, S), dtype=np.float32) if want_mcE else None
    rc = lib().orc_run_refcompat(C.byref(bs), n, _ptr(a), C.byref(m), S, seed, b0, b1,
                                 _ptr(hist), _ptr(mcE), nthreads, 1 if f64 else 0)
    if rc != 0:
        raise ValueError(f"orc_run_refcompat rc={rc}")
    return hist, mcE


def sample_bgpair(seed, bg_a, bg_d, dt, count):
    """(A, D) variates of the photon-mode background pair, unclipped."""
    A = np.zeros(count, dtype=np.int32)
    D = np.zeros(count, dtype=np.int32)
    rc = lib().orc_sample_bgpair(seed, bg_a, bg_d, dt, count, _ptr(A), _ptr(D))
    if rc != 0:
        raise ValueError(f"orc_sample_bgpair rc={rc}")
    return A, D


def _rc_bursts(d):
    arrs = {k: np.ascontiguousarray(d[k], dtype=t) for k, t in
            [("start", np.int64), ("stop", np.int64), ("istart", np.int64), ("phCount", np.int32),
             ("burst_ad", np.int64), ("burst_dd", np.int64), ("T", np.float32)]}
    bs = OrcRcBursts(arrs["start"].size, _ptr(arrs["start"]), _ptr(arrs["stop"]), _ptr(arrs["istart"]),
                     _ptr(arrs["phCount"]), _ptr(arrs["burst_ad"]), _ptr(arrs["burst_dd"]),
                     _ptr(arrs["T"]), d["clk_p"], d["bg_ad_rate"], d["bg_dd_rate"])
    return bs, arrs


def rc_record(rc_data, n, args, m, R, seed, cap):
    """The oracle's own Philox draws of every mc_kernel unit, in the tape
    format: (tape[B*R, cap], tape_len[B*R], mcE[B*R])."""
    bs, keep = _rc_bursts(rc_data)
    units = bs.B * R
    tape = np.zeros((units, cap), dtype=TAPE_DTYPE)
    tlen = np.zeros(units, dtype=np.int32)
    mcE = np.zeros(units, dtype=np.float32)
    a = np.ascontiguousarray(args, dtype=np.float32)
    rc = lib().orc_rc_record(C.byref(bs), n, _ptr(a), C.byref(m), R, seed, cap, _ptr(tape),
                             _ptr(tlen), _ptr(mcE))
    if rc != 0:
        raise ValueError(f"orc_rc_record rc={rc}")
    return tape, tlen, mcE


def rc_replay(rc_data, n, args, m, R, tape, tape_len, ref_mcE):
    """Replays recorded draws through the oracle's mc_kernel body. Returns
    (mcE, status per unit, stats dict); status 0 = bit-exact with ref_mcE,
    1 = differs, 2 = tape cut, 3 = draws out of order."""
    bs, keep = _rc_bursts(rc_data)
    units = bs.B * R
    tape = np.ascontiguousarray(tape, dtype=TAPE_DTYPE).reshape(units, -1)
    tl = np.ascontiguousarray(tape_len, dtype=np.int32)
    ref = np.ascontiguousarray(ref_mcE, dtype=np.float32).reshape(-1)
    out = np.zeros(units, dtype=np.float32)
    status = np.zeros(units, dtype=np.int8)
    st = OrcReplayStats()
    a = np.ascontiguousarray(args, dtype=np.float32)
    rc = lib().orc_rc_replay(C.byref(bs), n, _ptr(a), C.byref(m), R, _ptr(tape), _ptr(tl),
                             tape.shape[1], _ptr(ref), _ptr(out), _ptr(status), C.byref(st))
    if rc != 0:
        raise ValueError(f"orc_rc_replay rc={rc}")
    stats = {f: getattr(st, f) for f, _ in OrcReplayStats._fields_}
    return out, status, stats


def chi2(hist, ohist, nbins, left_pad, S, n_states):
    h = np.ascontiguousarray(hist, dtype=np.uint64)
    o = np.ascontiguousarray(ohist, dtype=np.float32)
    return lib().orc_chi2(_ptr(h), _ptr(o), nbins, left_pad, S, n_states)


def chi2_f32(mhist, ohist, nbins, left_pad, R, n_states):
    h = np.ascontiguousarray(mhist, dtype=np.float32)
    o = np.ascontiguousarray(ohist, dtype=np.float32)
    return lib().orc_chi2_f32(_ptr(h), _ptr(o), nbins, left_pad, R, n_states)


def bin_values(x, nbins):
    x = np.ascontiguousarray(x, dtype=np.float32)
    h = np.zeros(nbins, dtype=np.float32)
    lib().orc_bin_values(_ptr(x), x.size, nbins, _ptr(h))
    return h


def expected(N, T, n, args, m, S, seed, obs, anchor=None, grad=True, nthreads=0):
    """FP64 expected-histogram forward (+ gradient): hist (P, nbins), chi2 (P,),
    dE (P, n), dlnK (P, n(n-1)); the state skeleton is drawn under anchor."""
    N = np.ascontiguousarray(N, dtype=np.int32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
    P = a.size // (n * (n + 1))
    an = None if anchor is None else np.ascontiguousarray(anchor, dtype=np.float32).reshape(-1)
    o = np.ascontiguousarray(obs, dtype=np.float32)
    bs = OrcBursts(N.size, _ptr(N), _ptr(T), None, None)
    hist = np.zeros((P, m.nbins), dtype=np.float64)
    chi2 = np.zeros(P, dtype=np.float64)
    dE = np.zeros((P, n), dtype=np.float64) if grad else None
    dK = np.zeros((P, n * (n - 1)), dtype=np.float64) if grad else None
    rc = lib().orc_expected(C.byref(bs), n, _ptr(a), _ptr(an), P, C.byref(m), S, seed, _ptr(o),
                            _ptr(hist), _ptr(chi2), _ptr(dE), _ptr(dK), nthreads)
    if rc != 0:
        raise ValueError(f"orc_expected rc={rc}")
    return hist, chi2, dE, dK
