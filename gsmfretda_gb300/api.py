"""Python host API over the C ABI: a burst store in HBM plus fused
Monte-Carlo PDA runs (histogram + reduced chi-square on the device).

    eng = Engine(device=0, nbins=21)
    eng.upload(burst_set)                       # gsmfretda_gb300.synth.BurstSet
    eng.set_observed(ohist)
    hist, chi2 = eng.run_plain(MODE_PHOTON, n, args, samples=100, seed=1)
    hist, chi2 = eng.run_batched(MODE_OCCUPANCY, n, args_P, samples=50, seed=1)
"""
import ctypes as C

import numpy as np

from ._lib import (GPDA_OK, MODE_OCCUPANCY, MODE_PHOTON, GpdaError, default_model, load)

__all__ = ["Engine", "MODE_OCCUPANCY", "MODE_PHOTON", "build_params", "bin_values"]


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _check(rc, ctx=None):
    if rc != GPDA_OK:
        msg = ""
        if ctx:
            msg = (load().gpda_last_error(ctx) or b"").decode()
        raise GpdaError(rc, msg)
    return rc


def build_params(n, args, **model_kw):
    """Per-parameter-set device tables (host derivation; no GPU needed)."""
    lib = load()
    m = default_model(**model_kw)
    a = np.ascontiguousarray(args, dtype=np.float32)
    out = np.zeros(lib.gpda_params_size(), dtype=np.float32)
    _check(lib.gpda_build_params(C.byref(m), n, _p(a), _p(out)))
    return out


def bin_values(x, nbins):
    """The reference's histogram rule (Boost regular axis on [0,1), inner bins)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    h = np.zeros(nbins, dtype=np.float32)
    _check(load().gpda_bin_values(_p(x), x.size, nbins, _p(h)))
    return h


class Engine:
    def __init__(self, device=0, **model_kw):
        self.lib = load()
        self.model = default_model(**model_kw)
        st = C.c_int32(0)
        self.ctx = self.lib.gpda_create(device, C.byref(self.model), C.byref(st))
        if not self.ctx:
            raise GpdaError(st.value, f"gpda_create(device={device})")
        self.nbins = self.model.nbins
        self.B = 0
        self._keep = None

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.gpda_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- data
    def upload(self, bs=None, N=None, T=None, off_idx=None, offsets=None):
        if bs is not None:
            N, T, off_idx, offsets = bs.N, bs.T, bs.off_idx, bs.offsets
        N = np.ascontiguousarray(N, dtype=np.int32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        oi = None if off_idx is None else np.ascontiguousarray(off_idx, dtype=np.int64)
        of = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.float32)
        _check(self.lib.gpda_upload_bursts(self.ctx, _p(N), _p(T), _p(oi), _p(of), N.size), self.ctx)
        self.B = N.size

    def set_observed(self, ohist):
        o = np.ascontiguousarray(ohist, dtype=np.float32)
        _check(self.lib.gpda_set_observed(self.ctx, _p(o), o.size), self.ctx)

    # ---------------------------------------------------------------- runs
    def run_plain(self, mode, n, args, samples, seed, b0=0, b1=None):
        b1 = self.B if b1 is None else b1
        a = np.ascontiguousarray(args, dtype=np.float32)
        hist = np.zeros(self.nbins, dtype=np.uint64)
        chi2 = np.zeros(1, dtype=np.float64)
        _check(self.lib.gpda_run_plain(self.ctx, mode, n, _p(a), b0, b1, samples, seed,
                                       _p(hist), _p(chi2)), self.ctx)
        return hist, float(chi2[0])

    def run_batched(self, mode, n, args, samples, seed):
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        P = a.size // (n * (n + 1))
        hist = np.zeros((P, self.nbins), dtype=np.uint64)
        chi2 = np.zeros(P, dtype=np.float64)
        _check(self.lib.gpda_run_batched(self.ctx, mode, P, n, _p(a), samples, seed,
                                         _p(hist), _p(chi2)), self.ctx)
        return hist, chi2

    def run_units(self, mode, n, args, samples, seed, b0=0, b1=None):
        b1 = self.B if b1 is None else b1
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        P = a.size // (n * (n + 1))
        units = np.zeros((P, b1 - b0, samples), dtype=np.int32)
        hist = np.zeros((P, self.nbins), dtype=np.uint64)
        _check(self.lib.gpda_run_units(self.ctx, mode, P, n, _p(a), b0, b1, samples, seed,
                                       _p(units), _p(hist)), self.ctx)
        return units, hist

    def run_host(self, mode, n, args, samples, seed, bs=None, N=None, T=None, off_idx=None,
                 offsets=None, ranges=4):
        """Upload the bursts and run all parameter sets in one call, the copy
        overlapped with the simulation (ranges of bursts); the store stays
        uploaded. Returns hist (P, nbins) and chi2 (P,)."""
        if bs is not None:
            N, T, off_idx, offsets = bs.N, bs.T, bs.off_idx, bs.offsets
        N = np.ascontiguousarray(N, dtype=np.int32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        oi = None if off_idx is None else np.ascontiguousarray(off_idx, dtype=np.int64)
        of = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.float32)
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        P = a.size // (n * (n + 1))
        hist = np.zeros((P, self.nbins), dtype=np.uint64)
        chi2 = np.zeros(P, dtype=np.float64)
        rc = self.lib.gpda_run_host(self.ctx, mode, P, n, _p(a), _p(N), _p(T), _p(oi), _p(of), N.size,
                                    samples, seed, ranges, _p(hist), _p(chi2))
        self.B = N.size if rc == GPDA_OK else 0
        _check(rc, self.ctx)
        return hist, chi2

    # ---------------------------------------------------------------- captured launch
    def graph_create(self, mode, n, P, samples):
        """Capture one batched step (P parameter sets) as a CUDA graph."""
        _check(self.lib.gpda_graph_create(self.ctx, mode, P, n, samples), self.ctx)
        self._graph = (n, P)

    def graph_run(self, args, seed):
        n, P = self._graph
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        if a.size != P * n * (n + 1):
            raise ValueError("args must hold the captured number of parameter sets")
        hist = np.zeros((P, self.nbins), dtype=np.uint64)
        chi2 = np.zeros(P, dtype=np.float64)
        _check(self.lib.gpda_graph_run(self.ctx, _p(a), seed, _p(hist), _p(chi2)), self.ctx)
        return hist, chi2

    def autotune(self, mode, n, args, samples, seed=1):
        """Pick the fastest bursts-per-work-item for this launch shape; returns it."""
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        P = a.size // (n * (n + 1))
        t = C.c_int32(0)
        _check(self.lib.gpda_autotune(self.ctx, mode, P, n, _p(a), samples, seed, C.byref(t)), self.ctx)
        return t.value

    # ---------------------------------------------------------------- expected histogram
    def _exp_args(self, n, args, anchor):
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        P = a.size // (n * (n + 1))
        an = None if anchor is None else np.ascontiguousarray(anchor, dtype=np.float32).reshape(-1)
        if an is not None and an.size != a.size:
            raise ValueError("anchor must have the shape of args")
        return a, an, P

    def expected_hist(self, n, args, samples, seed, anchor=None):
        """Differentiable expected-histogram form (occupancy model, V = 0):
        expected counts (P, nbins) summed over samples and chi2 (P,)."""
        a, an, P = self._exp_args(n, args, anchor)
        hist = np.zeros((P, self.nbins), dtype=np.float64)
        chi2 = np.zeros(P, dtype=np.float64)
        _check(self.lib.gpda_expected_hist(self.ctx, P, n, _p(a), _p(an), samples, seed,
                                           _p(hist), _p(chi2)), self.ctx)
        return hist, chi2

    def expected_adjoint(self, n, args, samples, seed, anchor=None, dchi2=None):
        """Gradient of sum(dchi2 * chi2) in E (P, n) and ln K (P, n(n-1))."""
        a, an, P = self._exp_args(n, args, anchor)
        up = None if dchi2 is None else np.ascontiguousarray(dchi2, dtype=np.float64).reshape(P)
        dE = np.zeros((P, n), dtype=np.float64)
        dK = np.zeros((P, n * (n - 1)), dtype=np.float64)
        _check(self.lib.gpda_expected_hist_adjoint(self.ctx, P, n, _p(a), _p(an), samples, seed,
                                                   _p(up), _p(dE), _p(dK)), self.ctx)
        return dE, dK

    def expected_tape_limit(self, nbytes):
        """Device bytes the forward may keep for the adjoint (0: recompute)."""
        _check(self.lib.gpda_expected_set_tape_limit(self.ctx, int(nbytes)), self.ctx)

    def expected_grad(self, n, args, samples, seed, anchor=None):
        """Forward and gradient in one call: hist, chi2, dE, dlnK."""
        a, an, P = self._exp_args(n, args, anchor)
        hist = np.zeros((P, self.nbins), dtype=np.float64)
        chi2 = np.zeros(P, dtype=np.float64)
        dE = np.zeros((P, n), dtype=np.float64)
        dK = np.zeros((P, n * (n - 1)), dtype=np.float64)
        _check(self.lib.gpda_expected_grad(self.ctx, P, n, _p(a), _p(an), samples, seed, _p(hist),
                                           _p(chi2), _p(dE), _p(dK)), self.ctx)
        return hist, chi2, dE, dK

    def launch(self, mode, n, args, samples, seed, b0=0, b1=None):
        """Asynchronous: returns after the launch is queued on the context stream."""
        b1 = self.B if b1 is None else b1
        a = np.ascontiguousarray(args, dtype=np.float32).reshape(-1)
        self._keep = a
        P = a.size // (n * (n + 1))
        _check(self.lib.gpda_launch(self.ctx, mode, P, n, _p(a), b0, b1, samples, seed), self.ctx)
        return P

    def fetch(self, P):
        hist = np.zeros((P, self.nbins), dtype=np.uint64)
        chi2 = np.zeros(P, dtype=np.float64)
        _check(self.lib.gpda_fetch(self.ctx, _p(hist), _p(chi2)), self.ctx)
        return hist, chi2

    def query(self):
        rc = self.lib.gpda_query(self.ctx)
        if rc < 0:
            _check(rc, self.ctx)
        return rc == 1

    def synchronize(self):
        _check(self.lib.gpda_synchronize(self.ctx), self.ctx)

    @property
    def stream_handle(self):
        return self.lib.gpda_stream(self.ctx)

    @property
    def launch_count(self):
        return int(self.lib.gpda_launch_count(self.ctx))

    def limit_hits(self):
        return int(self.lib.gpda_limit_hits(self.ctx))
