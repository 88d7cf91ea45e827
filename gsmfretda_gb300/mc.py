"""Python mirror of the reference's `mc` engine object (src/mc.hpp:32-180)
over the gpda_mc_* C ABI: same member names, argument meaning and call
sequence as gpuWorker::run (src/gpuWorker.cpp:69-82).

    pdamc = mc(0, 2)                                  # mc::mc (src/mc.cu:212)
    pdamc.init_data_gpu(istart, start, stop, phCount, sz_tag, burst_ad,
                        burst_dd, T_burst_duration, SgDivSr, clk_p,
                        bg_ad_rate, bg_dd_rate)        # mc.cu:456
    old = pdamc.set_nstates(n, sid)                   # mc.cu:723
    pdamc.set_params(n, sid, args)                    # mc.cu:790
    N = pdamc.setBurstBd(start, stop, sid)            # mc.cu:523
    pdamc.init_randstate(N, sid)                      # mc.cu:366
    pdamc.set_params_buff(old, N, sid)                # mc.cu:783
    pdamc.run_kernel(N, sid)                          # mc.cu:567
    while not pdamc.streamQuery(sid): ...             # mc.cu:595
    values = pdamc.hmcE(sid)[:N * pdamc.reSampleTimes]
"""
import ctypes as C

import numpy as np

from ._lib import GPDA_OK, GpdaError, load

__all__ = ["mc"]


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class mc:  # noqa: N801  (the reference's class name)
    def __init__(self, devid=0, streamNum=16, debug=0, hdf5size=0, profiler=False):
        self.lib = load()
        st = C.c_int32(0)
        self.h = self.lib.gpda_mc_create(devid, streamNum, debug, hdf5size, int(profiler), C.byref(st))
        if not self.h:
            raise GpdaError(st.value, f"gpda_mc_create(devid={devid})")
        self.devid = devid
        self.streamNum = self.lib.gpda_mc_stream_num(self.h)
        self.s_n = [0] * self.streamNum
        self._keep = []

    def _check(self, rc):
        if rc < 0:
            raise GpdaError(rc, (self.lib.gpda_mc_last_error(self.h) or b"").decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.gpda_mc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def reSampleTimes(self):  # noqa: N802
        return self.lib.gpda_mc_resample_times(self.h)

    def set_reSampleTimes(self, t):  # noqa: N802
        self._check(self.lib.gpda_mc_set_resample_times(self.h, t))

    @property
    def sz_burst(self):
        return self.lib.gpda_mc_sz_burst(self.h)

    def getStreams(self):  # noqa: N802
        return self.streamNum

    def set_seed(self, seed):
        self._check(self.lib.gpda_mc_set_seed(self.h, seed))

    def set_hist_bins(self, nbins):
        self._check(self.lib.gpda_mc_set_hist_bins(self.h, nbins))

    def set_gpuid(self):
        """mc::set_gpuid: the C ABI sets the device on every call."""

    def init_data_gpu(self, istart, start, stop, phCount, sz_tag, burst_ad, burst_dd,
                      T_burst_duration, SgDivSr, clk_p, bg_ad_rate, bg_dd_rate):
        arrs = [np.ascontiguousarray(istart, dtype=np.int64), np.ascontiguousarray(start, dtype=np.int64),
                np.ascontiguousarray(stop, dtype=np.int64), np.ascontiguousarray(phCount, dtype=np.int32),
                np.ascontiguousarray(burst_ad, dtype=np.int64), np.ascontiguousarray(burst_dd, dtype=np.int64),
                np.ascontiguousarray(T_burst_duration, dtype=np.float32),
                None if SgDivSr is None else np.ascontiguousarray(SgDivSr, dtype=np.float32)]
        ist, sta, sto, ph, bad, bdd, T, sg = arrs
        self._check(self.lib.gpda_mc_init_data_gpu(self.h, _p(ist), _p(sta), _p(sto), _p(ph), ph.size,
                                                   int(sz_tag), _p(bad), _p(bdd), _p(T), _p(sg),
                                                   clk_p, bg_ad_rate, bg_dd_rate))

    def set_nstates(self, n, sid):
        r = self._check(self.lib.gpda_mc_set_nstates(self.h, n, sid))
        self.s_n[sid] = n
        return r

    def set_params(self, n, sid, args):
        a = np.ascontiguousarray(args, dtype=np.float32)
        return bool(self._check(self.lib.gpda_mc_set_params(self.h, n, sid, _p(a), a.size)))

    def setBurstBd(self, cstart, cstop, sid):  # noqa: N802
        return self._check(self.lib.gpda_mc_setBurstBd(self.h, cstart, cstop, sid))

    def init_randstate(self, N, sid):
        self._check(self.lib.gpda_mc_init_randstate(self.h, N, sid))

    def set_params_buff(self, oldS_n, N_sid, sid):  # noqa: N803
        self._check(self.lib.gpda_mc_set_params_buff(self.h, oldS_n, N_sid, sid))

    def run_kernel(self, N, sid):
        self._check(self.lib.gpda_mc_run_kernel(self.h, N, sid))
        self._lastN = getattr(self, "_lastN", {})
        self._lastN[sid] = N

    def streamQuery(self, sid):  # noqa: N802
        return self._check(self.lib.gpda_mc_streamQuery(self.h, sid)) == 1

    def hmcE(self, sid):  # noqa: N802
        """View of the pinned result buffer of stream sid (valid after streamQuery)."""
        ptr = self.lib.gpda_mc_hmcE(self.h, sid)
        n = self._lastN.get(sid, 0) * self.reSampleTimes
        if not ptr or n == 0:
            return np.zeros(0, dtype=np.float32)
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

    def hist(self, sid, nbins):
        out = np.zeros(nbins, dtype=np.float32)
        self._check(self.lib.gpda_mc_hist(self.h, sid, _p(out)))
        return out
