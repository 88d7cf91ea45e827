"""The worker side of the parameter-server protocol: streamWorker::run
(src/streamWorker.cpp:39-246) and gpuWorker::run (src/gpuWorker.cpp:38-88).

StreamWorker.run(sid, sz_burst, left_pad) follows the reference's state
machine on one REQ socket:
  0  'c' p_cap{cap = sz_burst}                      -> p_n{s_n}
  1  'p' p_str{str = node id, histNum, ohist}        -> p_ga{idx, start, stop, bestfv, params}
     (ohist and histNum only on the first request; idx -1: ask again;
      idx -2: stop)
  2-4 the parameter set is evaluated on the GPU; while it runs, every 60th
     0.5 s wait sends a keep-alive 'k' p_sid{sid = idx} (reply ignored)
  'r' res{ridx = idx, e = chi2, idx = node id, hist = (chi2 < bestfv),
          shist = simulated histogram / R when chi2 < bestfv} -> p_sid
     (sid -1: stop), then back to state 0.

Evaluators turn (n, params, start, stop) into (chi2, simulated histogram):
  McEvaluator   the mc drop-in (mc_kernel semantics) per stream, histogram
                binned on the device, chi-square in the reference's own FP32
                formula (src/streamWorker.cpp:197-206)
  PdaEvaluator  the fused engine (histogram + FP64 chi-square on the device)
  GpuWorker     a GPU thread that evaluates the pending parameter sets of all
                streams together: one batched launch per group with the same
                state count (the reference launches one per stream)
"""
import os
import queue
import threading
import time

import numpy as np

from . import sp, wire


def chi2_reference_f32(mhist, ohist, left_pad, R, n_states):
    """The reference's reduced chi-square in its own float arithmetic
    (src/streamWorker.cpp:197-206): pow() is double, the += rounds to float."""
    nb = len(mhist)
    effN = nb - left_pad
    chisqr = np.float32(0.0)
    for i in range(left_pad, nb):
        m = np.float32(mhist[i])
        if m > 0:
            mr = np.float32(m / np.float32(R))
            d = np.float32(np.float32(ohist[i]) - mr)
            term = float(d) ** 2 / float(mr)
            chisqr = np.float32(float(chisqr) + term)
        else:
            effN -= 1
    return float(np.float32(chisqr / np.float32(effN - n_states * (n_states + 1))))


def node_id(uuid_bytes, devid, sid):
    """genuid (src/tools.cpp:157-171): <gpu uuid hex>-<pid>-<thread>-<gid>-<sid>."""
    return f"{bytes(uuid_bytes).hex()}-{os.getpid()}-{threading.get_ident()}-{devid}-{sid}"


class McEvaluator:
    """Evaluates on the `mc` drop-in, stream `sid`, the way gpuWorker::run
    drives mc (src/gpuWorker.cpp:71-81), then bins and scores as streamWorker."""

    def __init__(self, pdamc, ohist, nbins, left_pad=2):
        self.mc = pdamc
        self.ohist = np.asarray(ohist, dtype=np.float32)
        self.nbins = nbins
        self.left_pad = left_pad
        self.N = {}
        pdamc.set_hist_bins(nbins)
        self.lock = threading.Lock()

    def evaluate(self, sid, n, params, start, stop):
        with self.lock:
            m = self.mc
            old = m.set_nstates(n, sid)
            m.set_params(n, sid, params)
            N = m.setBurstBd(start, stop, sid)
            if N != self.N.get(sid):
                m.init_randstate(N, sid)
                self.N[sid] = N
            if old != n or N != self.N[sid]:
                m.set_params_buff(old, N, sid)
            m.run_kernel(N, sid)
        while not m.streamQuery(sid):
            time.sleep(0.0005)
        hist = m.hist(sid, self.nbins)
        R = m.reSampleTimes
        return chi2_reference_f32(hist, self.ohist, self.left_pad, R, n), hist / np.float32(R)


class PdaEvaluator:
    """Evaluates on the fused engine (gsmfretda_gb300.api.Engine)."""

    def __init__(self, engine, mode, samples, seed=1):
        self.eng = engine
        self.mode = mode
        self.samples = samples
        self.seed = seed
        self.calls = 0
        self.lock = threading.Lock()

    def evaluate(self, sid, n, params, start, stop):
        with self.lock:
            self.calls += 1
            b1 = self.eng.B if (stop < 0 or stop >= self.eng.B) else stop
            b0 = 0 if (start < 0 or start >= b1) else start
            hist, chi2 = self.eng.run_plain(self.mode, n, params, self.samples,
                                            self.seed + 7919 * self.calls, b0, b1)
        return chi2, hist.astype(np.float32) / np.float32(self.samples)


class GpuWorker:
    """GPU thread shared by all streams: waits for pending requests, runs all
    that share a state count in one batched launch, and hands each stream its
    chi-square and histogram."""

    def __init__(self, engine, mode, samples, seed=1, max_batch=256, linger_s=0.002, record=False):
        self.eng = engine
        self.history = [] if record else None     # (seed, n, args) of every launch
        self.mode = mode
        self.samples = samples
        self.seed = seed
        self.max_batch = max_batch
        self.linger_s = linger_s
        self.q = queue.Queue()
        self.launches = 0
        self._stop = threading.Event()
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    def evaluate(self, sid, n, params, start, stop):
        done = threading.Event()
        slot = {}
        self.q.put((n, np.asarray(params, dtype=np.float32), done, slot))
        done.wait()
        if "error" in slot:
            raise slot["error"]
        return slot["chi2"], slot["hist"]

    def _loop(self):
        while not self._stop.is_set():
            try:
                first = self.q.get(timeout=0.1)
            except queue.Empty:
                continue
            batch = [first]
            t_end = time.monotonic() + self.linger_s
            while len(batch) < self.max_batch:
                try:
                    batch.append(self.q.get(timeout=max(0.0, t_end - time.monotonic())))
                except queue.Empty:
                    break
            groups = {}
            for item in batch:
                groups.setdefault(item[0], []).append(item)
            for n, items in groups.items():
                try:
                    args = np.stack([it[1] for it in items])
                    self.launches += 1
                    seed = self.seed + 104729 * self.launches
                    if self.history is not None:
                        self.history.append((seed, n, args))
                    hist, chi2 = self.eng.run_batched(self.mode, n, args, self.samples, seed)
                    for i, it in enumerate(items):
                        it[3]["chi2"] = float(chi2[i])
                        it[3]["hist"] = hist[i].astype(np.float32) / np.float32(self.samples)
                except Exception as e:  # noqa: BLE001 - handed to the waiting stream
                    for it in items:
                        it[3]["error"] = e
                for it in items:
                    it[2].set()

    def close(self):
        self._stop.set()
        self.thread.join(timeout=2)


class StreamWorker:
    def __init__(self, url, evaluator, ohist, fret_hist_num, uuid_bytes=b"\x00" * 16, devid=0,
                 wait_s=0.5, keepalive_every=60, reconnect_ivl=0.2, request_timeout=None,
                 resend_s=60.0):
        self.url = url
        self.evaluator = evaluator
        self.ohist = list(np.asarray(ohist, dtype=np.float32))
        self.fret_hist_num = fret_hist_num
        self.uuid = uuid_bytes
        self.devid = devid
        self.wait_s = wait_s
        self.keepalive_every = keepalive_every
        self.reconnect_ivl = reconnect_ivl
        self.request_timeout = request_timeout
        self.resend_s = resend_s
        self.evaluated = 0
        self.keepalives = 0

    def run(self, sid, sz_burst, left_pad=2):
        sock = sp.ReqSocket(self.url, reconnect_ivl=self.reconnect_ivl, resend_s=self.resend_s)
        nid = node_id(self.uuid, self.devid, sid)
        sent_ohist = False
        try:
            while True:
                # state 0
                rep = sock.request(wire.request("c", {"cap": sz_burst}), self.request_timeout)
                s_n = wire.decode("p_n", rep)["s_n"]
                # state 1
                while True:
                    p = {"str": nid}
                    if not sent_ohist:
                        p["histNum"] = self.fret_hist_num
                        p["ohist"] = self.ohist
                        sent_ohist = True
                    ga = wire.decode("p_ga", sock.request(wire.request("p", p), self.request_timeout))
                    if ga["idx"] == -1:
                        continue
                    break
                if ga["idx"] == -2:
                    return "quit"
                idx = ga["idx"]
                params = np.asarray(ga["params"][:s_n * (s_n + 1)], dtype=np.float32)
                # states 2-4: evaluate, with keep-alives while the GPU works
                result = {}

                def work():
                    try:
                        result["v"] = self.evaluator.evaluate(sid, s_n, params, ga["start"], ga["stop"])
                    except Exception as e:  # noqa: BLE001 - reported below
                        result["e"] = e

                th = threading.Thread(target=work, daemon=True)
                th.start()
                waits = 0
                while th.is_alive():
                    th.join(self.wait_s)
                    if th.is_alive():
                        waits += 1
                        if waits % self.keepalive_every == 0:
                            sock.request(wire.request("k", {"sid": idx}), self.request_timeout)
                            self.keepalives += 1
                if "e" in result:
                    raise result["e"]
                chi2, shist = result["v"]
                self.evaluated += 1
                send_hist = chi2 < ga["bestfv"]
                res = {"ridx": idx, "e": float(chi2), "idx": nid, "hist": bool(send_hist)}
                if send_hist:
                    res["shist"] = [float(x) for x in shist]
                gas = wire.decode("p_sid", sock.request(wire.request("r", res), self.request_timeout))
                if gas["sid"] == -1:
                    return "end"
        finally:
            sock.close()
