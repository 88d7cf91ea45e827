"""A parameter server speaking the reference's protocol (the server side of
src/streamWorker.cpp:39-246; the reference's own server lives in the separate
pySMFRETda project). Workers ask for parameter sets and return chi-square
values; an optimiser submits parameter sets and waits for their results.

  'c' p_cap  -> p_n{s_n}
  'p' p_str  -> p_ga{idx, start, stop, bestfv, params}; idx -1 when nothing is
                pending (the worker asks again), idx -2 once finished
  'k' p_sid  -> p_sid{sid}                         (keep-alive)
  'r' res    -> p_sid{sid}: 0 to continue, -1 once finished

The first 'p' of a worker carries the observed histogram (histNum > 0); it is
kept in `observed`. bestfv is the best chi-square seen so far, so workers send
their simulated histogram only when they improve on it.

Requests are idempotent under resends (a REQ socket sends a request again when
its reply is lost): a worker that asks with 'p' while it still holds a
parameter set it has not returned gets that same set again, and a repeated 'r'
overwrites its own result.

With `lease_s` set, a parameter set whose worker has sent nothing about it
(no keep-alive 'k', no result) for lease_s seconds goes back to the queue for
another worker; a late result from the first worker is still accepted.
"""
import threading
import time

import numpy as np

from . import sp, wire


class ParamServer:
    def __init__(self, n_states, url="tcp://127.0.0.1:0", start=0, stop=-1, lease_s=None):
        self.n = n_states
        self.lease_s = lease_s
        self.heard = {}               # idx -> time of the last word about it
        self.start = start
        self.stop = stop
        self.lock = threading.Condition()
        self.pending = []             # (idx, params)
        self.results = {}             # idx -> dict(e, shist, node)
        self.observed = None
        self.bestfv = 3.1e32          # the reference worker's initial value
        self.best_params = None
        self.finished = False
        self.next_idx = 0
        self.params_of = {}
        self.keepalives = 0
        self.workers = set()
        self.assigned = {}            # node id -> (idx, params) not yet returned
        self.requeued = 0
        self.rep = sp.RepServer(url, self.handle)
        self.url = self.rep.url

    # ------------------------------------------------------------ protocol
    def handle(self, body):
        op, msg = wire.parse_request(body)
        with self.lock:
            if op == "c":
                return wire.encode("p_n", {"s_n": self.n})
            if op == "p":
                self.workers.add(msg["str"])
                if msg["histNum"] > 0 and self.observed is None:
                    self.observed = np.asarray(msg["ohist"][:msg["histNum"]], dtype=np.float32)
                if self.finished:
                    return wire.encode("p_ga", {"idx": -2})
                self._expire()
                while self.pending and self.pending[0][0] in self.results:
                    self.pending.pop(0)       # requeued, then returned late by its first worker
                if msg["str"] in self.assigned:
                    idx, params = self.assigned[msg["str"]]
                elif not self.pending:
                    return wire.encode("p_ga", {"idx": -1, "bestfv": self.bestfv})
                else:
                    idx, params = self.pending.pop(0)
                    self.assigned[msg["str"]] = (idx, params)
                self.heard[idx] = time.monotonic()
                return wire.encode("p_ga", {"idx": idx, "start": self.start, "stop": self.stop,
                                            "bestfv": self.bestfv, "params": list(params)})
            if op == "k":
                self.keepalives += 1
                if msg["sid"] in self.heard:
                    self.heard[msg["sid"]] = time.monotonic()
                return wire.encode("p_sid", {"sid": msg["sid"]})
            if op == "r":
                idx = msg["ridx"]
                if self.assigned.get(msg["idx"], (None,))[0] == idx:
                    del self.assigned[msg["idx"]]
                self.results[idx] = {"e": msg["e"], "shist": np.asarray(msg["shist"], dtype=np.float32)
                                     if msg["hist"] else None, "node": msg["idx"]}
                if msg["e"] < self.bestfv:
                    self.bestfv = msg["e"]
                    self.best_params = self.params_of.get(idx)
                self.lock.notify_all()
                return wire.encode("p_sid", {"sid": -1 if self.finished else 0})
        return None

    def _expire(self):
        if self.lease_s is None:
            return
        now = time.monotonic()
        for node, (idx, params) in list(self.assigned.items()):
            if idx in self.results:
                del self.assigned[node]
            elif now - self.heard.get(idx, now) > self.lease_s:
                del self.assigned[node]
                self.pending.insert(0, (idx, params))
                self.requeued += 1

    # ------------------------------------------------------------ optimiser side
    def submit(self, params_list):
        idxs = []
        with self.lock:
            for p in params_list:
                p = np.asarray(p, dtype=np.float32).reshape(-1)
                if p.size != self.n * (self.n + 1):
                    raise ValueError("parameter vector must hold n(n+1) values")
                idx = self.next_idx
                self.next_idx += 1
                self.pending.append((idx, p))
                self.params_of[idx] = p
                idxs.append(idx)
        return idxs

    def wait(self, idxs, timeout=None):
        deadline = None if timeout is None else time.monotonic() + timeout
        with self.lock:
            while not all(i in self.results for i in idxs):
                left = None if deadline is None else deadline - time.monotonic()
                if left is not None and left <= 0:
                    raise TimeoutError("results missing for %s" % [i for i in idxs if i not in self.results])
                self.lock.wait(timeout=left if left is not None else 1.0)
            return [self.results[i]["e"] for i in idxs]

    def evaluate(self, params_list, timeout=None):
        return np.asarray(self.wait(self.submit(params_list), timeout), dtype=np.float64)

    def finish(self):
        with self.lock:
            self.finished = True
            self.lock.notify_all()

    def close(self):
        self.finish()
        self.rep.close()
