"""Parameter-server protocol (3rdparty/protobuf/args.proto, src/streamWorker.cpp):
protobuf wire codec, SP request/reply over TCP, the worker state machine
against a parameter server, and failure handling (replies that are dropped,
-1/-2 replies, keep-alives, a server that goes away), all on the host."""
import socket
import struct
import threading
import time

import numpy as np
import pytest

from gsmfretda_gb300.ps import server as psrv
from gsmfretda_gb300.ps import sp, wire
from gsmfretda_gb300.ps import worker as pw

# ------------------------------------------------------------------ wire codec


def test_known_encodings():
    assert wire.encode("p_n", {"s_n": 3}) == b"\x08\x03"
    assert wire.encode("p_n", {"s_n": 0}) == b""                       # proto3 default omitted
    assert wire.encode("p_ga", {"idx": -1}) == b"\x08" + b"\xff" * 9 + b"\x01"
    assert wire.encode("p_sid", {"sid": -2}) == b"\x08" + b"\xfe" + b"\xff" * 8 + b"\x01"
    assert wire.encode("p_cap", {"cap": 300}) == b"\x08\xac\x02"
    ga = wire.encode("p_ga", {"idx": 5, "start": 1, "stop": 7, "bestfv": 1.5, "params": [0.25, 2.0]})
    assert ga == (b"\x08\x05\x10\x01\x18\x07" + b"\x25" + struct.pack("<f", 1.5) +
                  b"\x2a\x08" + struct.pack("<2f", 0.25, 2.0))
    r = wire.encode("res", {"ridx": 2, "e": 0.5, "hist": True, "idx": "ab", "shist": [1.0]})
    assert r == (b"\x08\x02\x15" + struct.pack("<f", 0.5) + b"\x18\x01\x22\x02ab" +
                 b"\x2a\x04" + struct.pack("<f", 1.0))


def test_roundtrip_and_unpacked_floats():
    msg = {"histNum": 21, "str": "node-1", "ohist": [float(i) for i in range(21)]}
    got = wire.decode("p_str", wire.encode("p_str", msg))
    assert got["histNum"] == 21 and got["str"] == "node-1" and got["ohist"] == msg["ohist"]
    # repeated floats written unpacked (one fixed32 per element) are accepted too
    unpacked = b"".join(b"\x1d" + struct.pack("<f", v) for v in (1.0, 2.0))
    assert wire.decode("p_str", unpacked)["ohist"] == [1.0, 2.0]
    # unknown fields are skipped
    assert wire.decode("p_n", b"\x10\x05\x08\x04")["s_n"] == 4
    assert wire.decode("p_ga", wire.encode("p_ga", {"idx": -2}))["idx"] == -2


def _google_classes():
    pytest.importorskip("google.protobuf")
    from google.protobuf import descriptor_pb2, descriptor_pool, message_factory
    fdp = descriptor_pb2.FileDescriptorProto(name="args.proto", package="gSMFRETda.pb", syntax="proto3")
    T = descriptor_pb2.FieldDescriptorProto
    kinds = {"int32": T.TYPE_INT32, "float": T.TYPE_FLOAT, "bool": T.TYPE_BOOL, "string": T.TYPE_STRING,
             "floats": T.TYPE_FLOAT}
    for name, fields in wire.SCHEMA.items():
        m = fdp.message_type.add(name=name)
        for num, fname, kind in fields:
            f = m.field.add(name=fname, number=num, type=kinds[kind],
                            label=T.LABEL_REPEATED if kind == "floats" else T.LABEL_OPTIONAL)
            if kind == "floats":
                f.options.packed = True
    pool = descriptor_pool.DescriptorPool()
    fd = pool.Add(fdp)
    return {name: message_factory.GetMessageClass(fd.message_types_by_name[name]) for name in wire.SCHEMA}


def test_byte_compatible_with_google_protobuf():
    cls = _google_classes()
    rng = np.random.default_rng(1)
    for _ in range(200):
        name = str(rng.choice(list(wire.SCHEMA)))
        msg = {}
        for _, fname, kind in wire.SCHEMA[name]:
            if kind == "int32":
                msg[fname] = int(rng.integers(-3, 1 << 20)) if rng.random() < 0.8 else 0
            elif kind == "float":
                msg[fname] = float(np.float32(rng.normal() * 10))
            elif kind == "bool":
                msg[fname] = bool(rng.random() < 0.5)
            elif kind == "string":
                msg[fname] = "node-%d" % rng.integers(0, 1000)
            else:
                msg[fname] = [float(np.float32(x)) for x in rng.normal(size=int(rng.integers(0, 30)))]
        ours = wire.encode(name, msg)
        g = cls[name]()
        for k, v in msg.items():
            if isinstance(v, list):
                getattr(g, k).extend(v)
            else:
                setattr(g, k, v)
        assert ours == g.SerializeToString(deterministic=True), name
        back = wire.decode(name, g.SerializeToString())
        for k, v in msg.items():
            assert back[k] == v


# ------------------------------------------------------------------ SP transport


def test_sp_handshake_and_request_id_echo():
    seen = []

    def handler(body):
        seen.append(body)
        return b"re:" + body

    srv = sp.RepServer("tcp://127.0.0.1:0", handler)
    try:
        # raw client: header + framed message with a request id
        s = socket.create_connection(("127.0.0.1", srv.port))
        s.sendall(b"\x00SP\x00\x00\x30\x00\x00")
        hdr = s.recv(8)
        assert hdr == b"\x00SP\x00\x00\x31\x00\x00"                  # REP = 49
        rid = 0x80000007
        body = struct.pack(">I", rid) + b"hello"
        s.sendall(struct.pack(">Q", len(body)) + body)
        n = struct.unpack(">Q", s.recv(8))[0]
        reply = b""
        while len(reply) < n:
            reply += s.recv(n - len(reply))
        assert reply == struct.pack(">I", rid) + b"re:hello"
        s.close()
        c = sp.ReqSocket(srv.url)
        assert c.request(b"x") == b"re:x"
        assert c.request(b"y") == b"re:y"
        c.close()
    finally:
        srv.close()


def test_req_resends_after_a_dropped_reply():
    count = {"n": 0}

    def handler(body):
        count["n"] += 1
        return None if count["n"] == 1 else b"ok"

    srv = sp.RepServer("tcp://127.0.0.1:0", handler)
    try:
        c = sp.ReqSocket(srv.url, resend_s=0.2)
        assert c.request(b"q", deadline_s=10) == b"ok"
        assert c.resends >= 1
        c.close()
    finally:
        srv.close()


def test_req_reconnects_when_the_server_comes_back():
    port = sp.RepServer("tcp://127.0.0.1:0", lambda b: b"")
    url = port.url
    port.close()
    got = {}

    def client():
        c = sp.ReqSocket(url, reconnect_ivl=0.05)
        got["r"] = c.request(b"z", deadline_s=20)
        c.close()

    t = threading.Thread(target=client)
    t.start()
    time.sleep(0.3)
    srv = sp.RepServer(url, lambda b: b"back")
    t.join(timeout=20)
    srv.close()
    assert got.get("r") == b"back"


# ------------------------------------------------------------------ chi-square


def test_reference_fp32_chi2_matches_oracle(orc):
    rng = np.random.default_rng(3)
    for _ in range(50):
        nb = int(rng.integers(5, 60))
        mh = rng.integers(0, 400, nb).astype(np.float32)
        mh[rng.random(nb) < 0.2] = 0
        oh = rng.integers(0, 100, nb).astype(np.float32)
        R, n = int(rng.integers(1, 8)), int(rng.integers(1, 3))
        got = pw.chi2_reference_f32(mh, oh, 2, R, n)
        want = orc.chi2_f32(mh, oh, nb, 2, R, n)
        assert np.float32(got) == np.float32(want)


# ------------------------------------------------------------------ worker state machine


class FakeEval:
    """Deterministic stand-in for the GPU: chi2 = sum(params)."""

    def __init__(self, sleep=0.0):
        self.sleep = sleep
        self.calls = []

    def evaluate(self, sid, n, params, start, stop):
        self.calls.append((sid, n, start, stop))
        if self.sleep:
            time.sleep(self.sleep)
        return float(np.sum(params)), np.full(21, 0.5, dtype=np.float32)


def _run_workers(server, ev, nworkers, **kw):
    outs = [None] * nworkers
    ths = []
    for i in range(nworkers):
        w = pw.StreamWorker(server.url, ev, np.arange(21, dtype=np.float32), 21, **kw)

        def run(i=i, w=w):
            outs[i] = w.run(i, 1000)
        t = threading.Thread(target=run, daemon=True)
        t.start()
        ths.append((t, w))
    return outs, ths


def test_workers_evaluate_everything_and_stop():
    srv = psrv.ParamServer(2, start=3, stop=900)
    try:
        ev = FakeEval()
        outs, ths = _run_workers(srv, ev, 3)
        params = [np.full(6, v, dtype=np.float32) for v in (1.0, 0.5, 2.0, 0.25, 3.0)]
        chi = srv.evaluate(params, timeout=30)
        np.testing.assert_allclose(chi, [6.0, 3.0, 12.0, 1.5, 18.0])
        assert srv.bestfv == pytest.approx(1.5)
        np.testing.assert_array_equal(srv.observed, np.arange(21, dtype=np.float32))
        assert all(c[1] == 2 and c[2] == 3 and c[3] == 900 for c in ev.calls)
        srv.finish()
        for t, _ in ths:
            t.join(timeout=30)
        assert set(outs) <= {"quit", "end"} and None not in outs
    finally:
        srv.close()


def test_histogram_sent_only_when_chi2_improves():
    srv = psrv.ParamServer(2)
    try:
        ev = FakeEval()
        outs, ths = _run_workers(srv, ev, 1)
        srv.evaluate([np.full(6, 1.0, dtype=np.float32)], timeout=30)       # improves on 3.1e32
        srv.evaluate([np.full(6, 2.0, dtype=np.float32)], timeout=30)       # worse than 6.0
        assert srv.results[0]["shist"] is not None
        assert srv.results[1]["shist"] is None
        srv.finish()
        ths[0][0].join(timeout=30)
    finally:
        srv.close()


def test_keepalives_while_the_gpu_is_busy():
    srv = psrv.ParamServer(2)
    try:
        ev = FakeEval(sleep=0.3)
        outs, ths = _run_workers(srv, ev, 1, wait_s=0.01, keepalive_every=5)
        srv.evaluate([np.ones(6, dtype=np.float32)], timeout=30)
        assert srv.keepalives >= 2
        srv.finish()
        ths[0][0].join(timeout=30)
    finally:
        srv.close()


def test_worker_survives_dropped_replies_and_empty_queues():
    srv = psrv.ParamServer(2)
    base = srv.handle
    state = {"n": 0}

    def flaky(body):
        state["n"] += 1
        if state["n"] % 4 == 2:
            return None                       # lost reply: the worker resends
        return base(body)

    srv.rep.handler = flaky
    try:
        ev = FakeEval()
        outs, ths = _run_workers(srv, ev, 2, resend_s=0.1)
        time.sleep(0.3)                      # workers are spinning on idx -1 meanwhile
        chi = srv.evaluate([np.full(6, v, dtype=np.float32) for v in (1, 2, 3)], timeout=30)
        np.testing.assert_allclose(chi, [6, 12, 18])
        srv.finish()
        for t, _ in ths:
            t.join(timeout=30)
            assert not t.is_alive()
    finally:
        srv.close()


def test_lost_assignment_reply_is_sent_again():
    """A 'p' reply carrying a parameter set is lost; the worker's resend must
    get the same set, so nothing is skipped."""
    srv = psrv.ParamServer(2)
    base = srv.handle
    dropped = []

    def flaky(body):
        reply = base(body)
        op, _ = wire.parse_request(body)
        if op == "p" and not dropped and wire.decode("p_ga", reply)["idx"] >= 0:
            dropped.append(wire.decode("p_ga", reply)["idx"])
            return None
        return reply

    srv.rep.handler = flaky
    try:
        ev = FakeEval()
        outs, ths = _run_workers(srv, ev, 1, resend_s=0.1)
        chi = srv.evaluate([np.full(6, v, dtype=np.float32) for v in (1, 2)], timeout=30)
        np.testing.assert_allclose(chi, [6, 12])
        assert dropped == [0] and len(ev.calls) == 2
        srv.finish()
        ths[0][0].join(timeout=30)
    finally:
        srv.close()


def test_set_of_a_vanished_worker_is_requeued():
    """A worker takes a parameter set and disappears; after the lease another
    worker evaluates it."""
    srv = psrv.ParamServer(2, lease_s=0.3)
    try:
        idxs = srv.submit([np.full(6, 2.0, dtype=np.float32)])
        c = sp.ReqSocket(srv.url)
        wire.decode("p_n", c.request(wire.request("c", {"cap": 10})))
        ga = wire.decode("p_ga", c.request(wire.request("p", {"str": "gone"})))
        assert ga["idx"] == idxs[0]
        c.close()                                  # never returns a result
        ev = FakeEval()
        outs, ths = _run_workers(srv, ev, 1)
        assert srv.wait(idxs, timeout=30) == [12.0]
        assert srv.requeued == 1
        srv.finish()
        ths[0][0].join(timeout=30)
    finally:
        srv.close()


def test_keepalives_hold_the_lease():
    """Two workers, one parameter set: the idle worker keeps polling, so the
    lease is checked; keep-alives of the busy one hold it, and without them
    the set is handed to the other worker as well."""
    for every, requeued in ((2, 0), (10 ** 6, 1)):
        srv = psrv.ParamServer(2, lease_s=0.2)
        try:
            ev = FakeEval(sleep=0.8)
            outs, ths = _run_workers(srv, ev, 2, wait_s=0.02, keepalive_every=every)
            srv.evaluate([np.ones(6, dtype=np.float32)], timeout=30)
            assert srv.requeued == requeued
            assert len(ev.calls) == 1 + requeued
            srv.finish()
            for t, _ in ths:
                t.join(timeout=30)
        finally:
            srv.close()
