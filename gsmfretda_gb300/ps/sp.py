"""Request/reply over TCP in the Scalability Protocols wire format that nng
and nanomsg speak (the reference worker opens an NN_REQ socket,
src/streamWorker.cpp:49-55), written from the published SP specifications:

TCP mapping: after connecting, each peer sends an 8-byte header
    0x00 'S' 'P' 0x00 <protocol id, uint16 big-endian> 0x00 0x00
(REQ = 48, REP = 49, i.e. NN_PROTO_REQREP * 16 + {0, 1}); every message is then
framed as a 64-bit big-endian length followed by the payload.

Request/reply: a REQ prefixes each request body with a 32-bit big-endian
request id whose top bit is set; the REP reads the "backtrace" (32-bit words up
to and including the first one with the top bit set) and puts it in front of
its reply, which the REQ matches against the id it sent.
"""
import random
import socket
import struct
import threading
import time

PROTO_REQ = 48
PROTO_REP = 49


def _header(proto):
    return b"\x00SP\x00" + struct.pack(">H", proto) + b"\x00\x00"


def parse_url(url):
    if not url.startswith("tcp://"):
        raise ValueError(f"only tcp:// urls are supported: {url}")
    host, _, port = url[6:].rpartition(":")
    return (host or "127.0.0.1").strip("[]"), int(port)


class SPConnection:
    """One TCP connection after the SP handshake."""

    def __init__(self, sock, own_proto, peer_proto):
        self.sock = sock
        sock.sendall(_header(own_proto))
        hdr = self._read(8)
        if hdr[:4] != b"\x00SP\x00" or hdr[6:] != b"\x00\x00":
            raise ConnectionError("peer is not speaking the SP protocol")
        (proto,) = struct.unpack(">H", hdr[4:6])
        if proto != peer_proto:
            raise ConnectionError(f"peer protocol {proto}, expected {peer_proto}")

    def _read(self, n):
        buf = bytearray()
        while len(buf) < n:
            chunk = self.sock.recv(n - len(buf))
            if not chunk:
                raise ConnectionError("connection closed")
            buf += chunk
        return bytes(buf)

    def send(self, payload):
        self.sock.sendall(struct.pack(">Q", len(payload)) + payload)

    def recv(self, max_size=1 << 26):
        (n,) = struct.unpack(">Q", self._read(8))
        if n > max_size:
            raise ConnectionError(f"message of {n} bytes exceeds the limit")
        return self._read(n)

    def close(self):
        try:
            self.sock.close()
        except OSError:
            pass


class ReqSocket:
    """Client side (NN_REQ): connect, send a request, wait for its reply.
    Reconnects every `reconnect_ivl` seconds while the server is away (the
    reference sets NN_RECONNECT_IVL = 200 ms, src/streamWorker.cpp:51-52) and,
    like an nng REQ socket, sends a request again (same id) when no reply has
    come after `resend_s` seconds (nng's default is 60 s)."""

    def __init__(self, url, reconnect_ivl=0.2, resend_s=60.0):
        self.addr = parse_url(url)
        self.reconnect_ivl = reconnect_ivl
        self.resend_s = resend_s
        self.conn = None
        self.next_id = random.getrandbits(31)
        self.resends = 0

    def _connect(self, deadline):
        while self.conn is None:
            try:
                s = socket.create_connection(self.addr, timeout=5.0)
                s.settimeout(5.0)
                self.conn = SPConnection(s, PROTO_REQ, PROTO_REP)
                s.settimeout(self.resend_s)
            except OSError:
                if deadline is not None and time.monotonic() > deadline:
                    raise TimeoutError(f"cannot reach {self.addr}")
                time.sleep(self.reconnect_ivl)

    def request(self, body, deadline_s=None):
        deadline = None if deadline_s is None else time.monotonic() + deadline_s
        rid = 0x80000000 | (self.next_id & 0x7FFFFFFF)
        self.next_id = (self.next_id + 1) & 0x7FFFFFFF
        payload = struct.pack(">I", rid) + body
        while True:
            self._connect(deadline)
            try:
                self.conn.send(payload)
                while True:
                    try:
                        msg = self.conn.recv()
                    except socket.timeout:
                        if deadline is not None and time.monotonic() > deadline:
                            raise TimeoutError("no reply")
                        self.resends += 1
                        self.conn.send(payload)
                        continue
                    if len(msg) >= 4 and struct.unpack(">I", msg[:4])[0] == rid:
                        return msg[4:]
            except TimeoutError:
                raise
            except (OSError, ConnectionError):
                # resend on a fresh connection, as a REQ socket does
                if self.conn:
                    self.conn.close()
                self.conn = None
                if deadline is not None and time.monotonic() > deadline:
                    raise TimeoutError("no reply")

    def close(self):
        if self.conn:
            self.conn.close()
        self.conn = None


class RepServer:
    """Server side (NN_REP): each connection is served on its own thread;
    handler(body) -> reply body, or None to drop the request (the client then
    waits, as it would for a lost message)."""

    def __init__(self, url, handler):
        self.addr = parse_url(url)
        self.handler = handler
        self.lsock = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
        self.lsock.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
        self.lsock.bind(self.addr)
        self.lsock.listen(64)
        self.port = self.lsock.getsockname()[1]
        self.url = f"tcp://{self.addr[0]}:{self.port}"
        self._stop = threading.Event()
        self._threads = []
        self._conns = []
        self._accept = threading.Thread(target=self._accept_loop, daemon=True)
        self._accept.start()

    def _accept_loop(self):
        self.lsock.settimeout(0.2)
        while not self._stop.is_set():
            try:
                s, _ = self.lsock.accept()
            except socket.timeout:
                continue
            except OSError:
                return
            t = threading.Thread(target=self._serve, args=(s,), daemon=True)
            t.start()
            self._threads.append(t)

    def _serve(self, s):
        try:
            s.settimeout(None)
            conn = SPConnection(s, PROTO_REP, PROTO_REQ)
        except (OSError, ConnectionError):
            s.close()
            return
        self._conns.append(conn)
        try:
            while not self._stop.is_set():
                msg = conn.recv()
                pos = 0
                while pos + 4 <= len(msg):
                    word = struct.unpack(">I", msg[pos:pos + 4])[0]
                    pos += 4
                    if word & 0x80000000:
                        break
                else:
                    continue       # no request id: not a request, ignore
                reply = self.handler(msg[pos:])
                if reply is not None:
                    conn.send(msg[:pos] + reply)
        except (OSError, ConnectionError):
            pass
        finally:
            conn.close()

    def close(self):
        self._stop.set()
        try:
            self.lsock.close()
        except OSError:
            pass
        for c in self._conns:
            c.close()
