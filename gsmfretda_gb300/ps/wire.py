"""Protocol-buffers wire codec of the parameter-server messages
(3rdparty/protobuf/args.proto:4-44, package gSMFRETda.pb), written from the
public protobuf encoding rules so that it needs no protoc or protobuf runtime:

  p_ga  { int32 idx=1; int32 start=2; int32 stop=3; float bestfv=4;
          repeated float params=5 [packed] }
  p_n   { int32 s_n=1 }
  p_sid { int32 sid=1 }
  p_cap { int32 cap=1 }
  p_str { int32 histNum=1; string str=2; repeated float ohist=3 [packed] }
  res   { int32 ridx=1; float e=2; bool hist=3; string idx=4;
          repeated float shist=5 [packed] }

Messages are plain dicts. proto3 rules: fields at their default value are not
written; int32 is a varint (negative values as 10-byte two's complement);
float is fixed32 little-endian; repeated floats are written packed and read in
either form. Unknown fields are skipped. Each request on the wire is a
one-letter opcode followed by the serialized message
(src/streamWorker.cpp:84-241): 'c' p_cap, 'p' p_str, 'k' p_sid, 'r' res.
"""
import struct

VARINT, FIXED64, LEN, FIXED32 = 0, 1, 2, 5

# name -> [(field number, field name, kind)], kind in int32 float bool string floats
SCHEMA = {
    "p_ga": [(1, "idx", "int32"), (2, "start", "int32"), (3, "stop", "int32"),
             (4, "bestfv", "float"), (5, "params", "floats")],
    "p_n": [(1, "s_n", "int32")],
    "p_sid": [(1, "sid", "int32")],
    "p_cap": [(1, "cap", "int32")],
    "p_str": [(1, "histNum", "int32"), (2, "str", "string"), (3, "ohist", "floats")],
    "res": [(1, "ridx", "int32"), (2, "e", "float"), (3, "hist", "bool"), (4, "idx", "string"),
            (5, "shist", "floats")],
}

DEFAULTS = {"int32": 0, "float": 0.0, "bool": False, "string": "", "floats": ()}


def _varint(v):
    v &= (1 << 64) - 1
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _read_varint(buf, pos):
    shift = 0
    v = 0
    while True:
        if pos >= len(buf):
            raise ValueError("truncated varint")
        b = buf[pos]
        pos += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, pos
        shift += 7
        if shift > 63:
            raise ValueError("varint too long")


def _int32(v):
    v &= (1 << 64) - 1
    if v >= 1 << 63:
        v -= 1 << 64
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= 1 << 31 else v


def encode(name, msg):
    out = bytearray()
    for num, field, kind in SCHEMA[name]:
        v = msg.get(field, DEFAULTS[kind])
        if kind == "int32":
            if int(v) != 0:
                out += _varint(num << 3 | VARINT) + _varint(int(v))
        elif kind == "bool":
            if v:
                out += _varint(num << 3 | VARINT) + b"\x01"
        elif kind == "float":
            fv = struct.pack("<f", float(v))
            if fv != b"\x00\x00\x00\x00":
                out += _varint(num << 3 | FIXED32) + fv
        elif kind == "string":
            bv = v.encode() if isinstance(v, str) else bytes(v)
            if bv:
                out += _varint(num << 3 | LEN) + _varint(len(bv)) + bv
        elif kind == "floats":
            vals = list(v)
            if vals:
                payload = struct.pack("<%df" % len(vals), *vals)
                out += _varint(num << 3 | LEN) + _varint(len(payload)) + payload
    return bytes(out)


def decode(name, data):
    fields = {num: (field, kind) for num, field, kind in SCHEMA[name]}
    msg = {field: (list(DEFAULTS[kind]) if kind == "floats" else DEFAULTS[kind])
           for _, field, kind in SCHEMA[name]}
    buf = bytes(data)
    pos = 0
    while pos < len(buf):
        tag, pos = _read_varint(buf, pos)
        num, wt = tag >> 3, tag & 7
        if wt == VARINT:
            v, pos = _read_varint(buf, pos)
        elif wt == FIXED32:
            v = buf[pos:pos + 4]
            pos += 4
        elif wt == FIXED64:
            v = buf[pos:pos + 8]
            pos += 8
        elif wt == LEN:
            ln, pos = _read_varint(buf, pos)
            v = buf[pos:pos + ln]
            pos += ln
        else:
            raise ValueError(f"unsupported wire type {wt}")
        if pos > len(buf):
            raise ValueError("truncated field")
        if num not in fields:
            continue
        field, kind = fields[num]
        if kind == "int32" and wt == VARINT:
            msg[field] = _int32(v)
        elif kind == "bool" and wt == VARINT:
            msg[field] = bool(v)
        elif kind == "float" and wt == FIXED32:
            msg[field] = struct.unpack("<f", v)[0]
        elif kind == "string" and wt == LEN:
            msg[field] = v.decode(errors="replace")
        elif kind == "floats":
            if wt == LEN:
                msg[field].extend(struct.unpack("<%df" % (len(v) // 4), v[:len(v) // 4 * 4]))
            elif wt == FIXED32:
                msg[field].append(struct.unpack("<f", v)[0])
    return msg


# one-letter opcodes of the worker's requests
REQUESTS = {"c": "p_cap", "p": "p_str", "k": "p_sid", "r": "res"}
# the parameter server's reply to each opcode
REPLIES = {"c": "p_n", "p": "p_ga", "k": "p_sid", "r": "p_sid"}


def request(op, msg):
    return op.encode() + encode(REQUESTS[op], msg)


def parse_request(data):
    op = chr(data[0])
    return op, decode(REQUESTS[op], data[1:])
