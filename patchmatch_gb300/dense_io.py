"""Reading the dense map message and exporting it as PLY.

``write_ply`` / ``write_dense_msgpack`` in :mod:`patchmatch_gb300.native`
write the files (C ABI).  This module reads a dense map message back without
third-party packages and converts it to PLY the way the reference's
``export_dense_msg_to_ply.py`` does (landmark ``pos_w`` and ``color``, four
decimals, white when colours are not wanted).
"""
from __future__ import annotations

import os
import struct


def _unpack(b: bytes, o: int):
    t = b[o]
    if t <= 0x7F:
        return t, o + 1
    if 0x80 <= t <= 0x8F:
        return _map(b, o + 1, t & 0x0F)
    if 0x90 <= t <= 0x9F:
        return _arr(b, o + 1, t & 0x0F)
    if 0xA0 <= t <= 0xBF:
        n = t & 0x1F
        return b[o + 1:o + 1 + n].decode(), o + 1 + n
    if t >= 0xE0:
        return t - 256, o + 1
    if t == 0xC0:
        return None, o + 1
    if t in (0xC2, 0xC3):
        return t == 0xC3, o + 1
    fixed = {0xCA: ">f", 0xCB: ">d", 0xCC: ">B", 0xCD: ">H", 0xCE: ">I", 0xCF: ">Q",
             0xD0: ">b", 0xD1: ">h", 0xD2: ">i", 0xD3: ">q"}
    if t in fixed:
        fmt = fixed[t]
        n = struct.calcsize(fmt)
        return struct.unpack_from(fmt, b, o + 1)[0], o + 1 + n
    sized = {0xD9: (1, "s"), 0xDA: (2, "s"), 0xDB: (4, "s"), 0xC4: (1, "b"), 0xC5: (2, "b"), 0xC6: (4, "b"),
             0xDC: (2, "a"), 0xDD: (4, "a"), 0xDE: (2, "m"), 0xDF: (4, "m")}
    if t in sized:
        w, kind = sized[t]
        n = int.from_bytes(b[o + 1:o + 1 + w], "big")
        o += 1 + w
        if kind == "s":
            return b[o:o + n].decode(), o + n
        if kind == "b":
            return bytes(b[o:o + n]), o + n
        if kind == "a":
            return _arr(b, o, n)
        return _map(b, o, n)
    raise ValueError(f"unsupported MessagePack type 0x{t:02x} at offset {o}")


def _arr(b, o, n):
    out = []
    for _ in range(n):
        v, o = _unpack(b, o)
        out.append(v)
    return out, o


def _map(b, o, n):
    out = {}
    for _ in range(n):
        k, o = _unpack(b, o)
        v, o = _unpack(b, o)
        out[k] = v
    return out, o


def read_dense_msg(path) -> dict:
    """Decode a dense map message (MessagePack) into Python objects."""
    with open(path, "rb") as f:
        data = f.read()
    msg, end = _unpack(data, 0)
    if end != len(data):
        raise ValueError(f"{len(data) - end} trailing bytes in {path}")
    return msg


def msg_to_ply(msg_path, ply_path=None, nocolor: bool = False, scale: float = 1.0) -> str:
    """PLY of the message's landmarks: "x y z c0 c1 c2" per point with four
    decimals (the reference's exporter); returns the output path."""
    msg = read_dense_msg(msg_path)
    lms = msg["landmarks"]
    out = ply_path or str(msg_path) + ".ply"
    d = os.path.dirname(os.path.abspath(out))
    if not os.path.isdir(d):
        raise NotADirectoryError(d)
    with open(out, "w", encoding="utf-8") as f:
        f.write("ply\nformat ascii 1.0\n")
        f.write(f"element vertex {len(lms)}\n")
        f.write("property float x\nproperty float y\nproperty float z\n")
        f.write("property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n")
        for key in lms:
            p = lms[key]["pos_w"]
            c = (255, 255, 255) if nocolor else lms[key]["color"]
            f.write(f"{scale * p[0]:.4f} {scale * p[1]:.4f} {scale * p[2]:.4f} {int(c[0])} {int(c[1])} {int(c[2])}\n")
    return out
