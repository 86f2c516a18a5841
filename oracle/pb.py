"""Protobuf-2 wire-format reader for the reference's event files, restated
from Event.proto:1-38 and the two file layouts (EventLoader.h:15-111: one
PEventContainer message; PEventStore.h:25-80: little-endian uint32 count,
then per event varint type 1, varint size, PEvent bytes).

TEST INFRASTRUCTURE ONLY: checks the native decoder.  Pure Python loops;
meant for files of a few MB.
"""
from __future__ import annotations

import struct

import numpy as np

CONTAINER, EVENT_STORE = 0, 1


def _varint(b, i):
    r = s = 0
    while True:
        if i >= len(b):
            raise ValueError("truncated varint")
        c = b[i]
        i += 1
        r |= (c & 0x7F) << s
        s += 7
        if c < 0x80:
            return r, i
        if s >= 70:
            raise ValueError("varint longer than 10 bytes")


def _fields(b):
    i = 0
    while i < len(b):
        key, i = _varint(b, i)
        f, w = key >> 3, key & 7
        if w == 0:
            v, i = _varint(b, i)
        elif w == 1:
            v, i = b[i:i + 8], i + 8
        elif w == 5:
            if i + 4 > len(b):
                raise ValueError("truncated fixed32")
            v, i = b[i:i + 4], i + 4
        elif w == 2:
            n, i = _varint(b, i)
            if i + n > len(b):
                raise ValueError("truncated length-delimited field")
            v, i = b[i:i + n], i + n
        else:
            raise ValueError(f"wire type {w}")
        yield f, w, v


def _hit(b):
    d = {}
    for f, w, v in _fields(b):
        d[f] = (w, v)
    for f in (1, 2, 3, 4, 5):
        if f not in d:
            raise ValueError(f"PHit field {f} missing")
    pos = {f: struct.unpack("<f", v)[0] for f, w, v in _fields(d[1][1]) if w == 5}
    if set(pos) != {1, 2, 3}:
        raise ValueError("PGlobalPoint incomplete")
    t = d[2][1]
    t = t - (1 << 64) if t >= 1 << 63 else t
    return (pos[1], pos[2], pos[3], t, d[3][1] & 0xFFFFFFFF, d[4][1] & 0xFFFFFFFF, d[5][1],
            d.get(6, (0, 0))[1] & 0xFFFFFFFF,
            struct.unpack("<f", d[7][1])[0] if 7 in d else 0.0)


def _event(b):
    hdr, hits = {}, []
    for f, w, v in _fields(b):
        if f == 4 and w == 2:
            hits.append(_hit(v))
        elif f in (1, 2, 3) and w == 0:
            hdr[f] = v
    if set(hdr) != {1, 2, 3}:
        raise ValueError("PEvent header incomplete")
    return (hdr[1], hdr[2], hdr[3]), hits


def decode(buf: bytes, fmt=CONTAINER):
    """Returns dict of numpy columns (as the native decoder fills them)."""
    if fmt == CONTAINER:
        evs = [v for f, w, v in _fields(buf) if f == 1 and w == 2]
    else:
        n = struct.unpack("<I", buf[:4])[0]
        i, evs = 4, []
        for _ in range(n):
            t, i = _varint(buf, i)
            if t != 1:
                raise ValueError("unknown entry type")
            ln, i = _varint(buf, i)
            evs.append(buf[i:i + ln])
            i += ln
    hdrs, rows, off = [], [], [0]
    for e in evs:
        h, hits = _event(e)
        hdrs.append(h)
        rows.extend(hits)
        off.append(len(rows))
    cols = list(zip(*rows)) if rows else [()] * 9
    f32 = lambda c: np.array(c, np.float32)
    u32 = lambda c: np.array(c, np.uint32)
    return {"run": np.array([h[0] for h in hdrs], np.uint64),
            "lumi": np.array([h[1] for h in hdrs], np.uint64),
            "event_number": np.array([h[2] for h in hdrs], np.uint64),
            "hit_offset": np.array(off, np.uint64),
            "x": f32(cols[0]), "y": f32(cols[1]), "z": f32(cols[2]),
            "detector_type": np.array(cols[3], np.int32), "layer": u32(cols[4]),
            "detector_id": u32(cols[5]), "hit_id": np.array(cols[6], np.uint64),
            "sim_track_id": u32(cols[7]), "sim_track_pt": f32(cols[8])}
