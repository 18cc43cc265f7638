"""Test infrastructure: a CPU restatement of the BinaryData section of the reference's
"WorldState v2binary" state format, the checker of the engine's GPU codec.  Only tests/ and
the fixture generator use it.

The section follows the line "BinaryData" and one zero byte (dpd_state_io.hpp:452-461).  For
each polymer of the world, in order (write_polymer_binary, dpd_state_io.hpp:182-247):

* a 16-bit header: polymer type (bits 0-12), "polymer id is not previous + 1" (bit 13),
  "first bead id is not previous + 1" (bit 14), "bead ids inside the polymer are not
  consecutive" (bit 15) -- the PolymerBinary bit-field, low bits first;
* if bit 13: uint32 polymer id minus the previous polymer id (mod 2^32; the previous id
  starts at 0xFFFFFFFF);
* per bead: if it is the first bead and bit 14, or a later bead and bit 15, a uint32 bead id
  minus the previous bead id (mod 2^32, previous starting at 0xFFFFFFFF); then the position
  as 3 uint32 with 16 fractional bits (round(x * 65536), half away from zero; the box side
  itself wraps to 0); then v and f as CVec3Half.

CVec3Half (cvec3.hpp:132-252) packs a vector into 32 bits, low bits first: a 5-bit exponent
field and three 9-bit two's-complement mantissas.  For a non-zero vector with largest
component exponent e (frexp), each mantissa is round(c * 2^(8 - e)); if one rounds to +-256,
e grows by one and all are rounded again; the field holds e + 15.  Components that are zero
or subnormal count as zero; a vector with e < -14 encodes as zero; e > 15 (magnitude 2^15 or
more after rounding) and non-finite components are errors.  Decoding: c = m * 2^(field - 23).

All arithmetic here is exact in IEEE double (scaling by powers of two, rounding to integers
below 2^31), so the GPU codec must reproduce these bytes exactly.
"""

from __future__ import annotations

import struct

import numpy as np

POS_SCALE = 65536.0


class V2Error(ValueError):
    pass


def _round_half_away(a):
    return np.sign(a) * np.floor(np.abs(a) + 0.5)


def cvec3half_encode(p):
    """(n, 3) float64 -> (n,) uint32 CVec3Half words."""
    p = np.array(p, np.float64, copy=True).reshape(-1, 3)
    if not np.all(np.isfinite(p)):
        raise V2Error("Attempt to convert nan or inf to CVec3Half.")
    p[np.abs(p) < np.finfo(np.float64).tiny] = 0.0  # zero and subnormal components
    nz = p != 0
    _, ex = np.frexp(p)
    e = np.where(nz, ex, np.iinfo(np.int32).min // 2).max(axis=1)
    live = nz.any(axis=1)
    if np.any(e[live] > 15):
        raise V2Error("Vector overflowed while converting to CVec3Half, so magnitude is 65536 or more.")
    live &= e >= -14
    e = np.where(live, e, 0)
    fr = _round_half_away(np.ldexp(p, (8 - e)[:, None]))
    over = live & np.any(np.abs(fr) == 256, axis=1)
    if np.any(e[over] + 1 > 15):
        raise V2Error("Vector overflowed while converting to CVec3Half, so magnitude is 65536 or more.")
    e = np.where(over, e + 1, e)
    fr = np.where(over[:, None], _round_half_away(np.ldexp(p, (8 - e)[:, None])), fr)
    m = fr.astype(np.int64) & 0x1FF
    w = ((e + 15) & 0x1F) | (m[:, 0] << 5) | (m[:, 1] << 14) | (m[:, 2] << 23)
    return np.where(live, w, 0).astype(np.uint32)


def cvec3half_decode(w):
    """(n,) uint32 -> (n, 3) float64."""
    w = np.asarray(w, np.uint32).astype(np.int64)
    ex = w & 0x1F
    m = np.stack([(w >> 5) & 0x1FF, (w >> 14) & 0x1FF, (w >> 23) & 0x1FF], axis=1)
    m = np.where(m >= 256, m - 512, m)
    return np.ldexp(m.astype(np.float64), (ex - 23)[:, None])


def encode_positions(x, box):
    x = np.asarray(x, np.float64).reshape(-1, 3)
    L = np.asarray(box, np.float64)[None, :] * POS_SCALE
    rr = _round_half_away(x * POS_SCALE)
    rr = np.where(rr == L, 0.0, rr)
    if np.any(rr < 0) or np.any(rr >= L):
        raise V2Error("Bead is out of bounds.")
    return rr.astype(np.uint32)


def _polymers(world, polymer_ids=None):
    npoly = len(world.poly_type)
    ids = np.arange(npoly, dtype=np.uint32) if polymer_ids is None else np.asarray(polymer_ids, np.uint32)
    for p in range(npoly):
        yield int(ids[p]), int(world.poly_type[p]), world.poly_beads[world.poly_start[p]:world.poly_start[p + 1]]


def encode_section(world, x=None, v=None, f=None, polymer_ids=None) -> bytes:
    """The BinaryData section for the world's polymers with bead state x, v, f (default: the
    world's own)."""
    x = world.x if x is None else x
    v = world.v if v is None else v
    f = world.f if f is None else f
    pos = encode_positions(x, world.box)
    hv, hf = cvec3half_encode(v), cvec3half_encode(f)
    out = bytearray()
    M = 0xFFFFFFFF
    prev_pid, prev_bid = M, M
    for pid, ptype, beads in _polymers(world, polymer_ids):
        if ptype >= 1 << 13:
            raise V2Error("polymer type does not fit 13 bits")
        beads = [int(b) for b in beads]
        nsp = pid != ((prev_pid + 1) & M)
        nsi = beads[0] != ((prev_bid + 1) & M)
        nsa = any(beads[k - 1] + 1 != beads[k] for k in range(1, len(beads)))
        out += struct.pack("<H", ptype | (nsp << 13) | (nsi << 14) | (nsa << 15))
        if nsp:
            out += struct.pack("<I", (pid - prev_pid) & M)
        prev_pid = pid
        for k, b in enumerate(beads):
            if (k == 0 and nsi) or (k > 0 and nsa):
                out += struct.pack("<I", (b - prev_bid) & M)
            prev_bid = b
            out += pos[b].astype("<u4").tobytes()
            out += struct.pack("<II", int(hv[b]), int(hf[b]))
    return bytes(out)


def decode_section(world, data, polymer_ids=None):
    """Bead state (x, v, f), (n, 3) float64 each, from a BinaryData section of a world with the
    same polymers (read_polymer_binary, dpd_state_io.hpp:249-330)."""
    n = world.n_beads
    x, v, f = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    mv = memoryview(data)
    p = 0
    M = 0xFFFFFFFF
    prev_pid, prev_bid = M, M
    L = np.asarray(world.box, np.float64)
    for pid_expect, ptype_expect, beads_expect in _polymers(world, polymer_ids):
        (hdr,) = struct.unpack_from("<H", mv, p)
        p += 2
        if (hdr & 0x1FFF) != ptype_expect:
            raise V2Error("polymer type differs from the world's")
        if hdr & (1 << 13):
            (d,) = struct.unpack_from("<I", mv, p)
            p += 4
            pid = (prev_pid + d) & M
        else:
            pid = (prev_pid + 1) & M
        if pid != pid_expect:
            raise V2Error("polymer id differs from the world's")
        prev_pid = pid
        for k, b_expect in enumerate(beads_expect):
            if (k == 0 and hdr & (1 << 14)) or (k > 0 and hdr & (1 << 15)):
                (d,) = struct.unpack_from("<I", mv, p)
                p += 4
                b = (prev_bid + d) & M
            else:
                b = (prev_bid + 1) & M
            if b != int(b_expect):
                raise V2Error("bead id differs from the world's")
            prev_bid = b
            pos = np.frombuffer(mv, "<u4", 3, p).astype(np.float64)
            wv, wf = struct.unpack_from("<II", mv, p + 12)
            p += 20
            xb = np.ldexp(pos, -16)
            if np.any(xb < 0) or np.any(xb >= L):
                raise V2Error("Bead was out of box.")
            x[b] = xb
            v[b] = cvec3half_decode([wv])[0]
            f[b] = cvec3half_decode([wf])[0]
    if p != len(data):
        raise V2Error("trailing bytes after the last polymer")
    return x, v, f


def split_file(data: bytes):
    """(header text bytes, section bytes) of a v2binary file."""
    marker = b"BinaryData\n\x00"
    k = data.index(marker)
    return data[:k + len(marker)], data[k + len(marker):]
