"""A minimal Parquet writer and reader for tables of nullable float64 columns.

The result files of the solve path (the layout of crates/krets-result/src/lib.rs:20-208)
are flat tables of doubles, some entries missing.  This module writes them without a
third-party library, so the command line works where no Arrow binding is installed.
Format (Apache Parquet file format, version 1 data pages):

  "PAR1" | per column: PageHeader + data page | FileMetaData | len(FileMetaData) | "PAR1"

* one row group; every column OPTIONAL DOUBLE, uncompressed;
* a data page holds the definition levels (RLE / bit-packed hybrid, bit width 1, with its
  4-byte length prefix: runs of 1 = present, 0 = null) followed by the present values,
  PLAIN encoded (8-byte little-endian IEEE doubles);
* page headers and file metadata are Thrift structs in the compact protocol (field
  headers of delta-id and type nibbles, zigzag varints, length-prefixed binaries, list
  headers of size and element type).

read_parquet() reads files of this shape back (and the same shape written by other
writers: OPTIONAL or REQUIRED DOUBLE columns, PLAIN encoding, uncompressed v1 data pages).
"""
from __future__ import annotations

import struct
from typing import Dict, List, Optional

MAGIC = b"PAR1"

# compact-protocol element types
_T_TRUE, _T_FALSE, _T_BYTE, _T_I16, _T_I32, _T_I64, _T_DOUBLE, _T_BINARY, _T_LIST, _T_SET, _T_MAP, _T_STRUCT = \
    1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12
# parquet enums
_DOUBLE, _OPTIONAL, _REQUIRED = 5, 1, 0
_PLAIN, _RLE, _UNCOMPRESSED, _DATA_PAGE = 0, 3, 0, 0


# ------------------------------------------------------------------ compact protocol writer
def _varint(n: int) -> bytes:
    out = bytearray()
    while True:
        b = n & 0x7F
        n >>= 7
        if n:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _zigzag(n: int) -> int:
    return (n << 1) ^ (n >> 63)


class _Struct:
    """Builds one compact-protocol struct; fields must be added in increasing id order."""

    def __init__(self):
        self.buf = bytearray()
        self.last = 0

    def _field(self, fid: int, ftype: int):
        d = fid - self.last
        if 0 < d <= 15:
            self.buf.append((d << 4) | ftype)
        else:
            self.buf.append(ftype)
            self.buf += _varint(_zigzag(fid))
        self.last = fid

    def i32(self, fid, v):
        self._field(fid, _T_I32)
        self.buf += _varint(_zigzag(int(v)))
        return self

    def i64(self, fid, v):
        self._field(fid, _T_I64)
        self.buf += _varint(_zigzag(int(v)))
        return self

    def string(self, fid, s):
        b = s.encode() if isinstance(s, str) else bytes(s)
        self._field(fid, _T_BINARY)
        self.buf += _varint(len(b)) + b
        return self

    def struct(self, fid, st: "_Struct"):
        self._field(fid, _T_STRUCT)
        self.buf += st.done()
        return self

    def lst(self, fid, etype: int, items: List[bytes]):
        self._field(fid, _T_LIST)
        n = len(items)
        self.buf += bytes([(n << 4) | etype]) if n < 15 else bytes([0xF0 | etype]) + _varint(n)
        for it in items:
            self.buf += it
        return self

    def done(self) -> bytes:
        return bytes(self.buf) + b"\x00"


def _enc_i32(v):
    return _varint(_zigzag(int(v)))


def _enc_str(s):
    b = s.encode()
    return _varint(len(b)) + b


# ------------------------------------------------------------------ writer
def _def_levels(present: List[bool]) -> bytes:
    """RLE runs of the definition levels (bit width 1), with the 4-byte length prefix."""
    runs = bytearray()
    i = 0
    while i < len(present):
        j = i
        while j < len(present) and present[j] == present[i]:
            j += 1
        runs += _varint((j - i) << 1) + bytes([1 if present[i] else 0])
        i = j
    return struct.pack("<I", len(runs)) + bytes(runs)


def write_parquet(columns: Dict[str, List[Optional[float]]], filename) -> None:
    """Write {name: values (None = null)} as one row group of OPTIONAL DOUBLE columns."""
    names = list(columns)
    n_rows = len(columns[names[0]]) if names else 0
    for k in names:
        if len(columns[k]) != n_rows:
            raise ValueError(f"column {k!r} has {len(columns[k])} values, expected {n_rows}")
    body = bytearray(MAGIC)
    chunks = []
    for k in names:
        vals = columns[k]
        present = [v is not None for v in vals]
        data = _def_levels(present) + b"".join(struct.pack("<d", float(v)) for v in vals if v is not None)
        dph = _Struct().i32(1, n_rows).i32(2, _PLAIN).i32(3, _RLE).i32(4, _RLE)
        ph = _Struct().i32(1, _DATA_PAGE).i32(2, len(data)).i32(3, len(data)).struct(5, dph).done()
        offset = len(body)
        body += ph + data
        size = len(ph) + len(data)
        meta = (_Struct().i32(1, _DOUBLE).lst(2, _T_I32, [_enc_i32(_PLAIN), _enc_i32(_RLE)])
                .lst(3, _T_BINARY, [_enc_str(k)]).i32(4, _UNCOMPRESSED).i64(5, n_rows)
                .i64(6, size).i64(7, size).i64(9, offset))
        chunks.append((_Struct().i64(2, offset).struct(3, meta).done(), size))
    schema = [_Struct().string(4, "schema").i32(5, len(names)).done()]
    schema += [_Struct().i32(1, _DOUBLE).i32(3, _OPTIONAL).string(4, k).done() for k in names]
    rg = (_Struct().lst(1, _T_STRUCT, [c for c, _ in chunks]).i64(2, sum(s for _, s in chunks))
          .i64(3, n_rows).done())
    fmd = (_Struct().i32(1, 1).lst(2, _T_STRUCT, schema).i64(3, n_rows).lst(4, _T_STRUCT, [rg])
           .string(6, "krets_gb300").done())
    body += fmd + struct.pack("<I", len(fmd)) + MAGIC
    with open(filename, "wb") as f:
        f.write(bytes(body))


# ------------------------------------------------------------------ compact protocol reader
class _Reader:
    def __init__(self, b: bytes, pos: int = 0):
        self.b = b
        self.p = pos

    def varint(self) -> int:
        shift = out = 0
        while True:
            c = self.b[self.p]
            self.p += 1
            out |= (c & 0x7F) << shift
            if not c & 0x80:
                return out
            shift += 7

    def zz(self) -> int:
        v = self.varint()
        return (v >> 1) ^ -(v & 1)

    def value(self, t: int):
        if t in (_T_TRUE, _T_FALSE):
            return t == _T_TRUE
        if t == _T_BYTE:
            self.p += 1
            return self.b[self.p - 1]
        if t in (_T_I16, _T_I32, _T_I64):
            return self.zz()
        if t == _T_DOUBLE:
            self.p += 8
            return struct.unpack_from("<d", self.b, self.p - 8)[0]
        if t == _T_BINARY:
            n = self.varint()
            self.p += n
            return bytes(self.b[self.p - n:self.p])
        if t in (_T_LIST, _T_SET):
            h = self.b[self.p]
            self.p += 1
            n, et = h >> 4, h & 0x0F
            if n == 15:
                n = self.varint()
            if et in (_T_TRUE, _T_FALSE):  # booleans in lists are one byte each
                out = [self.b[self.p + i] == 1 for i in range(n)]
                self.p += n
                return out
            return [self.value(et) for _ in range(n)]
        if t == _T_MAP:
            n = self.varint()
            if n == 0:
                return {}
            kt, vt = self.b[self.p] >> 4, self.b[self.p] & 0x0F
            self.p += 1
            return {self.value(kt): self.value(vt) for _ in range(n)}
        if t == _T_STRUCT:
            return self.struct()
        raise ValueError(f"unknown compact type {t}")

    def struct(self) -> dict:
        out, last = {}, 0
        while True:
            h = self.b[self.p]
            self.p += 1
            if h == 0:
                return out
            t, d = h & 0x0F, h >> 4
            fid = last + d if d else self.zz()
            out[fid] = self.value(t)
            last = fid


def _rle_levels(b: bytes, pos: int, end: int, n: int) -> List[int]:
    """Decode n levels of bit width 1 from the RLE / bit-packed hybrid in b[pos:end]."""
    r = _Reader(b, pos)
    out: List[int] = []
    while len(out) < n and r.p < end:
        h = r.varint()
        if h & 1:  # bit-packed: (h >> 1) groups of 8 values
            cnt = (h >> 1) * 8
            for i in range(cnt):
                out.append((b[r.p + i // 8] >> (i % 8)) & 1)
            r.p += (cnt + 7) // 8
        else:
            v = b[r.p]
            r.p += 1
            out.extend([v & 1] * (h >> 1))
    return out[:n]


def read_parquet(filename) -> Dict[str, List[Optional[float]]]:
    """{name: values (None = null)} of a file of DOUBLE columns, PLAIN, uncompressed."""
    with open(filename, "rb") as f:
        b = f.read()
    if b[:4] != MAGIC or b[-4:] != MAGIC:
        raise ValueError("not a parquet file")
    n_meta = struct.unpack_from("<I", b, len(b) - 8)[0]
    fmd = _Reader(b, len(b) - 8 - n_meta).struct()
    schema = fmd[2]
    leaves = {s[4].decode(): s for s in schema[1:]}
    out: Dict[str, List[Optional[float]]] = {}
    for rg in fmd.get(4, []):
        for cc in rg[1]:
            md = cc[3]
            name = b".".join(md[3]).decode()
            if md[1] != _DOUBLE or md[4] != _UNCOMPRESSED:
                raise ValueError(f"column {name}: only uncompressed DOUBLE columns are supported")
            optional = leaves[name].get(3, _REQUIRED) == _OPTIONAL
            col = out.setdefault(name, [])
            pos = md.get(11, md[9])
            remaining = md[5]
            while remaining > 0:
                r = _Reader(b, pos)
                ph = r.struct()
                start = r.p
                if ph[1] != _DATA_PAGE:  # skip anything else (e.g. an index page)
                    pos = start + ph[3]
                    continue
                dph = ph[5]
                nv = dph[1]
                if dph[2] != _PLAIN:
                    raise ValueError(f"column {name}: only PLAIN data pages are supported")
                p = start
                if optional:
                    ln = struct.unpack_from("<I", b, p)[0]
                    levels = _rle_levels(b, p + 4, p + 4 + ln, nv)
                    p += 4 + ln
                else:
                    levels = [1] * nv
                k = sum(levels)
                vals = struct.unpack_from(f"<{k}d", b, p)
                it = iter(vals)
                col.extend(next(it) if lv else None for lv in levels)
                remaining -= nv
                pos = start + ph[3]
    return out
