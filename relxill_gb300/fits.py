"""Minimal FITS binary-table writer and reader (numpy only).

The relxill tables are FITS files with binary-table extensions. cfitsio and
astropy are not available here, so this module implements the small subset of
the FITS standard (v4.0, sections 4 and 7.3) that the tables use:

* a primary HDU without data,
* BINTABLE extensions whose columns are fixed-length vectors of
  ``E`` (float32), ``D`` (float64), ``J`` (int32) or ``A`` (characters),
* big-endian row storage, headers and data padded to 2880-byte blocks.

The writer is used by :mod:`relxill_gb300.synth_tables`; the reader is used by
the tests to check those files independently of the C++ loader.
"""
from __future__ import annotations

import io
from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple

import numpy as np

BLOCK = 2880
_CODE = {"E": (">f4", 4), "D": (">f8", 8), "J": (">i4", 4), "A": ("S1", 1)}


def _card(key: str, value=None, comment: str = "") -> bytes:
    """Format one 80-character header card."""
    if value is None:
        text = key.ljust(80)
    else:
        if isinstance(value, bool):
            v = "T" if value else "F"
            v = v.rjust(20)
        elif isinstance(value, int):
            v = str(value).rjust(20)
        elif isinstance(value, float):
            v = repr(value).upper().rjust(20)
        else:
            s = str(value).replace("'", "''")
            v = ("'" + s.ljust(8) + "'").ljust(20)
        text = key.ljust(8) + "= " + v
        if comment:
            text += " / " + comment
    text = text[:80].ljust(80)
    return text.encode("ascii")


def _pad(b: bytes, fill: bytes) -> bytes:
    rem = len(b) % BLOCK
    return b if rem == 0 else b + fill * (BLOCK - rem)


def primary_header() -> bytes:
    cards = [
        _card("SIMPLE", True),
        _card("BITPIX", 8),
        _card("NAXIS", 0),
        _card("EXTEND", True),
        _card("END"),
    ]
    return _pad(b"".join(cards), b" ")


@dataclass
class Column:
    name: str
    code: str  # one of E, D, J, A
    repeat: int
    data: np.ndarray  # shape (nrows, repeat) for numbers, (nrows,) of str for A


def bintable(extname: str, columns: Sequence[Column], nrows: int) -> bytes:
    """Serialise one BINTABLE HDU (header + data)."""
    width = 0
    dtype_fields = []
    for c in columns:
        np_code, size = _CODE[c.code]
        if c.code == "A":
            dtype_fields.append((c.name, f"S{c.repeat}"))
        else:
            dtype_fields.append((c.name, np_code, (c.repeat,)))
        width += size * c.repeat
    rec = np.zeros(nrows, dtype=np.dtype(dtype_fields))
    for c in columns:
        if c.code == "A":
            rec[c.name] = np.array([s.encode("ascii")[: c.repeat] for s in c.data])
        else:
            rec[c.name] = np.asarray(c.data).reshape(nrows, c.repeat)
    cards = [
        _card("XTENSION", "BINTABLE"),
        _card("BITPIX", 8),
        _card("NAXIS", 2),
        _card("NAXIS1", width),
        _card("NAXIS2", nrows),
        _card("PCOUNT", 0),
        _card("GCOUNT", 1),
        _card("TFIELDS", len(columns)),
    ]
    for i, c in enumerate(columns, 1):
        cards.append(_card(f"TTYPE{i}", c.name))
        cards.append(_card(f"TFORM{i}", f"{c.repeat}{c.code}"))
    cards.append(_card("EXTNAME", extname))
    cards.append(_card("END"))
    return _pad(b"".join(cards), b" ") + _pad(rec.tobytes(), b"\0")


class StreamingTable:
    """Write a BINTABLE HDU whose rows arrive in chunks (for tables of ~1 GB)."""

    def __init__(self, fh, extname: str, columns: Sequence[Tuple[str, str, int]], nrows: int):
        self.fh = fh
        self.nrows = nrows
        self.written = 0
        fields = []
        width = 0
        for name, code, repeat in columns:
            np_code, size = _CODE[code]
            fields.append((name, np_code, (repeat,)))
            width += size * repeat
        self.dtype = np.dtype(fields)
        cards = [
            _card("XTENSION", "BINTABLE"),
            _card("BITPIX", 8),
            _card("NAXIS", 2),
            _card("NAXIS1", width),
            _card("NAXIS2", nrows),
            _card("PCOUNT", 0),
            _card("GCOUNT", 1),
            _card("TFIELDS", len(columns)),
        ]
        for i, (name, code, repeat) in enumerate(columns, 1):
            cards.append(_card(f"TTYPE{i}", name))
            cards.append(_card(f"TFORM{i}", f"{repeat}{code}"))
        cards.append(_card("EXTNAME", extname))
        cards.append(_card("END"))
        fh.write(_pad(b"".join(cards), b" "))
        self.nbytes = width * nrows

    def write_rows(self, **cols):
        n = len(next(iter(cols.values())))
        rec = np.zeros(n, dtype=self.dtype)
        for k, v in cols.items():
            rec[k] = v
        self.fh.write(rec.tobytes())
        self.written += n

    def close(self):
        assert self.written == self.nrows, (self.written, self.nrows)
        rem = self.nbytes % BLOCK
        if rem:
            self.fh.write(b"\0" * (BLOCK - rem))


# ----------------------------------------------------------------------------
# reader
# ----------------------------------------------------------------------------

@dataclass
class HDU:
    header: Dict[str, str]
    offset: int  # byte offset of the data
    columns: List[Tuple[str, str, int]] = field(default_factory=list)
    nrows: int = 0
    width: int = 0

    @property
    def name(self) -> str:
        return self.header.get("EXTNAME", "").strip("' ").strip()


def _parse_value(raw: str) -> str:
    raw = raw.strip()
    if raw.startswith("'"):
        end = raw.find("'", 1)
        while end + 1 < len(raw) and raw[end + 1] == "'":
            end = raw.find("'", end + 2)
        return raw[1:end].replace("''", "'").rstrip()
    return raw.split("/")[0].strip()


def read_hdus(path: str) -> List[HDU]:
    hdus = []
    with open(path, "rb") as f:
        pos = 0
        while True:
            f.seek(pos)
            header = {}
            nbytes = 0
            done = False
            while not done:
                block = f.read(BLOCK)
                if len(block) < BLOCK:
                    return hdus
                nbytes += BLOCK
                for i in range(0, BLOCK, 80):
                    card = block[i:i + 80].decode("ascii")
                    key = card[:8].strip()
                    if key == "END":
                        done = True
                        break
                    if card[8:10] == "= ":
                        header[key] = _parse_value(card[10:])
            hdu = HDU(header=header, offset=pos + nbytes)
            naxis = int(header.get("NAXIS", "0"))
            if naxis == 2 and header.get("XTENSION", "") == "BINTABLE":
                hdu.width = int(header["NAXIS1"])
                hdu.nrows = int(header["NAXIS2"])
                for i in range(1, int(header["TFIELDS"]) + 1):
                    form = header[f"TFORM{i}"].strip()
                    rep = int(form[:-1]) if len(form) > 1 else 1
                    hdu.columns.append((header[f"TTYPE{i}"], form[-1], rep))
                datasize = hdu.width * hdu.nrows + int(header.get("PCOUNT", "0"))
            else:
                datasize = 0
            hdus.append(hdu)
            pos = hdu.offset + ((datasize + BLOCK - 1) // BLOCK) * BLOCK


def read_table(path: str, hdu: HDU, rows=None) -> Dict[str, np.ndarray]:
    """Read all columns of a BINTABLE HDU into a dict of native arrays."""
    fields = []
    for name, code, rep in hdu.columns:
        if code == "A":
            fields.append((name, f"S{rep}"))
        else:
            fields.append((name, _CODE[code][0], (rep,)))
    dt = np.dtype(fields)
    with open(path, "rb") as f:
        if rows is None:
            f.seek(hdu.offset)
            rec = np.frombuffer(f.read(hdu.width * hdu.nrows), dtype=dt)
        else:
            r0, r1 = rows
            f.seek(hdu.offset + r0 * hdu.width)
            rec = np.frombuffer(f.read(hdu.width * (r1 - r0)), dtype=dt)
    out = {}
    for name, code, rep in hdu.columns:
        col = rec[name]
        if code == "A":
            out[name] = np.array([s.decode("ascii").rstrip() for s in col])
        else:
            out[name] = col.astype(col.dtype.newbyteorder("="))
    return out


def find_hdu(hdus: List[HDU], extname: str) -> HDU:
    for h in hdus:
        if h.name.upper() == extname.upper():
            return h
    raise KeyError(extname)
