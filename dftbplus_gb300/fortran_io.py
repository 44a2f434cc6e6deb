"""Fortran input/output forms that the reference's files use, restated for the host side.

* ``ListDirected`` is Fortran list-directed input (``read(unit, *)``), which the reference uses for
  every data record of its Slater-Koster files (``type/oldskdata.F90:139-262``) and of its ASCII
  charge restart files (``dftb/sccinit.F90:290-356``).
* ``read_records`` / ``write_records`` are gfortran unformatted sequential files (``charges.bin``,
  ``dftb/sccinit.F90:700-760``): each record is its payload framed by a 4-byte little-endian byte
  count before and after.
"""
from __future__ import annotations

import struct
from typing import Callable, List, Optional, Sequence


def fortran_real(tok: str) -> float:
    """A real constant as list-directed input accepts it (D or E exponent)."""
    return float(tok.replace("D", "E").replace("d", "e"))


def fortran_logical(tok: str) -> bool:
    """A logical value: T/F, .TRUE./.FALSE. or any form whose first letter after an optional period
    is T or F (case-insensitive)."""
    t = tok.lstrip(".").upper()
    if t.startswith("T"):
        return True
    if t.startswith("F"):
        return False
    raise ValueError(f"not a Fortran logical: {tok!r}")


def fortran_int(tok: str) -> int:
    return int(tok)


class ListDirected:
    """Fortran list-directed input over the records (lines) of a file.

    Values are separated by blanks or a comma; ``r*c`` stands for r copies of c and ``r*`` for r null
    values; two commas with nothing between are one null value; a slash ends the read (the items left
    keep their values). One read consumes as many records as it needs and drops the rest of its last
    record; items are converted only when taken, so what follows them in the record may be anything.
    Null values come back as None.
    """

    def __init__(self, lines: Sequence[str], pos: int = 0):
        self.lines = lines
        self.pos = pos

    @staticmethod
    def _tokens(line: str):
        """Raw values of one record in order (None for a null, '/' for a slash)."""
        fields = line.split(",")
        for fi, field in enumerate(fields):
            toks = field.split()
            if not toks:
                # ",," or a leading comma: one null value (a trailing comma adds nothing)
                if fi < len(fields) - 1:
                    yield None
                continue
            for tok in toks:
                if tok.startswith("/"):
                    yield "/"
                    return
                if "*" in tok:
                    r, c = tok.split("*", 1)
                    for _ in range(int(r)):
                        yield c if c else None
                else:
                    yield tok

    def read(self, n: int, conv: Callable[[str], object] = fortran_real) -> List[Optional[object]]:
        """The next n items, each converted with conv (None where null or cut off by a slash)."""
        vals: List[Optional[object]] = []
        while len(vals) < n:
            if self.pos >= len(self.lines):
                raise ValueError("data ended in the middle of a list-directed read")
            line = self.lines[self.pos]
            self.pos += 1
            for tok in self._tokens(line):
                if tok == "/":                  # the remaining items are not read
                    vals.extend([None] * (n - len(vals)))
                    break
                vals.append(None if tok is None else conv(tok))
                if len(vals) == n:
                    break
        return vals

    def read_mixed(self, convs: Sequence[Callable[[str], object]]) -> List[Optional[object]]:
        """One read of len(convs) items of different types (item i converted with convs[i])."""
        raw = self.read(len(convs), conv=lambda t: t)
        return [None if r is None else c(r) for r, c in zip(raw, convs)]


def read_records(data: bytes) -> List[bytes]:
    """Payloads of a gfortran unformatted sequential file."""
    out, pos = [], 0
    while pos < len(data):
        if pos + 4 > len(data):
            raise ValueError("truncated record marker")
        (n,) = struct.unpack_from("<i", data, pos)
        if n < 0 or pos + 8 + n > len(data):
            raise ValueError("bad record length (sub-records or a damaged file)")
        payload = data[pos + 4:pos + 4 + n]
        (n2,) = struct.unpack_from("<i", data, pos + 4 + n)
        if n2 != n:
            raise ValueError("record markers do not match")
        out.append(payload)
        pos += 8 + n
    return out


def write_records(payloads: Sequence[bytes]) -> bytes:
    return b"".join(struct.pack("<i", len(p)) + p + struct.pack("<i", len(p)) for p in payloads)
