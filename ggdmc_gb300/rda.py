"""Reader for R's binary serialisation format (``.rda`` / ``.RData``, XDR, v2/v3).

ggdmc users keep fitted ``posterior`` objects, data-model instances (DMIs) and
priors in ``.rda`` files written by ``save()``; the reference's own test
fixtures (``tests/testthat/Group1/data/lba_data{0..6}.rda``) are in this
format.  This module decodes them into plain Python objects without R:

* atomic vectors -> ``RVector`` (a numpy array plus its R attributes),
* lists -> ``RList`` (a Python list plus attributes, names on ``.names``),
* S4 objects -> ``RS4`` (slots in ``.slots``, class in ``.cls``),
* pairlists -> ``dict`` (tag -> value), symbols -> ``RSymbol``.

Arrays stay column-major as R stores them; ``RVector.array()`` reshapes by the
``dim`` attribute with ``order="F"``.

The format is R's documented ``serialize()`` stream ("R Internals", section
1.8 "Serialization Formats"): a flags word per item (type in the low 8 bits,
object bit 8, attribute bit 9, tag bit 10, GP levels in bits 12..27), reference
back-links for symbols/environments, and big-endian XDR scalars.
"""

from __future__ import annotations

import gzip
import bz2
import lzma
import struct
from dataclasses import dataclass, field
from typing import Any

import numpy as np

# SEXP type codes (R Internals 1.1.1) and serialisation pseudo-types.
NILSXP, SYMSXP, LISTSXP, CLOSXP, ENVSXP, PROMSXP, LANGSXP = 0, 1, 2, 3, 4, 5, 6
SPECIALSXP, BUILTINSXP, CHARSXP, LGLSXP, INTSXP, REALSXP = 7, 8, 9, 10, 13, 14
CPLXSXP, STRSXP, DOTSXP, VECSXP, EXPRSXP, BCODESXP = 15, 16, 17, 19, 20, 21
EXTPTRSXP, WEAKREFSXP, RAWSXP, S4SXP = 22, 23, 24, 25
REFSXP, NILVALUE_SXP, GLOBALENV_SXP, UNBOUNDVALUE_SXP = 255, 254, 253, 252
MISSINGARG_SXP, BASENAMESPACE_SXP, NAMESPACESXP, PACKAGESXP = 251, 250, 249, 248
PERSISTSXP, EMPTYENV_SXP, BASEENV_SXP, ATTRLANGSXP, ATTRLISTSXP = 247, 242, 241, 240, 239
ALTREP_SXP = 238

NA_INTEGER = -(2**31)


@dataclass
class RSymbol:
    name: str


@dataclass
class RVector:
    """An R atomic vector: ``data`` is a numpy array (or list of str/None)."""
    data: Any
    attrs: dict = field(default_factory=dict)

    @property
    def names(self):
        n = self.attrs.get("names")
        return None if n is None else list(n.data)

    def array(self):
        dim = self.attrs.get("dim")
        arr = np.asarray(self.data)
        if dim is None:
            return arr
        return arr.reshape(tuple(int(d) for d in dim.data), order="F")

    def named(self) -> dict:
        return dict(zip(self.names, list(self.data)))


@dataclass
class RList:
    items: list
    attrs: dict = field(default_factory=dict)

    @property
    def names(self):
        n = self.attrs.get("names")
        return None if n is None else list(n.data)

    def __getitem__(self, key):
        if isinstance(key, str):
            return self.items[self.names.index(key)]
        return self.items[key]

    def __len__(self):
        return len(self.items)


@dataclass
class RS4:
    cls: str
    slots: dict

    def __getitem__(self, key):
        return self.slots[key]


@dataclass
class REnv:
    frame: dict = field(default_factory=dict)


class _Reader:
    def __init__(self, buf: bytes):
        self.buf = buf
        self.pos = 0
        self.refs: list = []

    def _int(self) -> int:
        v = struct.unpack_from(">i", self.buf, self.pos)[0]
        self.pos += 4
        return v

    def _length(self) -> int:
        n = self._int()
        if n == -1:
            hi, lo = self._int(), self._int()
            n = (hi << 32) + (lo & 0xFFFFFFFF)
        return n

    def _bytes(self, n: int) -> bytes:
        b = self.buf[self.pos:self.pos + n]
        self.pos += n
        return b

    def _charsxp(self):
        n = self._int()
        if n == -1:
            return None
        return self._bytes(n).decode("utf-8", errors="replace")

    def _strvec_plain(self):
        # InStringVec: a leading 0 then a length and CHARSXP items
        self._int()
        n = self._int()
        return [self.item() for _ in range(n)]

    def _attrs(self, has_attr: bool) -> dict:
        if not has_attr:
            return {}
        a = self.item()
        return a if isinstance(a, dict) else {}

    def item(self):
        flags = self._int()
        t = flags & 0xFF
        has_attr = bool(flags & (1 << 9))
        has_tag = bool(flags & (1 << 10))

        if t == NILVALUE_SXP or t == NILSXP:
            return None
        if t in (GLOBALENV_SXP, EMPTYENV_SXP, BASEENV_SXP, BASENAMESPACE_SXP,
                 UNBOUNDVALUE_SXP, MISSINGARG_SXP):
            return REnv()
        if t == REFSXP:
            idx = flags >> 8
            if idx == 0:
                idx = self._int()
            return self.refs[idx - 1]
        if t in (NAMESPACESXP, PACKAGESXP, PERSISTSXP):
            v = self._strvec_plain()
            self.refs.append(REnv())
            return self.refs[-1]
        if t == SYMSXP:
            name = self.item()  # a CHARSXP
            sym = RSymbol(name if isinstance(name, str) else str(name))
            self.refs.append(sym)
            return sym
        if t == ENVSXP:
            env = REnv()
            self.refs.append(env)
            self._int()  # locked
            self.item()  # enclos
            frame = self.item()
            hashtab = self.item()
            attr = self.item()
            if isinstance(frame, dict):
                env.frame.update(frame)
            if isinstance(hashtab, RList):
                for b in hashtab.items:
                    if isinstance(b, dict):
                        env.frame.update(b)
            return env
        if t in (LISTSXP, LANGSXP, CLOSXP, PROMSXP, DOTSXP, ATTRLANGSXP, ATTRLISTSXP):
            out: dict = {}
            unnamed = 0
            while True:
                if flags & (1 << 9):
                    self.item()  # attributes of the cons cell (ignored)
                tag = self.item() if flags & (1 << 10) else None
                car = self.item()
                if isinstance(tag, RSymbol):
                    key = tag.name
                else:
                    key = f"..{unnamed}"
                    unnamed += 1
                out[key] = car
                # The CDR follows as another item; keep walking while it is a
                # pairlist cell so long lists do not recurse.
                flags = self._int()
                t = flags & 0xFF
                if t in (LISTSXP, LANGSXP, ATTRLISTSXP, ATTRLANGSXP):
                    continue
                if t in (NILVALUE_SXP, NILSXP):
                    break
                # Any other terminator: rewind and read it as an item.
                self.pos -= 4
                self.item()
                break
            return out
        if t in (SPECIALSXP, BUILTINSXP):
            n = self._int()
            return RSymbol(self._bytes(n).decode())
        if t == CHARSXP:
            if flags & 0xFFFF0000 and False:
                pass
            return self._charsxp()
        if t in (LGLSXP, INTSXP):
            n = self._length()
            arr = np.frombuffer(self._bytes(4 * n), dtype=">i4").astype(np.int64)
            if t == LGLSXP:
                data = np.where(arr == NA_INTEGER, -1, arr).astype(np.int8)
            else:
                data = arr
            return RVector(data, self._attrs(has_attr))
        if t == REALSXP:
            n = self._length()
            arr = np.frombuffer(self._bytes(8 * n), dtype=">f8").astype(np.float64)
            return RVector(arr, self._attrs(has_attr))
        if t == CPLXSXP:
            n = self._length()
            arr = np.frombuffer(self._bytes(16 * n), dtype=">f8").astype(np.float64)
            return RVector(arr[0::2] + 1j * arr[1::2], self._attrs(has_attr))
        if t == RAWSXP:
            n = self._length()
            return RVector(np.frombuffer(self._bytes(n), dtype=np.uint8).copy(),
                           self._attrs(has_attr))
        if t == STRSXP:
            n = self._length()
            data = [self.item() for _ in range(n)]
            return RVector(data, self._attrs(has_attr))
        if t in (VECSXP, EXPRSXP):
            n = self._length()
            items = [self.item() for _ in range(n)]
            return RList(items, self._attrs(has_attr))
        if t == S4SXP:
            attrs = self._attrs(has_attr)
            cls = attrs.pop("class", None)
            cname = cls.data[0] if isinstance(cls, RVector) else str(cls)
            return RS4(cname, attrs)
        if t == EXTPTRSXP:
            self.refs.append(None)
            self.item()
            self.item()
            self._attrs(has_attr)
            return None
        if t == WEAKREFSXP:
            self.refs.append(None)
            self._attrs(has_attr)
            return None
        if t == ALTREP_SXP:
            info = self.item()
            state = self.item()
            attr = self.item()
            attrs = attr if isinstance(attr, dict) else {}
            return self._altrep(info, state, attrs)
        if t == BCODESXP:
            raise NotImplementedError("byte-code objects are not supported")
        raise ValueError(f"unsupported SEXP type {t} at offset {self.pos}")

    def _altrep(self, info, state, attrs):
        cls = None
        if isinstance(info, dict):
            first = list(info.values())[0]
            cls = first.name if isinstance(first, RSymbol) else None
        if cls == "compact_intseq":
            n, start, step = (state.data if isinstance(state, RVector) else state)[:3]
            data = (int(start) + int(step) * np.arange(int(n))).astype(np.int64)
            return RVector(data, attrs)
        if cls == "compact_realseq":
            n, start, step = state.data[:3]
            return RVector(float(start) + float(step) * np.arange(int(n)), attrs)
        if cls and cls.startswith("wrap_"):
            inner = state.items[0] if isinstance(state, RList) else state
            if isinstance(inner, RVector):
                merged = dict(inner.attrs)
                merged.update(attrs)
                return RVector(inner.data, merged)
            return inner
        if cls == "deferred_string":
            arg = list(state.values())[0] if isinstance(state, dict) else state
            vals = arg.data if isinstance(arg, RVector) else []
            return RVector([str(int(v)) if float(v).is_integer() else repr(float(v))
                            for v in vals], attrs)
        raise ValueError(f"unsupported ALTREP class {cls}")


def _decompress(raw: bytes) -> bytes:
    if raw[:2] == b"\x1f\x8b":
        return gzip.decompress(raw)
    if raw[:3] == b"BZh":
        return bz2.decompress(raw)
    if raw[:6] == b"\xfd7zXZ\x00":
        return lzma.decompress(raw)
    return raw


def load_rda(path: str) -> dict:
    """Load every object ``save()`` wrote to ``path``; returns name -> object."""
    with open(path, "rb") as fh:
        buf = _decompress(fh.read())
    if buf[:5] not in (b"RDX2\n", b"RDX3\n"):
        raise ValueError("not an R save() file (missing RDX2/RDX3 magic)")
    if buf[5:7] != b"X\n":
        raise ValueError("only the XDR (big-endian) serialisation is supported")
    r = _Reader(buf[7:])
    version = r._int()
    r._int()  # writer R version
    r._int()  # minimal reader version
    if version == 3:
        nelen = r._int()
        r._bytes(nelen)  # native encoding name
    top = r.item()
    if not isinstance(top, dict):
        raise ValueError("top-level object of a save() file must be a pairlist")
    return top
