"""Bitvector.BV for the GPU (lib/bitvector.mli:4-116).

phylocaml's BV8/16/32/64 hold one character per 8/16/32/64-bit element in
a C custom block (lib/bitvector/bv.h:57-63) and compute fitch_median_2 and
distance with scalar loops (lib/bitvector/bv.c:46-55, 148-160).  Here a
vector is packed lanes of ``lane_bits`` bits in uint32 words; the median
and the distance run as GPU kernels through the C ABI.  ``BV4`` (4-bit
lanes, eight DNA sites per word) has no reference counterpart; ``BV64``
keeps each 64-bit element as two words, low word first.

Functions keep the reference's names and argument meaning:
``fitch_median_2 s t -> (median, added cost)``, ``distance s t -> int``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .synth import pack_lanes, unpack_lanes

_code_counter = [0]


def _next_code() -> int:
    # bv_next_code (lib/bitvector/bv.c:25-27): a unique code per vector
    c = _code_counter[0]
    _code_counter[0] += 1
    return c


@dataclass
class Vector:
    words: np.ndarray        # uint32 packed lanes
    chars: int               # number of characters (cardinal)
    width: int               # maximum number of bits set per element (create w n)
    lane_bits: int
    code: int = field(default_factory=_next_code)


class BV:
    """One element width of the Bitvector.BV signature."""

    def __init__(self, lane_bits: int, ctx: _native.Context | None = None):
        if lane_bits not in (4, 8, 16, 32, 64):
            raise ValueError("lane_bits must be 4, 8, 16, 32 or 64")
        self.lane_bits = lane_bits
        self.max_width = lane_bits
        self._ctx = ctx

    @property
    def ctx(self) -> _native.Context:
        return self._ctx or _native.default_context()

    # -- creation (bitvector.mli:17-26) --
    def create(self, width: int, n: int) -> Vector:
        if width > self.max_width:
            raise ValueError("width above max_width")
        nw = (n * self.lane_bits + 31) // 32
        return Vector(np.zeros(nw, np.uint32), n, width, self.lane_bits)

    def copy(self, v: Vector) -> Vector:
        return Vector(v.words.copy(), v.chars, v.width, v.lane_bits)

    def of_array(self, width: int, elts) -> Vector:
        a = np.asarray(elts, dtype=np.uint64)
        if self.lane_bits < 64 and (a >> np.uint64(self.lane_bits)).any():
            raise ValueError("element does not fit the lane width")
        w = pack_lanes((a if self.lane_bits == 64 else a.astype(np.uint32))[None, :], self.lane_bits)[0]
        return Vector(w, len(a), width, self.lane_bits)

    # -- accessors (bitvector.mli:29-50) --
    def code(self, v: Vector) -> int:
        return v.code

    def cardinal(self, v: Vector) -> int:
        return v.chars

    def width(self, v: Vector) -> int:
        return v.width

    def get_elt(self, v: Vector, i: int) -> int:
        return int(unpack_lanes(v.words[None, :], v.chars, self.lane_bits)[0, i])

    def set_elt(self, v: Vector, i: int, x: int) -> None:
        if self.lane_bits == 64:
            v.words[2 * i] = np.uint32(x & 0xFFFFFFFF)
            v.words[2 * i + 1] = np.uint32((x >> 32) & 0xFFFFFFFF)
            return
        per = 32 // self.lane_bits
        mask = 0xFFFFFFFF if self.lane_bits == 32 else (1 << self.lane_bits) - 1
        sh = (i % per) * self.lane_bits
        w = int(v.words[i // per])
        v.words[i // per] = np.uint32((w & ~(mask << sh) & 0xFFFFFFFF) | ((x & mask) << sh))

    def elt_states(self, v: Vector, i: int) -> list[int]:
        x = self.get_elt(v, i)
        return [j for j in range(self.lane_bits) if (x >> j) & 1]

    def to_array(self, v: Vector) -> np.ndarray:
        return unpack_lanes(v.words[None, :], v.chars, self.lane_bits)[0]

    def compare(self, a: Vector, b: Vector) -> int:
        # bv_compare (lib/bitvector/bv.c:71-90): by size, then first difference
        if a.chars != b.chars:
            return 1 if a.chars > b.chars else -1
        x, y = self.to_array(a), self.to_array(b)
        d = np.nonzero(x != y)[0]
        if len(d) == 0:
            return 0
        return 1 if x[d[0]] > y[d[0]] else -1

    # -- phylogenetic operations (bitvector.mli:88-94), on the GPU --
    def _pair(self, a: Vector, b: Vector) -> None:
        if a.chars != b.chars or a.lane_bits != b.lane_bits:
            raise ValueError("vectors differ in length or lane width")

    def fitch_median_2(self, a: Vector, b: Vector) -> tuple[Vector, int]:
        self._pair(a, b)
        out = np.zeros_like(a.words)   # the call writes only the sites' bytes
        cnt = C.c_uint64(0)
        self.ctx.call("pgpu_fitch_median2", _native.ptr(a.words), _native.ptr(b.words),
                      _native.ptr(out), a.chars, self.lane_bits, C.byref(cnt))
        return Vector(out, a.chars, a.width, self.lane_bits), int(cnt.value)

    def distance(self, a: Vector, b: Vector) -> int:
        self._pair(a, b)
        cnt = C.c_uint64(0)
        self.ctx.call("pgpu_fitch_distance", _native.ptr(a.words), _native.ptr(b.words),
                      a.chars, self.lane_bits, C.byref(cnt))
        return int(cnt.value)


BV4 = BV(4)
BV8 = BV(8)
BV16 = BV(16)
BV32 = BV(32)
BV64 = BV(64)
