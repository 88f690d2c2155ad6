"""Proof codec of the oracle (test infrastructure only).

Restates the BitZ proof stream (src/proof_codec.rs:39-161; round-0 and
ring-switch framing, src/binary_pcs.rs:487-525) and the bincode 1.3
fixed-int encoding of flock's serde-derived LigeritoProof
(flock-core/src/pcs/ligerito.rs:1509-1551; write_ligerito / read_ligerito,
binary_pcs.rs:527-544).  bincode 1.3.3 is a third-party crate pinned by the
reference's Cargo.lock and absent here; its published format for these
types is: struct fields in declaration order with no tags, u64 as 8 LE
bytes, Vec<T> as a u64 length then the items, [u8; 32] as 32 raw bytes, and
the two-word Gf128 {lo, hi} as 16 bytes.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

MAX_PROOF_BYTES = 64 << 20  # binary_pcs.rs:63


class CodecError(Exception):
    """src/proof_codec.rs:14-25: kind is 'truncated', 'noncanonical' or 'bincode'."""

    def __init__(self, kind: str):
        super().__init__(kind)
        self.kind = kind


Gf = tuple  # (lo, hi)


@dataclass
class RecursiveProof:
    opened_rows: list = field(default_factory=list)   # list of list of (lo, hi)
    merkle_proof: list = field(default_factory=list)  # list of 32-byte bytes


@dataclass
class FinalProof:
    yr: list = field(default_factory=list)
    opened_rows: list = field(default_factory=list)
    merkle_proof: list = field(default_factory=list)


@dataclass
class LigeritoProof:
    initial_root: bytes = bytes(32)
    initial_proof: RecursiveProof = field(default_factory=RecursiveProof)
    recursive_roots: list = field(default_factory=list)
    recursive_proofs: list = field(default_factory=list)
    final_proof: FinalProof = field(default_factory=FinalProof)
    sumcheck_transcript: list = field(default_factory=list)  # list of ((lo,hi),(lo,hi))
    grinding_nonces: list = field(default_factory=list)
    ood_values: list = field(default_factory=list)
    fold_grinding_nonces: list = field(default_factory=list)


def _u64(v: int) -> bytes:
    return struct.pack("<Q", v)


def _gf(g) -> bytes:
    return struct.pack("<QQ", int(g[0]), int(g[1]))


def _rows(rows) -> bytes:
    out = [_u64(len(rows))]
    for r in rows:
        out.append(_u64(len(r)))
        out.extend(_gf(g) for g in r)
    return b"".join(out)


def _hashes(hs) -> bytes:
    assert all(len(h) == 32 for h in hs)
    return _u64(len(hs)) + b"".join(bytes(h) for h in hs)


def encode_ligerito(p: LigeritoProof) -> bytes:
    """bincode::serialize(&LigeritoProof)."""
    assert len(p.initial_root) == 32
    out = [bytes(p.initial_root), _rows(p.initial_proof.opened_rows),
           _hashes(p.initial_proof.merkle_proof), _hashes(p.recursive_roots),
           _u64(len(p.recursive_proofs))]
    for rp in p.recursive_proofs:
        out += [_rows(rp.opened_rows), _hashes(rp.merkle_proof)]
    out += [_u64(len(p.final_proof.yr)), b"".join(_gf(g) for g in p.final_proof.yr),
            _rows(p.final_proof.opened_rows), _hashes(p.final_proof.merkle_proof),
            _u64(len(p.sumcheck_transcript)),
            b"".join(_gf(a) + _gf(b) for a, b in p.sumcheck_transcript),
            _u64(len(p.grinding_nonces)), b"".join(_u64(n) for n in p.grinding_nonces),
            _u64(len(p.ood_values)), b"".join(_gf(g) for g in p.ood_values),
            _u64(len(p.fold_grinding_nonces)), b"".join(_u64(n) for n in p.fold_grinding_nonces)]
    return b"".join(out)


class _Blob:
    """bincode deserializer state: bounded by the blob, trailing bytes rejected."""

    def __init__(self, b: bytes):
        self.b, self.i = b, 0

    def take(self, n: int) -> bytes:
        if n > len(self.b) - self.i:
            raise CodecError("bincode")
        out = self.b[self.i:self.i + n]
        self.i += n
        return out

    def u64(self) -> int:
        return struct.unpack("<Q", self.take(8))[0]

    def gf(self):
        return struct.unpack("<QQ", self.take(16))

    def rows(self):
        return [[self.gf() for _ in range(self.u64())] for _ in range(self.u64())]

    def hashes(self):
        return [self.take(32) for _ in range(self.u64())]


def decode_ligerito(blob: bytes) -> LigeritoProof:
    d = _Blob(blob)
    p = LigeritoProof()
    p.initial_root = d.take(32)
    p.initial_proof = RecursiveProof(d.rows(), d.hashes())
    p.recursive_roots = d.hashes()
    p.recursive_proofs = [RecursiveProof(d.rows(), d.hashes()) for _ in range(d.u64())]
    yr = [d.gf() for _ in range(d.u64())]
    p.final_proof = FinalProof(yr, d.rows(), d.hashes())
    p.sumcheck_transcript = [(d.gf(), d.gf()) for _ in range(d.u64())]
    p.grinding_nonces = [d.u64() for _ in range(d.u64())]
    p.ood_values = [d.gf() for _ in range(d.u64())]
    p.fold_grinding_nonces = [d.u64() for _ in range(d.u64())]
    if d.i != len(blob):
        raise CodecError("bincode")
    return p


class Writer:
    """src/proof_codec.rs:39-89."""

    def __init__(self):
        self.buf = bytearray()

    def len(self, n: int):
        self.buf += _u64(n)

    def gf(self, g):
        self.buf += _gf(g)

    def bytes(self, b: bytes):
        self.buf += bytes(b)

    def round0(self, y, nonce: int | None):
        """write_round0 (binary_pcs.rs:487-496)."""
        self.gf(y)
        if nonce is None:
            self.len(0)
        else:
            self.len(1)
            self.len(nonce)

    def ring_switch(self, s_v):
        """write_ring_switch (:510-519)."""
        assert len(s_v) == 128
        for g in s_v:
            self.gf(g)

    def ligerito(self, p: LigeritoProof):
        """write_ligerito (:527-531)."""
        blob = encode_ligerito(p)
        self.len(len(blob))
        self.bytes(blob)


class Reader:
    """src/proof_codec.rs:91-161."""

    def __init__(self, buf: bytes):
        self.buf, self.cur = bytes(buf), 0

    def remaining(self) -> int:
        return len(self.buf) - self.cur

    def take(self, n: int) -> bytes:
        if n > self.remaining():
            raise CodecError("truncated")
        out = self.buf[self.cur:self.cur + n]
        self.cur += n
        return out

    def len(self) -> int:
        return struct.unpack("<Q", self.take(8))[0]

    def gf(self):
        return struct.unpack("<QQ", self.take(16))

    def round0(self):
        """read_round0 (:498-508): (y, nonce or None)."""
        y = self.gf()
        tag = self.len()
        if tag == 0:
            return y, None
        if tag == 1:
            return y, self.len()
        raise CodecError("noncanonical")

    def ring_switch(self):
        return [self.gf() for _ in range(128)]

    def ligerito(self) -> LigeritoProof:
        """read_ligerito (:533-544)."""
        n = self.len()
        if n > MAX_PROOF_BYTES or n > self.remaining():
            raise CodecError("truncated")
        return decode_ligerito(self.take(n))
