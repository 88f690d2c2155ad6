"""Fiat-Shamir transcript of the oracle (test infrastructure only).

Restates, over the oracle's own BLAKE3 (oracle.c: orc_blake3_xof), the two
transcript layers the Ligerito opening draws its randomness from:

* ``Blake3Transcript`` -- src/transcript/mod.rs:18-96 and the framing helper
  src/transcript/traits.rs:371-376 of BitZ-PoC.  The state is the BLAKE3
  hasher over every byte absorbed so far; this restatement keeps those bytes
  and rehashes them on every squeeze, which is slow but transparently equal.
* ``ZincChallenger`` -- src/ligerito_flock.rs:36-126: flock's ``Challenger``
  driven from that transcript (every observation framed by absorb_slice,
  challenges from get_field_challenge::<Gf128>, proof of work over a squeezed
  16-byte seed).

Only tests/, smoke() and the CPU leg of bench.py import this module.
"""
from __future__ import annotations

import struct

import numpy as np

from . import oracle as O

SAMPLING_READ_TAG = b"bitz/sampling-read/v1"


class Blake3Transcript:
    def __init__(self):
        self.buf = bytearray()

    def clone(self) -> "Blake3Transcript":
        t = Blake3Transcript()
        t.buf = bytearray(self.buf)
        return t

    def absorb(self, data: bytes) -> None:
        """absorb_inner (mod.rs:81-95): a plain hasher update."""
        self.buf += bytes(data)

    def absorb_slice(self, data: bytes) -> None:
        """traits.rs:371-376: 0x06 || len as u64 LE || data || 0x07."""
        self.absorb(b"\x06" + struct.pack("<Q", len(data)) + bytes(data) + b"\x07")

    def _xof(self, n: int) -> bytes:
        return O.blake3_xof(bytes(self.buf), n)

    def challenge_bytes(self, n: int) -> bytes:
        """get_challenge (mod.rs:65-80) for an n-byte type with no padding
        bits: squeeze n bytes, then absorb 0x12 || bytes || 0x34."""
        out = self._xof(n)
        self.absorb(b"\x12" + out + b"\x34")
        return out

    def fill_sampling_bytes(self, n: int) -> bytes:
        """mod.rs:58-63."""
        out = self._xof(n)
        self.absorb(SAMPLING_READ_TAG + struct.pack("<Q", n) + out)
        return out

    def state_digest(self) -> bytes:
        """mod.rs:40-42: the 32-byte hash of everything absorbed."""
        return O.blake3(bytes(self.buf))


def gf_bytes(v) -> bytes:
    v = np.asarray(v, dtype=np.uint64).reshape(2)
    return struct.pack("<QQ", int(v[0]), int(v[1]))


def gf_from_bytes(b: bytes) -> np.ndarray:
    lo, hi = struct.unpack("<QQ", b)
    return np.array([lo, hi], dtype=np.uint64)


class ZincChallenger:
    """src/ligerito_flock.rs:36-126."""

    def __init__(self, transcript: Blake3Transcript):
        self.t = transcript

    def observe_label(self, label: bytes) -> None:
        self.t.absorb_slice(label)

    def observe_f128(self, v) -> None:
        self.t.absorb_slice(gf_bytes(v))

    def observe_f128_slice(self, vs) -> None:
        self.t.absorb_slice(b"".join(gf_bytes(v) for v in np.asarray(vs, np.uint64).reshape(-1, 2)))

    def observe_bytes(self, data: bytes) -> None:
        self.t.absorb_slice(data)

    def sample_f128(self) -> np.ndarray:
        return gf_from_bytes(self.t.challenge_bytes(16))

    def sample_f128_vec(self, n: int) -> np.ndarray:
        """challenger.rs:60-62 default: n single draws."""
        return np.array([self.sample_f128() for _ in range(n)], dtype=np.uint64).reshape(n, 2)

    def grind_pow(self, bits: int) -> int:
        """ligerito_flock.rs:70-99,115-122: the seed is one squeezed field
        element (16 bytes, LE words); the nonce is the smallest with
        blake3(seed || nonce_le) having ``bits`` leading zero bits (0 when
        bits == 0); the nonce is then absorbed as an 8-byte slice."""
        seed = gf_bytes(self.sample_f128())
        nonce = 0 if bits == 0 else O.pow_first_nonce(seed, bits)
        assert nonce is not None
        self.t.absorb_slice(struct.pack("<Q", nonce))
        return nonce

    def verify_pow(self, nonce: int, bits: int) -> bool:
        """ligerito_flock.rs:101-113."""
        seed = gf_bytes(self.sample_f128())
        ok = nonce == 0 if bits == 0 else O.pow_ok(seed, nonce, bits)
        self.t.absorb_slice(struct.pack("<Q", nonce))
        return ok
