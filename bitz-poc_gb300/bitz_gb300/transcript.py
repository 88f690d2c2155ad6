"""Fiat-Shamir transcript and proof-of-work grinding over the C ABI.

* ``Blake3Transcript`` mirrors BitZ's transcript (src/transcript/mod.rs:18-96
  with the framing of src/transcript/traits.rs:371-376): a host-side
  incremental BLAKE3 state inside libbitzgpu.so.
* ``ZincChallenger`` mirrors src/ligerito_flock.rs:36-126, flock's
  ``Challenger`` driven from that transcript; ``grind_pow`` searches the
  nonce on the GPU.
* ``pow_first_nonce`` is first_pow_nonce (src/utils/blake3x4.rs:42-69) on the
  GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .pcs import Context, default_context


def _buf(data: bytes):
    data = bytes(data)
    return (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0"), len(data)


class Blake3Transcript:
    def __init__(self, _handle=None):
        if _handle is None:
            h = ctypes.c_void_p()
            check(None, lib().bz_transcript_create(ctypes.byref(h)))
            _handle = h
        self.handle = _handle

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                lib().bz_transcript_destroy(h)
            except Exception:
                pass
            self.handle = None

    def clone(self) -> "Blake3Transcript":
        h = ctypes.c_void_p()
        check(None, lib().bz_transcript_clone(self.handle, ctypes.byref(h)))
        return Blake3Transcript(h)

    def absorb(self, data: bytes) -> None:
        b, n = _buf(data)
        check(None, lib().bz_transcript_absorb(self.handle, b, n))

    def absorb_slice(self, data: bytes) -> None:
        b, n = _buf(data)
        check(None, lib().bz_transcript_absorb_slice(self.handle, b, n))

    def challenge_bytes(self, n: int) -> bytes:
        out = (ctypes.c_uint8 * max(n, 1))()
        check(None, lib().bz_transcript_challenge(self.handle, out, n))
        return bytes(out)[:n]

    def get_field_challenge(self) -> np.ndarray:
        out = np.zeros(2, np.uint64)
        check(None, lib().bz_transcript_sample_f128(self.handle, ptr(out)))
        return out

    def fill_sampling_bytes(self, n: int) -> bytes:
        out = (ctypes.c_uint8 * max(n, 1))()
        check(None, lib().bz_transcript_fill_sampling_bytes(self.handle, out, n))
        return bytes(out)[:n]

    def state_digest(self) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        check(None, lib().bz_transcript_state_digest(self.handle, out))
        return bytes(out)


def blake3_xof(data: bytes, out_len: int) -> bytes:
    b, n = _buf(data)
    out = (ctypes.c_uint8 * max(out_len, 1))()
    check(None, lib().bz_blake3_xof(b, n, out, out_len))
    return bytes(out)[:out_len]


def pow_first_nonce(prefix: bytes, bits: int, start: int = 0, end: int = 2**64 - 1,
                    ctx: Context | None = None) -> int | None:
    """Smallest nonce in [start, end) with blake3(prefix || nonce LE) having
    ``bits`` leading zero bits; None when the range has none."""
    ctx = ctx or default_context()
    b, n = _buf(prefix)
    out = ctypes.c_uint64()
    st = lib().bz_pow_first_nonce(ctx.handle, b, n, bits, start, end, ctypes.byref(out))
    if st == 8:
        return None
    check(ctx.handle, st)
    return int(out.value)


class ZincChallenger:
    def __init__(self, transcript: Blake3Transcript, ctx: Context | None = None):
        self.t = transcript
        self._ctx = ctx  # the GPU context is needed only by grind_pow

    def observe_label(self, label: bytes) -> None:
        self.t.absorb_slice(label)

    def observe_f128(self, v) -> None:
        a = np.ascontiguousarray(np.asarray(v, dtype=np.uint64).reshape(2))
        check(None, lib().bz_transcript_observe_f128(self.t.handle, ptr(a)))

    def observe_f128_slice(self, vs) -> None:
        a = np.ascontiguousarray(np.asarray(vs, dtype=np.uint64).reshape(-1, 2))
        self.t.absorb_slice(a.astype("<u8").tobytes())

    def observe_bytes(self, data: bytes) -> None:
        self.t.absorb_slice(data)

    def sample_f128(self) -> np.ndarray:
        return self.t.get_field_challenge()

    def sample_f128_vec(self, n: int) -> np.ndarray:
        return np.array([self.sample_f128() for _ in range(n)], dtype=np.uint64).reshape(n, 2)

    def grind_pow(self, bits: int) -> int:
        ctx = self._ctx or default_context()
        out = ctypes.c_uint64()
        check(ctx.handle, lib().bz_transcript_grind_pow(ctx.handle, self.t.handle, bits,
                                                        ctypes.byref(out)))
        return int(out.value)

    def verify_pow(self, nonce: int, bits: int) -> bool:
        ok = ctypes.c_int()
        check(None, lib().bz_transcript_verify_pow(self.t.handle, nonce, bits, ctypes.byref(ok)))
        return bool(ok.value)
