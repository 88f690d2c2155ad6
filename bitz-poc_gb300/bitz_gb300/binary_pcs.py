"""BitZ's BinaryPcs commit / open interface over the C ABI.

Mirrors src/binary_pcs.rs: ``commit`` (:313-318), ``prove_round0``
(:320-325), ``open_basis`` (:341-367) and ``open_bit_mle`` (:413-431), with
the BitMleOpening's stream encoding (``BitMleOpening::write``, :546-551).
The packed witness and every table stay on the device; the transcript is
the caller's Blake3Transcript, advanced in place.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import codec
from ._lib import check, lib, ptr
from .opening import LigeritoConfig
from .pcs import LOG_PACKING, Context, DeviceArray, PcsParams, ProverData, commit, default_context
from .transcript import Blake3Transcript


class Round0Prover:
    """The prover's round-0 claim: point (zeta^(2^i)), y and the nonce."""

    def __init__(self, handle, ctx: Context):
        self.handle = handle
        self.ctx = ctx
        y = np.zeros(2, np.uint64)
        has, nonce, vars_ = ctypes.c_int(), ctypes.c_uint64(), ctypes.c_uint32()
        check(ctx.handle, lib().bz_round0_get(handle, ptr(y), ctypes.byref(has),
                                              ctypes.byref(nonce), ctypes.byref(vars_)))
        self.y = y
        self.nonce = int(nonce.value) if has.value else None
        pt = np.zeros((max(vars_.value, 1), 2), np.uint64)
        check(ctx.handle, lib().bz_round0_point(handle, ptr(pt)))
        self.point = pt[:vars_.value].copy()

    def write(self, w: codec.Writer):
        """write_round0 (src/binary_pcs.rs:487-496)."""
        w.round0(self.y, self.nonce)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                lib().bz_round0_free(h)
            except Exception:
                pass
            self.handle = None


@dataclass
class BitMleOpening:
    s_v: np.ndarray                 # the ring switch's 128 partial evaluations
    lig: codec.LigeritoProof

    def write(self, w: codec.Writer):
        w.ring_switch(self.s_v)
        w.ligerito(self.lig)

    def to_bytes(self) -> bytes:
        w = codec.Writer()
        self.write(w)
        return w.into_bytes()


class BinaryPcs:
    """``packed_log`` packed variables, committed at rate 2^-log_inv_rate with
    2^initial_k interleaved lanes; ``config`` is the Ligerito ProverConfig and
    ``ood_grinding_bits`` the round-0 difficulty."""

    def __init__(self, packed_log: int, config: LigeritoConfig, ood_grinding_bits: int = 0,
                 ctx: Context | None = None):
        self.packed_log = packed_log
        self.config = config
        self.ood_grinding_bits = ood_grinding_bits
        self.ctx = ctx or default_context()
        self.params = PcsParams(packed_log + LOG_PACKING, config.log_inv_rates[0],
                                config.initial_k, config.hash_kind)

    def commit(self, packed):
        return commit(packed, self.params, self.ctx)

    def prove_round0(self, t: Blake3Transcript, packed: DeviceArray) -> Round0Prover:
        h = ctypes.c_void_p()
        check(self.ctx.handle, lib().bz_pcs_prove_round0(self.ctx.handle, t.handle, packed.ptr,
                                                         packed.n, self.ood_grinding_bits,
                                                         ctypes.byref(h)))
        return Round0Prover(h, self.ctx)

    def open_basis(self, t: Blake3Transcript, packed: DeviceArray, data: ProverData,
                   round0: Round0Prover, basis: DeviceArray, target) -> codec.LigeritoProof:
        """``basis`` (a device array of the witness's length) is updated in
        place with the round-0 term."""
        tg = np.ascontiguousarray(np.asarray(target, dtype=np.uint64).reshape(2))
        c, keep = self.config.to_c()
        h = ctypes.c_void_p()
        check(self.ctx.handle, lib().bz_pcs_open_basis(self.ctx.handle, t.handle, data._h(),
                                                       packed.ptr, round0.handle, basis.ptr,
                                                       ptr(tg), ctypes.byref(c), ctypes.byref(h)))
        del keep
        return codec._decoded(h)

    def open_bit_mle(self, t: Blake3Transcript, packed: DeviceArray, data: ProverData,
                     round0: Round0Prover, point) -> BitMleOpening:
        pt = np.ascontiguousarray(np.asarray(point, dtype=np.uint64).reshape(-1, 2))
        s_v = np.zeros((128, 2), np.uint64)
        c, keep = self.config.to_c()
        h = ctypes.c_void_p()
        check(self.ctx.handle, lib().bz_pcs_open_bit_mle(self.ctx.handle, t.handle, data._h(),
                                                         packed.ptr, round0.handle, ptr(pt),
                                                         pt.shape[0], ctypes.byref(c), ptr(s_v),
                                                         ctypes.byref(h)))
        del keep
        return BitMleOpening(s_v, codec._decoded(h))
