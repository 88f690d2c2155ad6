"""Ligerito opening against a device-resident commitment.

``prove`` runs the whole recursive prover (recursive_prover_with_basis,
flock-core/src/pcs/ligerito.rs:3455-3884) through ``bz_ligerito_prove`` and
returns the LigeritoProof (codec.LigeritoProof).  ``open_l0`` runs the
level-0 part of recursive_prover_with_basis_initial_impl
(flock-core/src/pcs/ligerito.rs:3566-3720) through ``bz_ligerito_open_l0``:
the transcript prefix, the lane folds with their grinding, the level-1
ligero_commit of the folded witness, the query grind, the distinct queries
and alpha_0, and the opened rows with their Merkle multi-proof.  All array
work runs on the GPU; the transcript advances in place on the host.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import BzError, check, lib, ptr
from .pcs import Context, DeviceArray, ProverData, default_context
from .transcript import Blake3Transcript

_U32 = ctypes.c_uint32
_S = ctypes.c_size_t


class L0ConfigC(ctypes.Structure):
    _fields_ = [("initial_k", _U32), ("recursive_k0", _U32), ("log_inv_rate1", _U32),
                ("fold_grinding_bits0", _U32), ("grinding_bits0", _U32), ("queries0", _U32),
                ("hash_kind", _U32), ("ood_samples1", _U32)]


class L0SizesC(ctypes.Structure):
    _fields_ = [("n_sumcheck", _S), ("n_fold_nonces", _S), ("n_queries", _S), ("n_alpha", _S),
                ("row_len", _S), ("n_proof_hashes", _S), ("folded_len", _S),
                ("n_ood_values", _S)]


@dataclass
class L0Config:
    """The ProverConfig fields the level-0 opening reads (ligerito.rs:
    initial_k, recursive_ks[0], log_inv_rates[1], fold_grinding_bits[0],
    grinding_bits[0], queries[0], merkle_hash)."""
    initial_k: int
    recursive_k0: int
    log_inv_rate1: int
    fold_grinding_bits0: int = 0
    grinding_bits0: int = 0
    queries0: int = 8
    hash_kind: int = 1
    ood_samples1: int = 0

    def to_c(self) -> L0ConfigC:
        return L0ConfigC(self.initial_k, self.recursive_k0, self.log_inv_rate1,
                         self.fold_grinding_bits0, self.grinding_bits0, self.queries0,
                         self.hash_kind, self.ood_samples1)


class _RowsOwner:
    """Owns opened rows moved out of a native level-0 opening; freed when the
    last array viewing them is gone."""

    def __init__(self, h):
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().bz_rows_free(self.h)
            self.h = None


class L0Opening:
    """Results of one level-0 opening; owns the level-1 commitment and the
    folded arrays on the device until ``free``."""

    def __init__(self, handle, ctx: Context):
        self.handle = handle
        self.ctx = ctx
        ctx.adopt(self)
        sz = L0SizesC()
        check(ctx.handle, lib().bz_l0_opening_sizes(handle, ctypes.byref(sz)))
        self.sizes = sz
        k = sz.n_sumcheck - 1
        sc = np.zeros((sz.n_sumcheck, 2, 2), np.uint64)
        fn = np.zeros(max(sz.n_fold_nonces, 1), np.uint64)
        ch = np.zeros((max(k, 1), 2), np.uint64)
        root1 = (ctypes.c_uint8 * 32)()
        gn = ctypes.c_uint64()
        qs = np.zeros(max(sz.n_queries, 1), np.uint64)
        al = np.zeros((max(sz.n_alpha, 1), 2), np.uint64)
        proof = np.empty((max(sz.n_proof_hashes, 1), 32), np.uint8)
        check(ctx.handle, lib().bz_l0_opening_copy(handle, ptr(sc), ptr(fn), ptr(ch), root1,
                                                   ctypes.byref(gn), ptr(qs), ptr(al), None,
                                                   ptr(proof)))
        # the opened rows move out of the opening and are viewed in place
        rh = ctypes.c_void_p()
        data = ctypes.POINTER(ctypes.c_uint64)()
        check(ctx.handle, lib().bz_l0_opening_take_rows(handle, ctypes.byref(rh),
                                                        ctypes.byref(data)))
        owner = _RowsOwner(rh)
        words = sz.n_queries * sz.row_len * 2
        if words and not data:
            raise BzError(7, "opened rows missing")
        if words:
            buf = (ctypes.c_uint64 * words).from_address(
                ctypes.cast(data, ctypes.c_void_p).value)
            buf._owner = owner
            rows = np.frombuffer(buf, dtype=np.uint64).reshape(sz.n_queries, sz.row_len, 2)
        else:
            rows = np.zeros((0, sz.row_len, 2), np.uint64)
        self.sumcheck = [(sc[i, 0].copy(), sc[i, 1].copy()) for i in range(sz.n_sumcheck)]
        self.fold_nonces = [int(x) for x in fn[:sz.n_fold_nonces]]
        self.fold_challenges = ch[:k].copy()
        self.root1 = bytes(root1)
        self.grinding_nonce = int(gn.value)
        self.queries = [int(x) for x in qs[:sz.n_queries]]
        self.alpha = al[:sz.n_alpha].copy()
        self.opened_rows = rows
        self.merkle_proof = proof[:sz.n_proof_hashes]
        ov = np.zeros((max(sz.n_ood_values, 1), 2), np.uint64)
        check(ctx.handle, lib().bz_l0_opening_ood_values(handle, ptr(ov)))
        self.ood_values = ov[:sz.n_ood_values].copy()

    def folded(self) -> tuple[int, int, int]:
        """Device pointers of f^1 and the folded basis, and their length."""
        f, b, n = ctypes.c_void_p(), ctypes.c_void_p(), _S()
        check(self.ctx.handle, lib().bz_l0_opening_folded(self.handle, ctypes.byref(f),
                                                          ctypes.byref(b), ctypes.byref(n)))
        return f.value, b.value, n.value

    def folded_host(self) -> tuple[np.ndarray, np.ndarray]:
        f, b, n = self.folded()
        out_f = np.zeros((n, 2), np.uint64)
        out_b = np.zeros((n, 2), np.uint64)
        check(self.ctx.handle, lib().bz_memcpy_d2h(self.ctx.handle, ptr(out_f), f, out_f.nbytes))
        check(self.ctx.handle, lib().bz_memcpy_d2h(self.ctx.handle, ptr(out_b), b, out_b.nbytes))
        return out_f, out_b

    def free(self):
        if self.handle:
            if self.ctx.handle:
                lib().bz_l0_opening_free(self.handle)
            self.handle = None

    release = free

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def open_l0(transcript: Blake3Transcript, data: ProverData, packed: DeviceArray,
            basis: DeviceArray, target, cfg: L0Config, ctx: Context | None = None) -> L0Opening:
    ctx = ctx or data.ctx or default_context()
    t = np.ascontiguousarray(np.asarray(target, dtype=np.uint64).reshape(2))
    c = cfg.to_c()
    h = ctypes.c_void_p()
    check(ctx.handle, lib().bz_ligerito_open_l0(ctx.handle, transcript.handle, data._h(),
                                                packed.ptr, basis.ptr, ptr(t), ctypes.byref(c),
                                                ctypes.byref(h)))
    return L0Opening(h, ctx)


class LigeritoConfigC(ctypes.Structure):
    _fields_ = [("initial_k", _U32), ("recursive_steps", _U32),
                ("recursive_ks", ctypes.POINTER(_U32)), ("log_inv_rates", ctypes.POINTER(_U32)),
                ("queries", ctypes.POINTER(_U32)), ("grinding_bits", ctypes.POINTER(_U32)),
                ("fold_grinding_bits", ctypes.POINTER(_U32)),
                ("ood_samples", ctypes.POINTER(_U32)), ("hash_kind", _U32)]


@dataclass
class LigeritoConfig:
    """ProverConfig (ligerito.rs:124-160): recursive_ks has one entry per
    recursive step, the other lists one more (level 0 first)."""
    initial_k: int
    recursive_ks: list
    log_inv_rates: list
    queries: list
    grinding_bits: list
    fold_grinding_bits: list | None = None
    ood_samples: list | None = None
    hash_kind: int = 1

    def to_c(self):
        r = len(self.recursive_ks)
        keep = []

        def arr(v, n):
            if v is None:
                return None
            if len(v) != n:
                raise ValueError("config list of the wrong length")
            a = (_U32 * n)(*v)
            keep.append(a)
            return ctypes.cast(a, ctypes.POINTER(_U32))

        c = LigeritoConfigC(self.initial_k, r, arr(self.recursive_ks, r),
                            arr(self.log_inv_rates, r + 1), arr(self.queries, r + 1),
                            arr(self.grinding_bits, r + 1), arr(self.fold_grinding_bits, r + 1),
                            arr(self.ood_samples, r + 1), self.hash_kind)
        return c, keep


class ProofHandle:
    """An undecoded bz_ligerito_proof (host memory); ``decode`` converts and frees it."""

    def __init__(self, h):
        self.h = h

    def decode(self):
        from .codec import _decoded

        h, self.h = self.h, None
        return _decoded(h)

    def free(self):
        if self.h:
            lib().bz_ligerito_proof_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def prove(transcript: Blake3Transcript, data: ProverData, packed: DeviceArray,
          basis: DeviceArray, target, cfg: LigeritoConfig, ctx: Context | None = None,
          decode: bool = True):
    """The LigeritoProof of ``target`` against the commitment in ``data``
    (with ``decode=False``, the undecoded ProofHandle)."""

    ctx = ctx or data.ctx or default_context()
    t = np.ascontiguousarray(np.asarray(target, dtype=np.uint64).reshape(2))
    c, keep = cfg.to_c()
    h = ctypes.c_void_p()
    check(ctx.handle, lib().bz_ligerito_prove(ctx.handle, transcript.handle, data._h(),
                                              packed.ptr, basis.ptr, ptr(t), ctypes.byref(c),
                                              ctypes.byref(h)))
    del keep
    ph = ProofHandle(h)
    return ph.decode() if decode else ph
