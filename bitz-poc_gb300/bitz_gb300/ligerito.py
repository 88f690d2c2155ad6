"""Opening-side device kernels behind the reference's prover interface.

* ``fold_and_msg_lsb`` / ``round_msg_lsb`` / ``partial_eval_lsb`` mirror the
  functions of the same names in flock-core/src/pcs/ligerito.rs
  (:2634-2735, :2500-2537, :1678-1695).
* ``SumcheckProver`` mirrors the reference's stateful prover
  (ligerito.rs:2981-3182): ``new`` sends the first message, ``fold(r)`` folds
  f and the combined basis at the LSB variable and returns the next message,
  ``introduce_new`` / ``glue`` batch a new basis polynomial in.
* ``build_eq_lsb``, ``sv_fold``, ``phi_from_words`` are the ring-switch passes
  of BitZ src/ligerito.rs (:317-427) and src/poly/utils.rs (:46-120).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .pcs import Context, DeviceArray, default_context


def _gf(x) -> np.ndarray:
    if isinstance(x, (int, np.integer)):
        x = int(x)
        return np.array([x & (2**64 - 1), x >> 64], dtype=np.uint64)
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64).reshape(2))


def round_msg_lsb(f: DeviceArray, b: DeviceArray, ctx: Context | None = None):
    ctx = ctx or f.ctx
    u0 = np.zeros(2, np.uint64)
    u2 = np.zeros(2, np.uint64)
    check(ctx.handle, lib().bz_round_msg_lsb(ctx.handle, f.ptr, b.ptr, f.n, ptr(u0), ptr(u2)))
    return u0, u2


def fold_and_msg_lsb(f: DeviceArray, b: DeviceArray, r, ctx: Context | None = None):
    """Returns (folded f, folded b, (u0, u2))."""
    ctx = ctx or f.ctx
    if f.n != b.n:
        raise ValueError("f and b lengths differ")
    nf = DeviceArray(f.n // 2, ctx)
    nb = DeviceArray(f.n // 2, ctx)
    u0 = np.zeros(2, np.uint64)
    u2 = np.zeros(2, np.uint64)
    check(ctx.handle, lib().bz_fold_and_msg_lsb(ctx.handle, f.ptr, b.ptr, f.n, ptr(_gf(r)),
                                                nf.ptr, nb.ptr, ptr(u0), ptr(u2)))
    return nf, nb, (u0, u2)


def fold_gate_check(f: DeviceArray, b: DeviceArray, r, mode: int, limit_ns: int = 0,
                    ctx: Context | None = None):
    """The armed fold that the prover uses for its small rounds, driven by
    hand (bz_fold_gate_check): mode 0 posts r and returns (folded f, folded b,
    (u0, u2)) like fold_and_msg_lsb; mode 1 cancels the round; mode 2 posts
    nothing and raises BzError(BZ_ERR_TIMEOUT) once the kernel's bounded wait
    has run out."""
    ctx = ctx or f.ctx
    if f.n != b.n:
        raise ValueError("f and b lengths differ")
    nf = DeviceArray(f.n // 2, ctx)
    nb = DeviceArray(f.n // 2, ctx)
    u0 = np.zeros(2, np.uint64)
    u2 = np.zeros(2, np.uint64)
    check(ctx.handle, lib().bz_fold_gate_check(ctx.handle, f.ptr, b.ptr, f.n, ptr(_gf(r)),
                                               nf.ptr, nb.ptr, mode, limit_ns, ptr(u0),
                                               ptr(u2)))
    return nf, nb, (u0, u2)


def partial_eval_lsb(evals: DeviceArray, rs, ctx: Context | None = None) -> DeviceArray:
    ctx = ctx or evals.ctx
    r = np.ascontiguousarray(np.asarray(rs, dtype=np.uint64).reshape(-1, 2))
    k = r.shape[0]
    out = DeviceArray(evals.n >> k, ctx)
    check(ctx.handle, lib().bz_partial_eval_lsb(ctx.handle, evals.ptr, evals.n,
                                                ptr(r) if k else None, k, out.ptr))
    return out


class SumcheckProver:
    """Device-resident mirror of flock-core's SumcheckProver (single combined
    basis; ligerito.rs:2981-3182)."""

    def __init__(self, f: DeviceArray, b1: DeviceArray, h1):
        if f.n != b1.n:
            raise ValueError("f and b1 lengths differ")
        self.f = f
        self.combined_basis = b1
        self.t_r = _gf(h1)
        self.transcript = []
        self.pending_glue = None

    @classmethod
    def new(cls, f: DeviceArray, b1: DeviceArray, h1):
        inst = cls(f, b1, h1)
        msg = round_msg_lsb(f, b1)
        inst.transcript.append(msg)
        return inst, msg

    def fold(self, r):
        nf, nb, msg = fold_and_msg_lsb(self.f, self.combined_basis, r)
        self.f, self.combined_basis = nf, nb
        self.transcript.append(msg)
        return msg

    def introduce_new(self, b_new: DeviceArray, h_new):
        if b_new.n != self.f.n:
            raise ValueError("basis length mismatch")
        msg = round_msg_lsb(self.f, b_new)
        self.transcript.append(msg)
        self.pending_glue = (b_new, _gf(h_new))
        return msg


def build_eq_lsb(point, ctx: Context | None = None) -> DeviceArray:
    ctx = ctx or default_context()
    p = np.ascontiguousarray(np.asarray(point, dtype=np.uint64).reshape(-1, 2))
    out = DeviceArray(1 << p.shape[0], ctx)
    check(ctx.handle, lib().bz_build_eq_lsb(ctx.handle, ptr(p) if p.shape[0] else None,
                                            p.shape[0], out.ptr))
    return out


def sv_fold(packed: DeviceArray, eq: DeviceArray, ctx: Context | None = None) -> np.ndarray:
    ctx = ctx or packed.ctx
    sv = np.zeros((128, 2), np.uint64)
    check(ctx.handle, lib().bz_sv_fold(ctx.handle, packed.ptr, eq.ptr, packed.n, ptr(sv)))
    return sv


def phi_from_words(eq_hi: DeviceArray, eq_r2: np.ndarray, ctx: Context | None = None) -> DeviceArray:
    ctx = ctx or eq_hi.ctx
    r2 = np.ascontiguousarray(np.asarray(eq_r2, dtype=np.uint64).reshape(128, 2))
    out = DeviceArray(eq_hi.n, ctx)
    check(ctx.handle, lib().bz_phi_from_words(ctx.handle, eq_hi.ptr, eq_hi.n, ptr(r2), out.ptr))
    return out
