"""Bit-matrix ingest on the GPU (BitZ src/ligerito.rs:19-33, 655-717;
src/ligerito_flock.rs:198-245): ``repack_leaf_bits``,
``pack_columns_from_rows``, ``rows_from_packed_cols`` and ``commit_rows``
(commit_rs_flock_from_rows), over device buffers of uint64 words."""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib
from .pcs import Commitment, Context, PcsParams, ProverData, default_context


class DeviceWords:
    """n uint64 words in device memory."""

    def __init__(self, n: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.n = int(n)
        p = ctypes.c_void_p()
        check(self.ctx.handle, lib().bz_device_alloc(self.ctx.handle, max(self.n, 1) * 8,
                                                     ctypes.byref(p)))
        self.ptr = p
        self.ctx.adopt(self)

    @classmethod
    def from_host(cls, a: np.ndarray, ctx: Context | None = None) -> "DeviceWords":
        a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1)
        d = cls(a.size, ctx)
        check(d.ctx.handle, lib().bz_memcpy_h2d(d.ctx.handle, d.ptr,
                                                a.ctypes.data_as(ctypes.c_void_p), a.nbytes))
        return d

    def to_host(self) -> np.ndarray:
        out = np.zeros(self.n, np.uint64)
        check(self.ctx.handle, lib().bz_memcpy_d2h(self.ctx.handle,
                                                   out.ctypes.data_as(ctypes.c_void_p), self.ptr,
                                                   out.nbytes))
        return out

    def free(self):
        if self.ptr:
            if self.ctx.handle:
                lib().bz_device_free(self.ctx.handle, self.ptr)
            self.ptr = None

    release = free

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def row_words(rv: int) -> int:
    return max(((1 << rv) + 63) // 64, 1)


def repack_leaf_bits(cells: DeviceWords, rv: int, cv: int) -> DeviceWords:
    ctx = cells.ctx
    rows = DeviceWords((1 << cv) * row_words(rv), ctx)
    check(ctx.handle, lib().bz_repack_leaf_bits(ctx.handle, cells.ptr, rv, cv, rows.ptr))
    return rows


def pack_columns_from_rows(rows: DeviceWords, rv: int, cv: int) -> DeviceWords:
    ctx = rows.ctx
    out = DeviceWords((((1 << cv) + 63) // 64) * (1 << rv), ctx)
    check(ctx.handle, lib().bz_pack_columns_from_rows(ctx.handle, rows.ptr, rv, cv, out.ptr))
    return out


def rows_from_packed_cols(packed: DeviceWords, rv: int, cv: int) -> DeviceWords:
    ctx = packed.ctx
    rows = DeviceWords((1 << cv) * row_words(rv), ctx)
    check(ctx.handle, lib().bz_rows_from_packed_cols(ctx.handle, packed.ptr, rv, cv, rows.ptr))
    return rows


def commit_rows(rows: DeviceWords, rv: int, cv: int, log_inv_rate: int, log_batch: int,
                hash_kind: int = 1):
    """commit_rs_flock_from_rows: (Commitment, ProverData) of the packed
    message the rows form (2^(rv - 7 + cv) elements)."""
    ctx = rows.ctx
    h = ctypes.c_void_p()
    root = (ctypes.c_uint8 * 32)()
    check(ctx.handle, lib().bz_commit_rows(ctx.handle, rows.ptr, rv, cv, log_inv_rate, log_batch,
                                           hash_kind, ctypes.byref(h), root))
    m_p = rv - 7 + cv
    params = PcsParams(m_p + 7, log_inv_rate, log_batch, hash_kind)
    return Commitment(bytes(root), params), ProverData(h, params, ctx)
