"""Bit-matrix ingest of the oracle (test infrastructure only).

Restates, with numpy bit operations, BitZ's repack_leaf_bits
(src/ligerito.rs:19-33), pack_columns_from_rows and rows_from_packed_cols
(src/ligerito.rs:655-717; the 64 x 64 bit transpose of :632-651 by its
definition) and the packed message of commit_rs_flock_from_rows
(src/ligerito_flock.rs:198-245).  Layouts: cells (2^(rv+cv), 2) uint64 words
of one u128 per cell, cell (b, c) at row (b << cv) | c; rows (2^cv, W) with
W = ceil(2^rv / 64); packed columns (ceil(2^cv / 64), 2^rv).
"""
from __future__ import annotations

import numpy as np


def repack_leaf_bits(cells: np.ndarray, rv: int, cv: int) -> np.ndarray:
    cells = np.asarray(cells, np.uint64).reshape(1 << rv, 1 << cv, 2)
    if (cells[..., 1] != 0).any() or (cells[..., 0] > 1).any():
        raise ValueError("binary matrix cell")
    bits = cells[..., 0].astype(np.uint8).T                   # [c, b]
    words = max(((1 << rv) + 63) // 64, 1)
    pad = np.zeros((1 << cv, words * 64), np.uint8)
    pad[:, : 1 << rv] = bits
    return np.packbits(pad, axis=1, bitorder="little").view("<u8").reshape(1 << cv, words) \
        .astype(np.uint64)


def _bits(words: np.ndarray) -> np.ndarray:
    """(n, W) uint64 -> (n, 64 W) bits, bit i of row = bit i % 64 of word i // 64."""
    w = np.ascontiguousarray(words, "<u8")
    return np.unpackbits(w.view(np.uint8).reshape(w.shape[0], -1), axis=1, bitorder="little")


def pack_columns_from_rows(rows: np.ndarray, rv: int, cv: int) -> np.ndarray:
    nrows, cols = 1 << rv, 1 << cv
    groups = (cols + 63) // 64
    bits = _bits(rows)[:, :nrows]                             # [c, i]
    full = np.zeros((groups * 64, nrows), np.uint8)
    full[:cols] = bits
    per = full.reshape(groups, 64, nrows).transpose(0, 2, 1)  # [g, i, k]
    return np.packbits(np.ascontiguousarray(per), axis=2, bitorder="little") \
        .view("<u8").reshape(groups, nrows).astype(np.uint64)


def rows_from_packed_cols(packed: np.ndarray, rv: int, cv: int) -> np.ndarray:
    nrows, cols = 1 << rv, 1 << cv
    groups = (cols + 63) // 64
    words = max((nrows + 63) // 64, 1)
    bits = _bits(np.asarray(packed, np.uint64).reshape(groups * nrows, 1))  # [(g, i), k]
    per = bits.reshape(groups, nrows, 64).transpose(0, 2, 1).reshape(groups * 64, nrows)
    pad = np.zeros((groups * 64, words * 64), np.uint8)
    pad[:, :nrows] = per
    out = np.packbits(pad, axis=1, bitorder="little").view("<u8").reshape(groups * 64, words)
    return out[:cols].astype(np.uint64)


def message_from_rows(rows: np.ndarray, rv: int, cv: int) -> np.ndarray:
    """commit_rs_flock_from_rows: {lo: row[2i], hi: row[2i+1]} for
    i < 2^(rv - 7), column after column."""
    assert rv >= 7
    hi_count = 1 << (rv - 7)
    r = np.asarray(rows, np.uint64).reshape(1 << cv, -1)[:, : 2 * hi_count]
    return np.ascontiguousarray(r.reshape(-1, 2))
