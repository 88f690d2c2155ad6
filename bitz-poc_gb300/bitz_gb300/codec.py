"""Proof types and codec over the C ABI.

Mirrors flock's proof types (flock-core/src/pcs/ligerito.rs:1509-1551:
``RecursiveProof``, ``FinalProof``, ``LigeritoProof``) and BitZ's proof
stream (src/proof_codec.rs ``Writer`` / ``Reader``; ``write_round0`` /
``read_round0``, ``write_ring_switch``, ``write_ligerito`` /
``read_ligerito`` in src/binary_pcs.rs:487-557).  Encoding and decoding run
in libbitzgpu.so (csrc/codec.cpp).  Field elements are (lo, hi) uint64
pairs; hashes are 32-byte rows of uint8.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from ._lib import BzError, check, lib

_S = ctypes.c_size_t
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U8P = ctypes.POINTER(ctypes.c_uint8)


class RowsView(ctypes.Structure):
    _fields_ = [("n_rows", _S), ("row_lens", ctypes.POINTER(_S)), ("data", _U64P)]


class LevelView(ctypes.Structure):
    _fields_ = [("rows", RowsView), ("n_hashes", _S), ("hashes", _U8P)]


class ProofView(ctypes.Structure):
    _fields_ = [("initial_root", ctypes.c_uint8 * 32), ("initial_proof", LevelView),
                ("n_recursive_roots", _S), ("recursive_roots", _U8P),
                ("n_recursive_proofs", _S), ("recursive_proofs", ctypes.POINTER(LevelView)),
                ("n_yr", _S), ("yr", _U64P), ("final_rows", LevelView),
                ("n_sumcheck", _S), ("sumcheck", _U64P),
                ("n_grinding_nonces", _S), ("grinding_nonces", _U64P),
                ("n_ood_values", _S), ("ood_values", _U64P),
                ("n_fold_grinding_nonces", _S), ("fold_grinding_nonces", _U64P)]


def _gfs(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64).reshape(-1, 2))


def _hs(a) -> np.ndarray:
    if isinstance(a, (list, tuple)):
        a = [np.frombuffer(bytes(h), np.uint8) for h in a]
        a = np.stack(a) if a else np.zeros((0, 32), np.uint8)
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint8).reshape(-1, 32))


@dataclass
class RecursiveProof:
    # (len, 2) uint64 arrays: a list, or one (rows, len, 2) array when decoded
    opened_rows: list = field(default_factory=list)
    merkle_proof: np.ndarray = field(default_factory=lambda: np.zeros((0, 32), np.uint8))


@dataclass
class FinalProof:
    yr: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.uint64))
    opened_rows: list = field(default_factory=list)
    merkle_proof: np.ndarray = field(default_factory=lambda: np.zeros((0, 32), np.uint8))


@dataclass
class LigeritoProof:
    initial_root: bytes = bytes(32)
    initial_proof: RecursiveProof = field(default_factory=RecursiveProof)
    recursive_roots: np.ndarray = field(default_factory=lambda: np.zeros((0, 32), np.uint8))
    recursive_proofs: list = field(default_factory=list)
    final_proof: FinalProof = field(default_factory=FinalProof)
    sumcheck_transcript: np.ndarray = field(
        default_factory=lambda: np.zeros((0, 2, 2), np.uint64))   # (n, [u_0, u_2], [lo, hi])
    grinding_nonces: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))
    ood_values: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.uint64))
    fold_grinding_nonces: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))


class _Keep:
    """Holds the numpy buffers a view points into."""

    def __init__(self):
        self.items = []

    def arr(self, a, ctype):
        a = np.ascontiguousarray(a)
        self.items.append(a)
        return a.ctypes.data_as(ctypes.POINTER(ctype)) if a.size else None


def _rows_view(keep: _Keep, rows) -> RowsView:
    if isinstance(rows, np.ndarray) and rows.ndim == 3:
        data = np.ascontiguousarray(rows, dtype=np.uint64).reshape(-1, 2)
        lens = np.full(rows.shape[0], rows.shape[1], dtype=np.uintp)
        return RowsView(rows.shape[0], keep.arr(lens, _S), keep.arr(data, ctypes.c_uint64))
    rows = [_gfs(r) for r in rows]
    lens = np.array([r.shape[0] for r in rows], dtype=np.uintp)
    data = np.concatenate(rows) if rows else np.zeros((0, 2), np.uint64)
    return RowsView(len(rows), keep.arr(lens, _S), keep.arr(data, ctypes.c_uint64))


def _level_view(keep: _Keep, rows, hashes) -> LevelView:
    h = _hs(hashes)
    return LevelView(_rows_view(keep, rows), h.shape[0], keep.arr(h, ctypes.c_uint8))


def _view(p: LigeritoProof):
    keep = _Keep()
    v = ProofView()
    ctypes.memmove(v.initial_root, bytes(p.initial_root), 32)
    v.initial_proof = _level_view(keep, p.initial_proof.opened_rows, p.initial_proof.merkle_proof)
    rr = _hs(p.recursive_roots)
    v.n_recursive_roots, v.recursive_roots = rr.shape[0], keep.arr(rr, ctypes.c_uint8)
    levels = (LevelView * max(len(p.recursive_proofs), 1))()
    for i, rp in enumerate(p.recursive_proofs):
        levels[i] = _level_view(keep, rp.opened_rows, rp.merkle_proof)
    keep.items.append(levels)
    v.n_recursive_proofs = len(p.recursive_proofs)
    v.recursive_proofs = ctypes.cast(levels, ctypes.POINTER(LevelView))
    yr = _gfs(p.final_proof.yr)
    v.n_yr, v.yr = yr.shape[0], keep.arr(yr, ctypes.c_uint64)
    v.final_rows = _level_view(keep, p.final_proof.opened_rows, p.final_proof.merkle_proof)
    sc = np.ascontiguousarray(np.asarray(p.sumcheck_transcript, np.uint64).reshape(-1, 4))
    v.n_sumcheck, v.sumcheck = sc.shape[0], keep.arr(sc, ctypes.c_uint64)
    for name in ("grinding_nonces", "fold_grinding_nonces"):
        a = np.ascontiguousarray(np.asarray(getattr(p, name), np.uint64).reshape(-1))
        setattr(v, "n_" + name, a.shape[0])
        setattr(v, name, keep.arr(a, ctypes.c_uint64))
    ov = _gfs(p.ood_values)
    v.n_ood_values, v.ood_values = ov.shape[0], keep.arr(ov, ctypes.c_uint64)
    return v, keep


class _ProofOwner:
    """Owns a native LigeritoProof whose opened rows decoded arrays view in
    place: the proof is freed when the last such array is gone."""

    def __init__(self, h):
        self.h = h

    def __del__(self):
        if self.h:
            try:
                lib().bz_ligerito_proof_free(self.h)
            except Exception:  # interpreter shutdown: the process frees it
                pass
            self.h = None


def _rows_from(rv: RowsView, owner: _ProofOwner | None = None):
    """Opened rows, each a (lanes, 2) array: views into the native proof when
    an owner keeps it alive (no copy of the rows), copies otherwise.  Rows of
    one length (every opening's) come as a single (rows, lanes, 2) array,
    which indexes and iterates row by row like the list it stands for."""
    if not rv.n_rows:
        return []
    lens = np.ctypeslib.as_array(rv.row_lens, shape=(rv.n_rows,)).astype(np.int64)
    total = int(lens.sum())
    if not total:
        return [np.zeros((0, 2), np.uint64) for _ in range(rv.n_rows)]
    if owner is None:
        flat = np.ctypeslib.as_array(rv.data, shape=(2 * total,)).copy()
    else:
        buf = (ctypes.c_uint64 * (2 * total)).from_address(
            ctypes.cast(rv.data, ctypes.c_void_p).value)
        buf._owner = owner
        flat = np.frombuffer(buf, dtype=np.uint64)
    if (lens == lens[0]).all():
        return flat.reshape(rv.n_rows, int(lens[0]), 2)
    return np.split(flat.reshape(total, 2), np.cumsum(lens)[:-1])


def _hashes_from(n, ptr) -> np.ndarray:
    if not n:
        return np.zeros((0, 32), np.uint8)
    return np.ctypeslib.as_array(ptr, shape=(n * 32,)).reshape(n, 32).copy()


def _words_from(n, ptr, per) -> np.ndarray:
    if not n:
        return np.zeros((0,) if per == 1 else (0, per), np.uint64)
    a = np.ctypeslib.as_array(ptr, shape=(n * per,)).copy()
    return a if per == 1 else a.reshape(n, per)


def _from_view(v: ProofView, owner: _ProofOwner | None = None) -> LigeritoProof:
    p = LigeritoProof()
    p.initial_root = bytes(v.initial_root)
    p.initial_proof = RecursiveProof(_rows_from(v.initial_proof.rows, owner),
                                     _hashes_from(v.initial_proof.n_hashes, v.initial_proof.hashes))
    p.recursive_roots = _hashes_from(v.n_recursive_roots, v.recursive_roots)
    p.recursive_proofs = [RecursiveProof(_rows_from(v.recursive_proofs[i].rows),
                                         _hashes_from(v.recursive_proofs[i].n_hashes,
                                                      v.recursive_proofs[i].hashes))
                          for i in range(v.n_recursive_proofs)]
    p.final_proof = FinalProof(_words_from(v.n_yr, v.yr, 2), _rows_from(v.final_rows.rows),
                               _hashes_from(v.final_rows.n_hashes, v.final_rows.hashes))
    p.sumcheck_transcript = _words_from(v.n_sumcheck, v.sumcheck, 4).reshape(-1, 2, 2)
    p.grinding_nonces = _words_from(v.n_grinding_nonces, v.grinding_nonces, 1)
    p.ood_values = _words_from(v.n_ood_values, v.ood_values, 2)
    p.fold_grinding_nonces = _words_from(v.n_fold_grinding_nonces, v.fold_grinding_nonces, 1)
    return p


def encode_ligerito(p: LigeritoProof) -> bytes:
    """bincode::serialize(&LigeritoProof)."""
    v, keep = _view(p)
    n = _S()
    check(None, lib().bz_ligerito_proof_encode(ctypes.byref(v), None, 0, ctypes.byref(n)))
    out = (ctypes.c_uint8 * max(n.value, 1))()
    check(None, lib().bz_ligerito_proof_encode(ctypes.byref(v), out, n.value, ctypes.byref(n)))
    del keep
    return bytes(out)[:n.value]


def _decoded(h) -> LigeritoProof:
    """Decode a native proof handle; the level-0 opened rows (the bulk of
    the proof) stay in the native proof, which the returned arrays keep
    alive."""
    owner = _ProofOwner(h)
    v = ProofView()
    check(None, lib().bz_ligerito_proof_view_of(h, ctypes.byref(v)))
    return _from_view(v, owner)


def decode_ligerito(blob: bytes) -> LigeritoProof:
    """bincode fixint decode bounded by the blob, trailing bytes rejected."""
    b = (ctypes.c_uint8 * max(len(blob), 1)).from_buffer_copy(bytes(blob) or b"\0")
    h = ctypes.c_void_p()
    check(None, lib().bz_ligerito_proof_decode(b, len(blob), ctypes.byref(h)))
    return _decoded(h)


class Writer:
    """src/proof_codec.rs:39-89 plus the framing helpers of binary_pcs.rs."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(None, lib().bz_writer_create(ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().bz_writer_destroy(self.h)
            self.h = None

    def len(self, n: int):
        check(None, lib().bz_writer_len(self.h, n))

    def gf(self, g):
        check(None, lib().bz_writer_gf(self.h, _gfs(g).ctypes.data_as(ctypes.c_void_p)))

    def bytes(self, b: bytes):
        buf = (ctypes.c_uint8 * max(len(b), 1)).from_buffer_copy(bytes(b) or b"\0")
        check(None, lib().bz_writer_bytes(self.h, buf, len(b)))

    def round0(self, y, nonce: int | None):
        check(None, lib().bz_write_round0(self.h, _gfs(y).ctypes.data_as(ctypes.c_void_p),
                                          0 if nonce is None else 1, nonce or 0))

    def ring_switch(self, s_v):
        a = _gfs(s_v)
        if a.shape[0] != 128:
            raise ValueError("ring switch sends 128 partial evaluations")
        check(None, lib().bz_write_ring_switch(self.h, a.ctypes.data_as(ctypes.c_void_p)))

    def ligerito(self, p: LigeritoProof):
        v, keep = _view(p)
        check(None, lib().bz_write_ligerito(self.h, ctypes.byref(v)))
        del keep

    def into_bytes(self) -> bytes:
        d, n = ctypes.POINTER(ctypes.c_uint8)(), _S()
        check(None, lib().bz_writer_data(self.h, ctypes.byref(d), ctypes.byref(n)))
        return ctypes.string_at(d, n.value) if n.value else b""


class Reader:
    """src/proof_codec.rs:91-161; raises BzError (status 9 truncated, 10
    non-canonical, 11 bincode) where the reference returns CodecError."""

    def __init__(self, buf: bytes):
        self._buf = (ctypes.c_uint8 * max(len(buf), 1)).from_buffer_copy(bytes(buf) or b"\0")
        h = ctypes.c_void_p()
        check(None, lib().bz_reader_create(self._buf, len(buf), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().bz_reader_destroy(self.h)
            self.h = None

    def remaining(self) -> int:
        return int(lib().bz_reader_remaining(self.h))

    def len(self) -> int:
        n = ctypes.c_uint64()
        check(None, lib().bz_reader_len(self.h, ctypes.byref(n)))
        return int(n.value)

    def gf(self):
        g = np.zeros(2, np.uint64)
        check(None, lib().bz_reader_gf(self.h, g.ctypes.data_as(ctypes.c_void_p)))
        return g

    def take(self, n: int) -> bytes:
        d = ctypes.POINTER(ctypes.c_uint8)()
        check(None, lib().bz_reader_take(self.h, n, ctypes.byref(d)))
        return ctypes.string_at(d, n) if n else b""

    def round0(self):
        y = np.zeros(2, np.uint64)
        has, nonce = ctypes.c_int(), ctypes.c_uint64()
        check(None, lib().bz_read_round0(self.h, y.ctypes.data_as(ctypes.c_void_p),
                                         ctypes.byref(has), ctypes.byref(nonce)))
        return y, (int(nonce.value) if has.value else None)

    def ring_switch(self) -> np.ndarray:
        s = np.zeros((128, 2), np.uint64)
        check(None, lib().bz_read_ring_switch(self.h, s.ctypes.data_as(ctypes.c_void_p)))
        return s

    def ligerito(self) -> LigeritoProof:
        h = ctypes.c_void_p()
        check(None, lib().bz_read_ligerito(self.h, ctypes.byref(h)))
        return _decoded(h)


__all__ = ["BzError", "FinalProof", "LigeritoProof", "Reader", "RecursiveProof", "Writer",
           "decode_ligerito", "encode_ligerito"]
