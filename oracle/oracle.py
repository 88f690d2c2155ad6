"""ctypes binding of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The GPU library never imports
or links it.  Arrays of GF(2^128) elements are numpy ``uint64`` arrays of shape
``(n, 2)`` holding ``(lo, hi)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_SO), exist_ok=True)
        import platform

        arch = ["-march=armv8-a+crypto"] if platform.machine() in ("aarch64", "arm64") else []
        subprocess.check_call(
            ["gcc", "-O2", "-fPIC", "-pthread", "-std=c11", *arch, "-shared", "-o", _SO, src]
        )
    return _SO


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_S = ctypes.c_size_t
_I = ctypes.c_int
_U64 = ctypes.c_uint64


def _declare(L):
    sig = {
        "orc_clmul_kind": (ctypes.c_char_p, []),
        "orc_gf_mul": (None, [_P, _P, _P]),
        "orc_gf_mul_bitwise": (None, [_P, _P, _P]),
        "orc_gf_inv": (None, [_P, _P]),
        "orc_gf_mul_many": (None, [_P, _P, _P, _S]),
        "orc_ghash_chain": (None, [_P, _P, _S, _P]),
        "orc_ntt_twiddle": (None, [_I, _I, _U64, _P]),
        "orc_ntt_evals": (None, [_I, _P]),
        "orc_ntt_forward_interleaved": (None, [_P, _S, _I, _I, _I]),
        "orc_ntt_forward": (None, [_P, _I]),
        "orc_ntt_forward_interleaved_blocked": (None, [_P, _S, _I, _I, _I]),
        "orc_sha256": (None, [_P, _S, _P]),
        "orc_blake3_hash": (None, [_P, _S, _P]),
        "orc_blake3_xof": (None, [_P, _S, _P, _S]),
        "orc_pow_ok": (_I, [_P, _S, _U64, ctypes.c_uint]),
        "orc_pow_first_nonce": (_U64, [_P, _S, _U64, _U64, ctypes.c_uint]),
        "orc_blake3_leaf_cv": (None, [_P, _S, _P]),
        "orc_blake3_parent_cv": (None, [_P, _P, _P]),
        "orc_blake3_subtree_cv": (None, [_P, _S, _U64, _P]),
        "orc_blake3_rows_subtree_cvs": (None, [_P, _S, _S, _U64, _P]),
        "orc_hash_leaf": (None, [_P, _S, _I, _P]),
        "orc_hash_pair": (None, [_P, _P, _I, _P]),
        "orc_merkle_tree": (None, [_P, _S, _S, _I, _P, _I]),
        "orc_merkle_tree_from_leaves": (None, [_P, _S, _I]),
        "orc_merkle_multi_proof": (_S, [_P, _S, _P, _S, _P]),
        "orc_verify_merkle_multi_proof": (_I, [_P, _S, _P, _P, _S, _P, _S, _I]),
        "orc_commit": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _I]),
        "orc_partial_eval_lsb": (None, [_P, _S, _P, _S, _P]),
        "orc_round_msg_lsb": (None, [_P, _P, _S, _P, _P]),
        "orc_fold_and_msg_lsb": (None, [_P, _P, _S, _P, _P, _P, _P, _P]),
        "orc_build_eq_lsb": (None, [_P, _S, _P]),
        "orc_induce_basis": (None, [_I, _P, _S, _P, _P]),
        "orc_sv_fold": (None, [_P, _S, _P, _P]),
        "orc_phi_from_words": (None, [_P, _S, _P, _P]),
        "orc_chacha_words": (None, [_U64, _U64, _P, _S]),
        "orc_chacha20_block": (None, [_P, ctypes.c_uint32, _P, _P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def clmul_kind() -> str:
    return lib().orc_clmul_kind().decode()


def gf(x) -> np.ndarray:
    """One element from an int (< 2^128) or a (lo, hi) pair."""
    if isinstance(x, (int, np.integer)):
        x = int(x)
        return np.array([x & (2**64 - 1), x >> 64], dtype=np.uint64)
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64).reshape(2))


def gf_int(a) -> int:
    a = np.asarray(a, dtype=np.uint64).reshape(2)
    return int(a[0]) | (int(a[1]) << 64)


def gf_mul(a, b) -> np.ndarray:
    out = np.zeros(2, np.uint64)
    lib().orc_gf_mul(_p(gf(a)), _p(gf(b)), _p(out))
    return out


def gf_mul_bitwise(a, b) -> np.ndarray:
    out = np.zeros(2, np.uint64)
    lib().orc_gf_mul_bitwise(_p(gf(a)), _p(gf(b)), _p(out))
    return out


def gf_inv(a) -> np.ndarray:
    out = np.zeros(2, np.uint64)
    lib().orc_gf_inv(_p(gf(a)), _p(out))
    return out


def gf_mul_many(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, np.uint64)
    b = np.ascontiguousarray(b, np.uint64)
    out = np.zeros_like(a)
    lib().orc_gf_mul_many(_p(a), _p(b), _p(out), a.shape[0])
    return out


def ghash_chain(h, blocks: np.ndarray) -> np.ndarray:
    blocks = np.ascontiguousarray(blocks, np.uint64).reshape(-1, 2)
    out = np.zeros(2, np.uint64)
    lib().orc_ghash_chain(_p(gf(h)), _p(blocks), blocks.shape[0], _p(out))
    return out


def ntt_twiddle(log_domain: int, layer: int, block: int) -> np.ndarray:
    out = np.zeros(2, np.uint64)
    lib().orc_ntt_twiddle(log_domain, layer, block, _p(out))
    return out


def ntt_evals(log_domain: int) -> np.ndarray:
    out = np.zeros((log_domain, log_domain, 2), np.uint64)
    lib().orc_ntt_evals(log_domain, _p(out))
    return out


def ntt_forward_interleaved(data: np.ndarray, num_ntts: int, start_layer: int = 0,
                            n_threads: int = 1) -> np.ndarray:
    d = np.ascontiguousarray(data, np.uint64).copy()
    log_d = (d.shape[0] // num_ntts).bit_length() - 1
    lib().orc_ntt_forward_interleaved(_p(d), num_ntts, log_d, start_layer, n_threads)
    return d


def ntt_forward_interleaved_blocked(data: np.ndarray, num_ntts: int, start_layer: int = 0,
                                    n_threads: int = 1) -> np.ndarray:
    d = np.ascontiguousarray(data, np.uint64).copy()
    log_d = (d.shape[0] // num_ntts).bit_length() - 1
    lib().orc_ntt_forward_interleaved_blocked(_p(d), num_ntts, log_d, start_layer, n_threads)
    return d


def ntt_forward(data: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(data, np.uint64).copy()
    lib().orc_ntt_forward(_p(d), d.shape[0].bit_length() - 1)
    return d


def _bytes_in(b: bytes):
    arr = np.frombuffer(bytes(b), dtype=np.uint8).copy() if len(b) else np.zeros(1, np.uint8)
    return arr


def sha256(data: bytes) -> bytes:
    a = _bytes_in(data)
    out = np.zeros(32, np.uint8)
    lib().orc_sha256(_p(a), len(data), _p(out))
    return out.tobytes()


def blake3(data: bytes) -> bytes:
    a = _bytes_in(data)
    out = np.zeros(32, np.uint8)
    lib().orc_blake3_hash(_p(a), len(data), _p(out))
    return out.tobytes()


def blake3_xof(data: bytes, out_len: int) -> bytes:
    a = _bytes_in(data)
    out = np.zeros(max(out_len, 1), np.uint8)
    lib().orc_blake3_xof(_p(a), len(data), _p(out), out_len)
    return out[:out_len].tobytes()


def pow_ok(prefix: bytes, nonce: int, bits: int) -> bool:
    return bool(lib().orc_pow_ok(_p(_bytes_in(prefix)), len(prefix), nonce, bits))


def pow_first_nonce(prefix: bytes, bits: int, start: int = 0, end: int = 2**64 - 1) -> int | None:
    """Smallest nonce in [start, end) with blake3(prefix || nonce_le) having
    ``bits`` leading zero bits (serial scan); None when there is none."""
    if not 0 < len(prefix) + 8 <= 64:
        raise ValueError("prefix + nonce must fit one 64-byte block")
    n = lib().orc_pow_first_nonce(_p(_bytes_in(prefix)), len(prefix), start, end, bits)
    return None if n == 2**64 - 1 else int(n)


def blake3_leaf_cv(data: bytes) -> bytes:
    a = _bytes_in(data)
    out = np.zeros(32, np.uint8)
    lib().orc_blake3_leaf_cv(_p(a), len(data), _p(out))
    return out.tobytes()


def blake3_subtree_cv(data: bytes, first_chunk: int) -> bytes:
    """Non-root CV of whole 1 KiB chunks that start at chunk `first_chunk` of a
    larger input (a power-of-two run of chunks: one node of that input's tree)."""
    a = _bytes_in(data)
    out = np.zeros(32, np.uint8)
    lib().orc_blake3_subtree_cv(_p(a), len(data), first_chunk, _p(out))
    return out.tobytes()


def rows_subtree_cvs(rows: np.ndarray, first_chunk: int) -> np.ndarray:
    """blake3_subtree_cv of every row of `rows` ((n, row_words, 2) uint64)."""
    rows = np.ascontiguousarray(rows, np.uint64)
    n = rows.shape[0]
    row_len = rows[0].nbytes if n else 0
    out = np.zeros((n, 32), np.uint8)
    lib().orc_blake3_rows_subtree_cvs(_p(rows), n, row_len, first_chunk, _p(out))
    return out


def blake3_parent_cv(l: bytes, r: bytes) -> bytes:
    out = np.zeros(32, np.uint8)
    lib().orc_blake3_parent_cv(_p(_bytes_in(l)), _p(_bytes_in(r)), _p(out))
    return out.tobytes()


SHA256, BLAKE3 = 0, 1


def hash_leaf(data: bytes, kind: int) -> bytes:
    out = np.zeros(32, np.uint8)
    lib().orc_hash_leaf(_p(_bytes_in(data)), len(data), kind, _p(out))
    return out.tobytes()


def hash_pair(l: bytes, r: bytes, kind: int) -> bytes:
    out = np.zeros(32, np.uint8)
    lib().orc_hash_pair(_p(_bytes_in(l)), _p(_bytes_in(r)), kind, _p(out))
    return out.tobytes()


def merkle_tree(data, num_leaves: int, kind: int, n_threads: int = 1) -> np.ndarray:
    d = np.ascontiguousarray(np.frombuffer(data, np.uint8) if isinstance(data, (bytes, bytearray))
                             else np.asarray(data).view(np.uint8).reshape(-1))
    tree = np.zeros((2 * num_leaves - 1, 32), np.uint8)
    lib().orc_merkle_tree(_p(d), d.size, num_leaves, kind, _p(tree), n_threads)
    return tree


def merkle_multi_proof(tree: np.ndarray, num_leaves: int, positions) -> np.ndarray:
    pos = np.ascontiguousarray(np.asarray(positions, np.uint64))
    depth = max(num_leaves.bit_length() - 1, 1)
    out = np.zeros((max(len(pos), 1) * depth, 32), np.uint8)
    n = lib().orc_merkle_multi_proof(_p(np.ascontiguousarray(tree)), num_leaves,
                                     _p(pos) if len(pos) else None, len(pos), _p(out))
    return out[:n].copy()


def verify_merkle_multi_proof(root: bytes, num_leaves: int, positions, leaf_hashes,
                              proof, kind: int) -> bool:
    pos = np.ascontiguousarray(np.asarray(positions, np.uint64))
    lh = np.ascontiguousarray(np.asarray(leaf_hashes, np.uint8).reshape(-1, 32))
    pr = np.ascontiguousarray(np.asarray(proof, np.uint8).reshape(-1, 32))
    r = np.frombuffer(root, np.uint8).copy()
    return bool(lib().orc_verify_merkle_multi_proof(
        _p(r), num_leaves, _p(pos) if len(pos) else None, _p(lh) if len(lh) else None,
        len(pos), _p(pr) if len(pr) else None, len(pr), kind))


def commit(msg: np.ndarray, log_inv_rate: int, log_batch_size: int, hash_kind: int,
           n_threads: int = 1):
    """Returns (codeword (n,2) uint64, tree (2L-1,32) uint8, root bytes)."""
    msg = np.ascontiguousarray(msg, np.uint64).reshape(-1, 2)
    log_msg_len = msg.shape[0].bit_length() - 1
    assert msg.shape[0] == 1 << log_msg_len
    k_code = log_msg_len - log_batch_size + log_inv_rate
    cw = np.zeros((msg.shape[0] << log_inv_rate, 2), np.uint64)
    tree = np.zeros((2 * (1 << k_code) - 1, 32), np.uint8)
    root = np.zeros(32, np.uint8)
    rc = lib().orc_commit(_p(msg), log_msg_len, log_inv_rate, log_batch_size, hash_kind,
                          _p(cw), _p(tree), _p(root), n_threads)
    if rc != 0:
        raise ValueError("bad commit shape")
    return cw, tree, root.tobytes()


def merkle_tree_from_leaves(leaves: np.ndarray, kind: int) -> np.ndarray:
    """Flat tree (2n-1, 32) over n given leaf hashes."""
    leaves = np.asarray(leaves, np.uint8).reshape(-1, 32)
    n = leaves.shape[0]
    tree = np.zeros((2 * n - 1, 32), np.uint8)
    tree[:n] = leaves
    lib().orc_merkle_tree_from_leaves(_p(tree), n, kind)
    return tree


# ---- lane-sharded BLAKE3 commit ---------------------------------------------
# Every lane's NTT is independent (flock-core/src/ntt/additive_ntt_f128.rs:
# 176-191) and a leaf's BLAKE3 CV is a tree over its 1 KiB chunks, each chunk
# being 64 lanes of one position with its index in the leaf as the counter
# (flock-core/src/merkle.rs:160-201).  So rank `rank` of `world` (a power of
# two, L / world >= 64 lanes) encodes lanes [rank L/world, (rank+1) L/world)
# as a commit of its own, and reduces each of its rows to the CV of the aligned
# run of chunks it holds; every leaf CV is then the merge of the world CVs of
# its position.


def lane_shard(msg: np.ndarray, log_batch_size: int, world: int, rank: int) -> np.ndarray:
    """Rank's message shard: msg[col * L + lane] for its lanes, compact."""
    L = 1 << log_batch_size
    Ls = L // world
    m = np.asarray(msg, np.uint64).reshape(-1, L, 2)
    return np.ascontiguousarray(m[:, rank * Ls:(rank + 1) * Ls]).reshape(-1, 2)


def commit_lane_shard(msg_shard: np.ndarray, log_inv_rate: int, log_batch_size: int,
                      world: int, rank: int):
    """(shard codeword (positions x L/world lanes), per-position subtree CVs)."""
    ls = log_batch_size - (world.bit_length() - 1)
    if world & (world - 1) or ls < 6:
        raise ValueError("world must be a power of two leaving >= 64 lanes per rank")
    cw, _, _ = commit(msg_shard, log_inv_rate, ls, BLAKE3)
    rows = cw.reshape(-1, 1 << ls, 2)
    return cw, rows_subtree_cvs(rows, rank * ((1 << ls) // 64))


def merkle_from_shard_cvs(cvs: np.ndarray):
    """Tree and root from the ranks' subtree CVs ((world, positions, 32), rank order)."""
    cvs = np.asarray(cvs, np.uint8)
    level = [cvs[r] for r in range(cvs.shape[0])]
    while len(level) > 1:
        nxt = []
        for i in range(0, len(level), 2):
            a, b = level[i], level[i + 1]
            nxt.append(np.stack([np.frombuffer(blake3_parent_cv(a[p].tobytes(), b[p].tobytes()),
                                               np.uint8) for p in range(a.shape[0])]))
        level = nxt
    tree = merkle_tree_from_leaves(level[0], BLAKE3)
    return tree, tree[-1].tobytes()


def partial_eval_lsb(evals: np.ndarray, rs: np.ndarray) -> np.ndarray:
    e = np.ascontiguousarray(evals, np.uint64).reshape(-1, 2)
    r = np.ascontiguousarray(rs, np.uint64).reshape(-1, 2)
    out = np.zeros((e.shape[0] >> r.shape[0], 2), np.uint64)
    lib().orc_partial_eval_lsb(_p(e), e.shape[0], _p(r), r.shape[0], _p(out))
    return out


def round_msg_lsb(f: np.ndarray, b: np.ndarray):
    f = np.ascontiguousarray(f, np.uint64)
    b = np.ascontiguousarray(b, np.uint64)
    u0 = np.zeros(2, np.uint64)
    u2 = np.zeros(2, np.uint64)
    lib().orc_round_msg_lsb(_p(f), _p(b), f.shape[0], _p(u0), _p(u2))
    return u0, u2


def fold_and_msg_lsb(f: np.ndarray, b: np.ndarray, r):
    f = np.ascontiguousarray(f, np.uint64)
    b = np.ascontiguousarray(b, np.uint64)
    nf = np.zeros((f.shape[0] // 2, 2), np.uint64)
    nb = np.zeros_like(nf)
    u0 = np.zeros(2, np.uint64)
    u2 = np.zeros(2, np.uint64)
    lib().orc_fold_and_msg_lsb(_p(f), _p(b), f.shape[0], _p(gf(r)), _p(nf), _p(nb), _p(u0),
                               _p(u2))
    return nf, nb, u0, u2


def induce_basis(log_n: int, queries, weights) -> np.ndarray:
    """Dense induced basis: sum_i weights[i] * W^_j(queries[i]) for j < 2^log_n."""
    q = np.ascontiguousarray(np.asarray(queries, dtype=np.uint64))
    w = np.ascontiguousarray(np.asarray(weights, dtype=np.uint64).reshape(-1, 2))
    assert w.shape[0] == q.shape[0]
    out = np.zeros((1 << log_n, 2), np.uint64)
    lib().orc_induce_basis(log_n, _p(q) if len(q) else None, len(q), _p(w) if len(q) else None,
                           _p(out))
    return out


def build_eq_lsb(point: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(point, np.uint64).reshape(-1, 2)
    out = np.zeros((1 << p.shape[0], 2), np.uint64)
    lib().orc_build_eq_lsb(_p(p), p.shape[0], _p(out))
    return out


def sv_fold(packed: np.ndarray, eq: np.ndarray) -> np.ndarray:
    packed = np.ascontiguousarray(packed, np.uint64)
    eq = np.ascontiguousarray(eq, np.uint64)
    sv = np.zeros((128, 2), np.uint64)
    lib().orc_sv_fold(_p(packed), packed.shape[0], _p(eq), _p(sv))
    return sv


def phi_from_words(eq_hi: np.ndarray, eq_r2: np.ndarray) -> np.ndarray:
    eq_hi = np.ascontiguousarray(eq_hi, np.uint64)
    eq_r2 = np.ascontiguousarray(eq_r2, np.uint64)
    out = np.zeros_like(eq_hi)
    lib().orc_phi_from_words(_p(eq_hi), eq_hi.shape[0], _p(eq_r2), _p(out))
    return out


def chacha_words(seed: int, n_words: int, first_word: int = 0) -> np.ndarray:
    out = np.zeros((n_words, 2), np.uint64)
    lib().orc_chacha_words(seed, first_word, _p(out), n_words)
    return out


def chacha20_block(key: bytes, counter: int, nonce: bytes) -> bytes:
    k = np.frombuffer(key, np.uint32).copy()
    n = np.frombuffer(nonce, np.uint32).copy()
    out = np.zeros(64, np.uint8)
    lib().orc_chacha20_block(_p(k), counter, _p(n), _p(out))
    return out.tobytes()
