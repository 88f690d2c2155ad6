"""BitZ BinaryPcs opening of the oracle (test infrastructure only).

Restates, over the oracle's field, hash and Ligerito prover:

* prove_round0 (src/binary_pcs.rs:320-325; prove_ood_round_packed,
  src/ligerito_flock.rs:1520-1557, with the header of :1488-1496, ood_point
  :1424-1434, ood_eval :1456-1486 split at 2^12-element blocks, and
  absorb_ood_value src/ligerito.rs:69-73), including the typed grinding
  boundary of src/piop/spartan/grinding.rs:139-172, 264-268;
* ring_switch_prove_with (src/ligerito.rs:445-496) with absorb_sv (:248-250)
  and transpose_bits_128 (:108-120);
* open_basis (src/binary_pcs.rs:341-367) with add_ood_basis
  (src/ligerito_flock.rs:1590-1650);
* open_bit_mle (src/binary_pcs.rs:413-431).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

from . import oracle as O
from .ligerito import LigeritoConfig, prove
from .transcript import Blake3Transcript, ZincChallenger, gf_bytes, gf_from_bytes

OOD_ROUND_DOMAIN = b"bitz/core/ood-round/v1"
OOD_GRINDING_DOMAIN = b"bitz/core/ood-round-grinding/v1"
GRINDING_FRAME = b"bitz/spartan/fiat-shamir-grinding/v1"
GRINDING_NONCE_FRAME = b"bitz/spartan/fiat-shamir-grinding/nonce/v1"
OOD_BLOCK_LOG = 12
LOG_PACKING = 7


@dataclass
class Round0:
    point: np.ndarray  # (vars, 2)
    y: np.ndarray
    nonce: int | None


def _gf_slice(tag: int, vals) -> bytes:
    return bytes([tag]) + b"".join(gf_bytes(v) for v in np.asarray(vals, np.uint64).reshape(-1, 2))


def grind_and_absorb_in_domain(t: Blake3Transcript, domain: bytes, index: int, bits: int) -> int:
    assert 1 <= bits <= 256
    t.absorb_slice(GRINDING_FRAME)
    t.absorb_slice(domain)
    t.absorb_slice(struct.pack("<Q", index))
    t.absorb_slice(struct.pack("<I", bits))
    seed = t.challenge_bytes(32)
    nonce = O.pow_first_nonce(seed, bits)
    assert nonce is not None
    t.absorb_slice(GRINDING_NONCE_FRAME)
    t.absorb_slice(struct.pack("<Q", nonce))
    return nonce


def ood_point(zeta, vars_: int) -> np.ndarray:
    out, cur = [], np.asarray(zeta, np.uint64)
    for _ in range(vars_):
        out.append(cur)
        cur = O.gf_mul(cur, cur)
    return np.array(out, dtype=np.uint64).reshape(vars_, 2)


def _split_eq(point, scalar=None):
    vars_ = point.shape[0]
    lo = min(vars_, OOD_BLOCK_LOG)
    tail = O.build_eq_lsb(point[:lo])
    head = O.build_eq_lsb(point[lo:])
    if scalar is not None:
        head = O.gf_mul_many(np.tile(np.asarray(scalar, np.uint64), (head.shape[0], 1)), head)
    return lo, tail, head


def ood_eval(packed: np.ndarray, point: np.ndarray) -> np.ndarray:
    """MLE[P](point): sum over 2^12-element blocks of head[h] * <block, tail>."""
    lo, tail, head = _split_eq(point)
    blocks = packed.reshape(head.shape[0], 1 << lo, 2)
    acc = np.zeros(2, np.uint64)
    for h in range(head.shape[0]):
        inner = np.bitwise_xor.reduce(O.gf_mul_many(np.ascontiguousarray(blocks[h]), tail), axis=0)
        acc ^= O.gf_mul(inner, head[h])
    return acc


def prove_round0(t: Blake3Transcript, packed: np.ndarray, grinding_bits: int) -> Round0:
    vars_ = packed.shape[0].bit_length() - 1
    t.absorb_slice(OOD_ROUND_DOMAIN)
    t.absorb_slice(struct.pack("<Q", vars_))
    t.absorb_slice(struct.pack("<I", grinding_bits))
    nonce = None
    if grinding_bits:
        nonce = grind_and_absorb_in_domain(t, OOD_GRINDING_DOMAIN, 0, grinding_bits)
    zeta = gf_from_bytes(t.challenge_bytes(16))
    point = ood_point(zeta, vars_)
    y = ood_eval(packed, point)
    t.absorb_slice(_gf_slice(0x50, [y]))
    return Round0(point, y, nonce)


def transpose_bits_128(s: np.ndarray) -> np.ndarray:
    bits = np.unpackbits(np.ascontiguousarray(s, "<u8").view(np.uint8).reshape(128, 16),
                         axis=1, bitorder="little")          # bits[v, u]
    t = np.ascontiguousarray(bits.T)                          # t[u, v]
    return np.packbits(t, axis=1, bitorder="little").view("<u8").reshape(128, 2).astype(np.uint64)


def ring_switch_prove(t: Blake3Transcript, packed: np.ndarray, r_hi: np.ndarray):
    """(s_v, B, beta0)."""
    eq_hi = O.build_eq_lsb(r_hi)
    s = O.sv_fold(packed, eq_hi)
    t.absorb_slice(_gf_slice(0x20, s))
    r2 = np.array([gf_from_bytes(t.challenge_bytes(16)) for _ in range(LOG_PACKING)])
    eq_r2 = O.build_eq_lsb(r2)
    s_u = transpose_bits_128(s)
    beta0 = np.bitwise_xor.reduce(O.gf_mul_many(s_u, eq_r2), axis=0)
    b = O.phi_from_words(eq_hi, eq_r2)
    return s, b, beta0


def open_basis(t: Blake3Transcript, cfg: LigeritoConfig, packed, codeword, tree, root,
               round0: Round0, basis: np.ndarray, target):
    eta = gf_from_bytes(t.challenge_bytes(16))
    lo, tail, head = _split_eq(round0.point, eta)
    add = O.gf_mul_many(np.repeat(head, 1 << lo, axis=0), np.tile(tail, (head.shape[0], 1)))
    basis = basis ^ add
    target = np.asarray(target, np.uint64) ^ O.gf_mul(eta, round0.y)
    return prove(ZincChallenger(t), cfg, packed, basis, target, codeword, tree, root)


def open_bit_mle(t: Blake3Transcript, cfg: LigeritoConfig, packed, codeword, tree, root,
                 round0: Round0, point):
    point = np.asarray(point, np.uint64).reshape(-1, 2)
    assert point.shape[0] == packed.shape[0].bit_length() - 1 + LOG_PACKING
    s_v, b, target = ring_switch_prove(t, packed, point[LOG_PACKING:])
    return s_v, open_basis(t, cfg, packed, codeword, tree, root, round0, b, target)
