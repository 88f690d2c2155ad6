"""CPU restatement of BitZ's batched grand-product GKR prover and verifier
(test infrastructure only: the checker for the GPU prover, never a product
path).

Follows src/bitz/gkr.rs of the reference:
  * ``batched_eval``        GrandProductCircuit::batched_eval (gkr.rs:93-108):
                            layer k+1 = first half x second half of layer k,
                            until ``groups`` roots remain;
  * ``prove``               gpgkr_prove (gkr.rs:113-125) over prove_layer /
                            prove_dense_rounds (gkr.rs:127-282) with the
                            column-free weights (s = 0, Weighing::Off): the
                            round sums of kernels.rs:80-113 (round_sums) and
                            the deferred fold of kernels.rs:146-186, 312-348
                            (fused_fold_round, fold v0 + rho (v1 - v0));
  * ``verify``              gpgkr_verify / verify_layer (gkr.rs:297-348);
  * ``eq_factor``           src/bitz/mod.rs:328-331;
  * ``forest_leaves``       the leaf grid of src/bitz/forest_tests.rs:42-68
                            (leaf (row, column) = image[row] where the
                            column's bit of the row is set, else 1).

The reference's transcript is the third-party ``spongefish`` crate 0.7.4
(not vendored with the reference).  These functions take the transcript as
two callables instead: ``send(stage, [a, b])`` absorbs a prover message and
``challenge(stage)`` returns the next challenge, stage ``ROUND`` for
Stage::GkrRound and ``CLOSE`` for Stage::GkrClose; ``HashChallenges`` below
is a deterministic stand-in used by the tests.  Field elements are (2,)
uint64 arrays (lo, hi) in GF(2^128) with the GHASH polynomial; addition is
XOR and subtraction equals addition.
"""
from __future__ import annotations

import hashlib

import numpy as np

from . import oracle as O

ROUND, CLOSE = 0, 1
ONE = np.array([1, 0], np.uint64)
ZERO = np.array([0, 0], np.uint64)


def _mul(a, b):
    return O.gf_mul(a, b)


def _mul_many(a, b):
    return O.gf_mul_many(np.ascontiguousarray(a, np.uint64), np.ascontiguousarray(b, np.uint64))


def _is_zero(a) -> bool:
    return int(a[0]) == 0 and int(a[1]) == 0


def eq_factor(r, z):
    """eq(r, z) = r z + (1 - r)(1 - z)."""
    return _mul(r, z) ^ _mul(ONE ^ r, ONE ^ z)


def eq_table(point: list) -> np.ndarray:
    """eq(., point) over the hypercube, index bit j <-> point[j] (the
    reference's build_eq_x_r_vec); [1] for the empty point."""
    if not point:
        return ONE.reshape(1, 2).copy()
    return O.build_eq_lsb(np.array(point, np.uint64).reshape(-1, 2))


def batched_eval(leaves: np.ndarray, groups: int):
    """(roots, witnesses leaves-first).  The leaves are padded with ones to a
    power of two as GrandProductCircuit::new does."""
    v = np.ascontiguousarray(leaves, np.uint64).reshape(-1, 2)
    n = v.shape[0]
    if n and n & (n - 1):
        pad = np.tile(ONE, ((1 << n.bit_length()) - n, 1))
        v = np.concatenate([v, pad])
    witnesses = []
    while v.shape[0] > groups:
        mid = v.shape[0] // 2
        nxt = _mul_many(v[:mid], v[mid:])
        witnesses.append(v)
        v = nxt
    return v, witnesses


def mle(values: np.ndarray, point: list) -> np.ndarray:
    """Little-endian multilinear evaluation (adjacent entries differ in the
    first coordinate), forest_tests.rs:28-40."""
    v = np.ascontiguousarray(values, np.uint64).reshape(-1, 2).copy()
    assert v.shape[0] == 1 << len(point)
    for r in point:
        lo, hi = v[0::2], v[1::2]
        v = lo ^ _mul_many(hi ^ lo, np.tile(r, (lo.shape[0], 1)))
    return v[0]


def _fold_halves(v: np.ndarray, rho) -> np.ndarray:
    half = v.shape[0] // 2
    lo, hi = v[:half], v[half:]
    return lo ^ _mul_many(hi ^ lo, np.tile(rho, (half, 1)))


def _round_sums(l_lo, l_hi, r_lo, r_hi, w, send_one):
    """(sum_c w l_end r_end, sum_c w (l_hi - l_lo)(r_hi - r_lo))."""
    le, re = (l_hi, r_hi) if send_one else (l_lo, r_lo)
    end = _mul_many(_mul_many(w, le), re)
    inf = _mul_many(_mul_many(w, l_hi ^ l_lo), r_hi ^ r_lo)
    return np.bitwise_xor.reduce(end, axis=0), np.bitwise_xor.reduce(inf, axis=0)


def prove_layer(send, challenge, point: list, wnext: np.ndarray):
    """One layer (MSB-first ``point`` of k coordinates, ``wnext`` of 2^(k+1)
    entries): k rounds then the close.  Returns (next MSB-first point,
    claim)."""
    mid = wnext.shape[0] // 2
    left, right = wnext[:mid].copy(), wnext[mid:].copy()
    external = list(reversed(point))
    total = len(point)
    factor = ONE.copy()
    next_point = []
    pending = None
    for rnd, z in enumerate(point):
        remaining = total - 1 - rnd
        h = 1 << remaining
        if pending is not None:
            # the previous round's fold (deferred into this pass in the reference)
            left = _fold_halves(left, pending)
            right = _fold_halves(right, pending)
        assert left.shape[0] == 2 * h
        w = eq_table(external[:remaining])
        se, si = _round_sums(left[:h], left[h:], right[:h], right[h:], w, _is_zero(z))
        send(ROUND, [_mul(factor, se), _mul(factor, si)])
        r = challenge(ROUND)
        next_point.append(r)
        pending = r
        factor = _mul(factor, eq_factor(r, z))
    if pending is not None:
        left = _fold_halves(left, pending)
        right = _fold_halves(right, pending)
    l0, r0 = left[0], right[0]
    send(CLOSE, [l0, r0])
    rc = challenge(CLOSE)
    claim = l0 ^ _mul(rc, r0 ^ l0)
    return [rc] + next_point, claim


def prove(send, challenge, point: list, witnesses: list):
    """gpgkr_prove: from a claim at the little-endian ``point`` on the roots
    down to (little-endian leaf point, claimed leaf MLE value)."""
    p = list(reversed(point))
    claim = ZERO.copy()
    for wnext in reversed(witnesses):
        p, claim = prove_layer(send, challenge, p, np.ascontiguousarray(wnext, np.uint64))
    return list(reversed(p)), claim


def verify(recv, challenge, claim, point: list, rounds: int):
    """gpgkr_verify: ``recv(stage)`` returns the next prover message (two
    elements).  Returns (little-endian point, claim) or None when a check
    fails."""
    p = list(reversed(point))
    for _ in range(rounds):
        prefix = ONE.copy()
        nxt = []
        for z in p:
            se, si = recv(ROUND)
            if _is_zero(z):
                s0, s1 = claim, se
            else:
                s0 = se
                s1 = _mul(claim ^ _mul(ONE ^ z, se), O.gf_inv(z))
            r = challenge(ROUND)
            nxt.append(r)
            f = eq_factor(r, z)
            bracket = (s1 ^ s0) ^ _mul(r ^ ONE, si)
            claim = _mul(f, s0 ^ _mul(r, bracket))
            prefix = _mul(prefix, f)
        el, er = recv(CLOSE)
        if gf_key(_mul(_mul(prefix, el), er)) != gf_key(claim):
            return None
        rc = challenge(CLOSE)
        claim = el ^ _mul(rc, er ^ el)
        p = [rc] + nxt
    return list(reversed(p)), claim


def gf_key(a) -> tuple:
    return int(a[0]), int(a[1])


def forest_leaves(packed: np.ndarray, images: np.ndarray, t: int, s: int) -> np.ndarray:
    """Leaf (row, column) at row * 2^s + column: images[row] where bit
    (column mod 64) of packed[column // 64][row] is set, else 1."""
    rows, cols = 1 << t, 1 << s
    packed = np.asarray(packed, np.uint64).reshape(-1, rows)
    images = np.asarray(images, np.uint64).reshape(rows, 2)
    col = np.arange(cols)
    bits = (packed[col // 64, :].T >> (col % 64).astype(np.uint64)) & np.uint64(1)  # (rows, cols)
    out = np.tile(ONE, (rows * cols, 1))
    sel = bits.reshape(-1).astype(bool)
    out[sel] = np.repeat(images, cols, axis=0)[sel]
    return out


class HashChallenges:
    """A deterministic transcript stand-in: every message is hashed into a
    running SHA-256 state and challenges are its digests.  Records every
    message so prover and verifier runs can be compared byte for byte."""

    def __init__(self, seed: bytes = b"gkr"):
        self.h = hashlib.sha256(seed)
        self.messages: list[tuple[int, bytes]] = []
        self._read = 0

    def send(self, stage: int, msg):
        b = b"".join(np.asarray(m, np.uint64).astype("<u8").tobytes() for m in msg)
        self.messages.append((stage, b))
        self.h.update(bytes([stage]) + b)

    def recv(self, stage: int):
        st, b = self.messages[self._read]
        self._read += 1
        assert st == stage
        self.h.update(bytes([stage]) + b)
        w = np.frombuffer(b, "<u8").astype(np.uint64)
        return w[0:2].copy(), w[2:4].copy()

    def challenge(self, stage: int):
        d = self.h.copy().digest()
        self.h.update(b"c" + bytes([stage]))
        w = np.frombuffer(d[:16], "<u8").astype(np.uint64)
        return w.copy()
