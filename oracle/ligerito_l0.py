"""Level-0 Ligerito opening of the oracle (test infrastructure only).

Restates the opening sequence of
vendor/flock-mod/crates/flock-core/src/pcs/ligerito.rs:3566-3720
(recursive_prover_with_basis_initial_impl) from its first observation up to
the opened level-0 rows -- the part whose arrays are the committed
codeword, its Merkle tree and the 2^n packed witness:

1. observe_label("flock-ligerito-basis-v0"), observe_f128(target),
   observe_bytes(initial_root)                                  (:3566-3571)
2. SumcheckProver::new: first message round_msg_lsb(f, basis)   (:2998-3007)
3. initial_k lane folds; round j grinds fold_grinding_bits[0] - j bits
   when positive, samples r, folds, observes (u_0, u_2)         (:3621-3657)
4. ligero_commit of the folded f^1 (recursive_ks[0] lanes, rate
   log_inv_rates[1]); observe its root                         (:3662-3679)
5. ood_samples[1] == 0 here (no OOD rounds)                     (:3686-3706)
6. grind_pow(grinding_bits[0]); sample_distinct_queries(block_len_0,
   queries[0]); alpha_0 = sample_f128_vec(ceil_log2(queries[0])) (:3713-3718)
7. open_initial: the opened rows and the Merkle multi-proof (:3476-3481)

The lookahead fold schedule of the reference (:3606-3651) gives a
bit-identical transcript (an exact polynomial identity) and is not restated.
Only tests/, smoke() and the CPU leg of bench.py import this module.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import oracle as O
from .transcript import ZincChallenger

BASIS_LABEL = b"flock-ligerito-basis-v0"


@dataclass
class L0Config:
    initial_k: int
    recursive_k0: int
    log_inv_rate0: int
    log_inv_rate1: int
    fold_grinding_bits0: int = 0
    grinding_bits0: int = 0
    queries0: int = 8
    hash_kind: int = O.BLAKE3


@dataclass
class L0Opening:
    sumcheck: list = field(default_factory=list)       # [(u_0, u_2)], 1 + initial_k
    fold_nonces: list = field(default_factory=list)
    fold_challenges: list = field(default_factory=list)
    folded: np.ndarray | None = None                    # f^1, 2^(n - initial_k)
    folded_basis: np.ndarray | None = None
    root1: bytes = b""
    grinding_nonce: int = 0
    queries: list = field(default_factory=list)
    alpha: np.ndarray | None = None
    opened_rows: np.ndarray | None = None                # (q, 2^initial_k, 2)
    merkle_proof: np.ndarray | None = None               # (h, 32)


def ceil_log2(n: int) -> int:
    """ligerito.rs:1844-1850."""
    return 0 if n <= 1 else (n - 1).bit_length()


def sample_distinct_queries(ch: ZincChallenger, block_len: int, count: int) -> list:
    """ligerito.rs:3191-3221: draw until ``count`` distinct q = lo % block_len,
    then sort."""
    if count > block_len:
        raise ValueError("query count exceeds block length")
    seen, out = set(), []
    while len(out) < count:
        q = int(ch.sample_f128()[0]) % block_len
        if q not in seen:
            seen.add(q)
            out.append(q)
    return sorted(out)


def open_l0(ch: ZincChallenger, packed: np.ndarray, basis: np.ndarray, target,
            codeword: np.ndarray, tree: np.ndarray, root: bytes, cfg: L0Config) -> L0Opening:
    packed = np.ascontiguousarray(packed, np.uint64).reshape(-1, 2)
    basis = np.ascontiguousarray(basis, np.uint64).reshape(-1, 2)
    log_n = packed.shape[0].bit_length() - 1
    assert packed.shape == basis.shape and packed.shape[0] == 1 << log_n
    k = cfg.initial_k
    block_len_0 = 1 << (log_n - k + cfg.log_inv_rate0)
    lanes = 1 << k
    res = L0Opening()

    ch.observe_label(BASIS_LABEL)
    ch.observe_f128(target)
    ch.observe_bytes(root)

    u0, u2 = O.round_msg_lsb(packed, basis)
    ch.observe_f128(u0)
    ch.observe_f128(u2)
    res.sumcheck.append((u0, u2))
    f, b = packed, basis
    for j in range(k):
        bits = max(cfg.fold_grinding_bits0 - j, 0)
        if bits > 0:
            res.fold_nonces.append(ch.grind_pow(bits))
        r = ch.sample_f128()
        f, b, u0, u2 = O.fold_and_msg_lsb(f, b, r)
        ch.observe_f128(u0)
        ch.observe_f128(u2)
        res.sumcheck.append((u0, u2))
        res.fold_challenges.append(r)
    res.folded, res.folded_basis = f, b

    n1 = log_n - k
    assert n1 >= cfg.recursive_k0
    _, _, root1 = O.commit(f, cfg.log_inv_rate1, cfg.recursive_k0, cfg.hash_kind)
    res.root1 = root1
    ch.observe_bytes(root1)

    res.grinding_nonce = ch.grind_pow(cfg.grinding_bits0)
    res.queries = sample_distinct_queries(ch, block_len_0, cfg.queries0)
    res.alpha = ch.sample_f128_vec(ceil_log2(cfg.queries0))

    cw = np.ascontiguousarray(codeword, np.uint64).reshape(block_len_0, lanes, 2)
    res.opened_rows = cw[res.queries].copy()
    res.merkle_proof = O.merkle_multi_proof(tree, block_len_0, res.queries)
    return res
