"""Recursive Ligerito prover of the oracle (test infrastructure only).

Restates recursive_prover_with_basis_initial_impl
(vendor/flock-mod/crates/flock-core/src/pcs/ligerito.rs:3524-3884) with the
level-0 part of oracle/ligerito_l0.py and then every recursive level:

* induce the level's basis from its queries with the dense
  induce_sumcheck_poly (:1968-2072, oracle.c orc_induce_basis), introduce it
  (round_msg_lsb, :3099-3107), observe, glue with beta (:3125-3145);
* level i: recursive_ks[i] folds, round j ground with
  fold_grinding_bits[i+1] - j bits when positive (:3755-3774);
* last level: yr = f, every element observed, grind_pow(grinding_bits[r]),
  queries, the final rows and multi-proof (:3776-3860);
* otherwise: ligero_commit of the next level, its OOD rounds
  (introduce_new_with_eval with eq(z), :3114-3123), grind, queries, alpha,
  rows, induce, introduce + glue (:3863-3946).

Returns oracle/codec.py's LigeritoProof.  The claimed sums of introduced
polynomials (SumcheckProver::t_r) enter no message, so they are not kept.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import codec as C
from . import oracle as O
from .ligerito_l0 import BASIS_LABEL, ceil_log2, sample_distinct_queries
from .transcript import ZincChallenger


@dataclass
class LigeritoConfig:
    """ProverConfig (ligerito.rs:124-160) fields the prover reads."""
    initial_k: int
    recursive_ks: list
    log_inv_rates: list
    queries: list
    grinding_bits: list
    fold_grinding_bits: list | None = None
    ood_samples: list | None = None
    hash_kind: int = O.BLAKE3

    def fold_bits(self, lvl):
        return self.fold_grinding_bits[lvl] if self.fold_grinding_bits else 0

    def ood(self, lvl):
        return self.ood_samples[lvl] if self.ood_samples else 0


def _t(g) -> tuple:
    return (int(g[0]), int(g[1]))


def _xor_sum(a: np.ndarray) -> np.ndarray:
    return np.bitwise_xor.reduce(a, axis=0) if a.shape[0] else np.zeros(2, np.uint64)


class _Sumcheck:
    """SumcheckProver (ligerito.rs:2981-3182) on host arrays."""

    def __init__(self, ch: ZincChallenger, f, b):
        self.ch, self.f, self.b, self.msgs = ch, f, b, []

    def record(self, u0, u2):
        self.ch.observe_f128(u0)
        self.ch.observe_f128(u2)
        self.msgs.append((_t(u0), _t(u2)))

    def fold(self, r):
        self.f, self.b, u0, u2 = O.fold_and_msg_lsb(self.f, self.b, r)
        self.record(u0, u2)

    def introduce_glue(self, b_new):
        u0, u2 = O.round_msg_lsb(self.f, b_new)
        self.record(u0, u2)
        beta = self.ch.sample_f128()
        self.glue(beta, b_new)

    def glue(self, beta, b_new):
        self.b = self.b ^ O.gf_mul_many(np.tile(beta, (b_new.shape[0], 1)), b_new)

    def ood(self, count, ood_values):
        n = self.f.shape[0].bit_length() - 1
        for _ in range(count):
            z = self.ch.sample_f128_vec(n)
            eq = O.build_eq_lsb(z)
            u0, u2 = O.round_msg_lsb(self.f, eq)
            y = _xor_sum(O.gf_mul_many(self.f, eq))
            self.ch.observe_f128(y)
            ood_values.append(_t(y))
            self.record(u0, u2)
            beta = self.ch.sample_f128()
            self.glue(beta, eq)


def _rows_and_proof(cw, tree, block_len, lanes, queries):
    rows = np.ascontiguousarray(cw, np.uint64).reshape(block_len, lanes, 2)[queries]
    proof = O.merkle_multi_proof(tree, block_len, queries)
    return [[_t(g) for g in r] for r in rows], [bytes(h) for h in proof]


def _induce(log_msg_cols, queries, alpha):
    w = O.build_eq_lsb(np.asarray(alpha, np.uint64).reshape(-1, 2))[:len(queries)]
    return O.induce_basis(log_msg_cols, queries, w)


def prove(ch: ZincChallenger, cfg: LigeritoConfig, packed, basis, target, codeword, tree,
          root: bytes, trace: dict | None = None) -> C.LigeritoProof:
    """``trace``, when given, receives each opened level's (root, block_len,
    queries) in order, for checks that need the queries the proof omits."""
    packed = np.ascontiguousarray(packed, np.uint64).reshape(-1, 2)
    basis = np.ascontiguousarray(basis, np.uint64).reshape(-1, 2)
    log_n = packed.shape[0].bit_length() - 1
    r = len(cfg.recursive_ks)
    k0 = cfg.initial_k
    assert r >= 1 and len(cfg.log_inv_rates) == r + 1 and cfg.ood(0) == 0
    n1 = log_n - k0
    block_len_0 = 1 << (n1 + cfg.log_inv_rates[0])
    proof = C.LigeritoProof(initial_root=bytes(root))

    ch.observe_label(BASIS_LABEL)
    ch.observe_f128(target)
    ch.observe_bytes(root)
    sc = _Sumcheck(ch, packed, basis)
    u0, u2 = O.round_msg_lsb(packed, basis)
    sc.record(u0, u2)
    for j in range(k0):
        bits = max(cfg.fold_bits(0) - j, 0)
        if bits > 0:
            proof.fold_grinding_nonces.append(ch.grind_pow(bits))
        sc.fold(ch.sample_f128())

    k1 = cfg.recursive_ks[0]
    cw1, tree1, root1 = O.commit(sc.f, cfg.log_inv_rates[1], k1, cfg.hash_kind)
    ch.observe_bytes(root1)
    sc.ood(cfg.ood(1), proof.ood_values)
    proof.grinding_nonces.append(ch.grind_pow(cfg.grinding_bits[0]))
    queries_0 = sample_distinct_queries(ch, block_len_0, cfg.queries[0])
    alpha_0 = ch.sample_f128_vec(ceil_log2(cfg.queries[0]))
    rows, hashes = _rows_and_proof(codeword, tree, block_len_0, 1 << k0, queries_0)
    proof.initial_proof = C.RecursiveProof(rows, hashes)
    levels = [(bytes(root), block_len_0, queries_0)]
    sc.introduce_glue(_induce(n1, queries_0, alpha_0))

    prev = (cw1, tree1, 1 << (n1 - k1 + cfg.log_inv_rates[1]), 1 << k1, root1)
    proof.recursive_roots = [root1]
    for i in range(r):
        for j in range(cfg.recursive_ks[i]):
            bits = max(cfg.fold_bits(i + 1) - j, 0)
            if bits > 0:
                proof.fold_grinding_nonces.append(ch.grind_pow(bits))
            sc.fold(ch.sample_f128())
        cw_p, tree_p, block_len, lanes, root_p = prev
        if i == r - 1:
            yr = [_t(v) for v in sc.f]
            for v in sc.f:
                ch.observe_f128(v)
            proof.grinding_nonces.append(ch.grind_pow(cfg.grinding_bits[i + 1]))
            qs = sample_distinct_queries(ch, block_len, cfg.queries[i + 1])
            rows, hashes = _rows_and_proof(cw_p, tree_p, block_len, lanes, qs)
            proof.final_proof = C.FinalProof(yr, rows, hashes)
            proof.sumcheck_transcript = sc.msgs
            if trace is not None:
                trace["levels"] = levels + [(root_p, block_len, qs)]
            return proof
        n_next = sc.f.shape[0].bit_length() - 1
        k_next = cfg.recursive_ks[i + 1]
        rate_next = cfg.log_inv_rates[i + 2]
        cw_n, tree_n, root_n = O.commit(sc.f, rate_next, k_next, cfg.hash_kind)
        ch.observe_bytes(root_n)
        proof.recursive_roots.append(root_n)
        sc.ood(cfg.ood(i + 2), proof.ood_values)
        proof.grinding_nonces.append(ch.grind_pow(cfg.grinding_bits[i + 1]))
        qs = sample_distinct_queries(ch, block_len, cfg.queries[i + 1])
        alpha = ch.sample_f128_vec(ceil_log2(cfg.queries[i + 1]))
        rows, hashes = _rows_and_proof(cw_p, tree_p, block_len, lanes, qs)
        proof.recursive_proofs.append(C.RecursiveProof(rows, hashes))
        levels.append((root_p, block_len, qs))
        sc.introduce_glue(_induce(n_next, qs, alpha))
        prev = (cw_n, tree_n, 1 << (n_next - k_next + rate_next), 1 << k_next, root_n)
    raise AssertionError("unreachable")
