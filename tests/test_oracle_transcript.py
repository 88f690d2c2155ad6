"""Oracle transcript, BLAKE3 extended output and proof of work (CPU).

Pins:
* BLAKE3 XOF of the empty input, 131 bytes -- the published BLAKE3 test
  vector for input length 0 (the `blake3` crate's test_vectors.json, the
  crate pinned by BitZ's Cargo.lock at 1.8.7); the first 32 bytes are the
  32-byte hash already pinned in test_oracle_hash.py.
* Framing and sampling behaviour the reference's own transcript tests check
  (src/transcript/mod.rs:173-190): absorb_slice is length framed, and two
  samplings from one state differ.
* Proof of work: the found nonce passes and every smaller nonce fails
  (first_pow_nonce, src/utils/blake3x4.rs:42-69), verify_pow accepts it and
  rejects a failing one, zero bits gives nonce 0.
"""
import os
import struct

import numpy as np
import pytest

EMPTY_XOF_131 = (
    "af1349b9f5f9a1a6a0404dea36dcc9499bcb25c9adc112b7cc9a93cae41f3262"
    "e00f03e7b69af26b7faaf09fcd333050338ddfe085b8cc869ca98b206c08243a"
    "26f5487789e8f660afe6c99ef9e0c52b92e7393024a80459cf91f476f9ffdbda"
    "7001c22e159b402631f277ca96f2defdf1078282314e763699a31c5363165421"
    "cce14d"
)


def test_blake3_xof_empty_kat(oracle):
    assert oracle.blake3_xof(b"", 131).hex() == EMPTY_XOF_131


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 1023, 1024, 1025, 2048, 3072, 5000, 70000])
def test_blake3_xof_prefix_is_hash(oracle, n):
    d = np.random.default_rng(n).integers(0, 256, n, dtype=np.uint8).tobytes()
    x = oracle.blake3_xof(d, 300)
    assert x[:32] == oracle.blake3(d)
    assert oracle.blake3_xof(d, 64) == x[:64]
    assert oracle.blake3_xof(d, 65) == x[:65]


def test_transcript_framing(oracle):
    from oracle.transcript import Blake3Transcript

    a, b = Blake3Transcript(), Blake3Transcript()
    a.absorb_slice(bytes([1, 7, 6, 2]))
    b.absorb_slice(bytes([1]))
    b.absorb_slice(bytes([2]))
    first = a.fill_sampling_bytes(16)
    second = a.fill_sampling_bytes(16)
    other = b.fill_sampling_bytes(16)
    assert first != second and first != other
    # absorb_slice is exactly 0x06 || len LE || data || 0x07
    c = Blake3Transcript()
    c.absorb(b"\x06" + struct.pack("<Q", 4) + bytes([1, 7, 6, 2]) + b"\x07")
    a2 = Blake3Transcript()
    a2.absorb_slice(bytes([1, 7, 6, 2]))
    assert c.state_digest() == a2.state_digest()


def test_transcript_challenge_replays(oracle):
    from oracle.transcript import Blake3Transcript

    a, b = Blake3Transcript(), Blake3Transcript()
    for t in (a, b):
        t.absorb_slice(b"label")
    xs = [a.challenge_bytes(16) for _ in range(8)]
    ys = [b.challenge_bytes(16) for _ in range(8)]
    assert xs == ys and len(set(xs)) == 8
    # a squeeze does not consume the state: digest is over absorbed bytes
    c = Blake3Transcript()
    c.absorb_slice(b"label")
    out = c._xof(16)
    assert out == Blake3Transcript.challenge_bytes(c.clone(), 16)


@pytest.mark.parametrize("bits", [1, 4, 8, 12])
@pytest.mark.parametrize("plen", [16, 24, 31, 32, 56])
def test_pow_first_nonce_is_smallest(oracle, bits, plen):
    prefix = bytes((7 * i + bits) & 0xFF for i in range(plen))
    n = oracle.pow_first_nonce(prefix, bits)
    assert n is not None and oracle.pow_ok(prefix, n, bits)
    for m in range(n):
        assert not oracle.pow_ok(prefix, m, bits)
    # the serial scan from a later start finds the next passing nonce
    n2 = oracle.pow_first_nonce(prefix, bits, start=n + 1)
    assert n2 > n and oracle.pow_ok(prefix, n2, bits)


def test_pow_bit_order(oracle):
    # leading zeros are counted from the most significant bit of byte 0
    prefix = b"\x00" * 16
    for n in range(200):
        h = oracle.blake3(prefix + struct.pack("<Q", n))
        lz = 0
        for byte in h:
            if byte == 0:
                lz += 8
                continue
            lz += 8 - byte.bit_length()
            break
        for bits in range(0, 12):
            assert oracle.pow_ok(prefix, n, bits) == (lz >= bits)


def test_challenger_grind_and_verify(oracle):
    from oracle.transcript import Blake3Transcript, ZincChallenger

    p = ZincChallenger(Blake3Transcript())
    v = ZincChallenger(Blake3Transcript())
    for ch in (p, v):
        ch.observe_label(b"flock-ligerito-basis-v0")
        ch.observe_f128([5, 6])
    nonce = p.grind_pow(10)
    assert v.verify_pow(nonce, 10)
    assert p.t.state_digest() == v.t.state_digest()
    assert p.grind_pow(0) == 0
    assert v.verify_pow(0, 0)
    assert p.sample_f128().tolist() == v.sample_f128().tolist()
    # a wrong nonce is rejected and the states stay in lockstep
    q = ZincChallenger(Blake3Transcript())
    w = ZincChallenger(Blake3Transcript())
    good = q.grind_pow(8)
    bad = next(m for m in range(good + 1, good + 100000)
               if not oracle.pow_ok(w.t.clone().challenge_bytes(16), m, 8))
    assert not w.verify_pow(bad, 8)
    assert not ZincChallenger(Blake3Transcript()).verify_pow(1, 0)


def test_sample_distinct_queries(oracle):
    from oracle.ligerito_l0 import ceil_log2, sample_distinct_queries
    from oracle.transcript import Blake3Transcript, ZincChallenger

    ch = ZincChallenger(Blake3Transcript())
    qs = sample_distinct_queries(ch, 16, 16)
    assert qs == list(range(16))
    ch2 = ZincChallenger(Blake3Transcript())
    qs2 = sample_distinct_queries(ch2, 1 << 14, 148)
    assert qs2 == sorted(set(qs2)) and len(qs2) == 148
    with pytest.raises(ValueError):
        sample_distinct_queries(ch2, 4, 5)
    assert [ceil_log2(n) for n in (0, 1, 2, 3, 4, 5, 148, 256)] == [0, 0, 1, 2, 2, 3, 8, 8]


def test_oracle_l0_opening_consistency(oracle):
    """The oracle's level-0 opening: its rows authenticate against the root,
    its folds agree with partial_eval_lsb at the fold challenges, and the
    first sumcheck message matches a direct round_msg_lsb."""
    from oracle.ligerito_l0 import L0Config, open_l0
    from oracle.transcript import Blake3Transcript, ZincChallenger

    lm, r, k = 12, 2, 4
    packed = oracle.chacha_words(3, 1 << lm)
    basis = oracle.chacha_words(4, 1 << lm)
    cw, tree, root = oracle.commit(packed, r, k, oracle.BLAKE3)
    cfg = L0Config(initial_k=k, recursive_k0=3, log_inv_rate0=r, log_inv_rate1=2,
                   fold_grinding_bits0=6, grinding_bits0=8, queries0=12)
    res = open_l0(ZincChallenger(Blake3Transcript()), packed, basis, [9, 10], cw, tree, root, cfg)
    assert len(res.sumcheck) == k + 1 and len(res.fold_nonces) == k
    u0, u2 = oracle.round_msg_lsb(packed, basis)
    assert (res.sumcheck[0][0] == u0).all() and (res.sumcheck[0][1] == u2).all()
    rs = np.array(res.fold_challenges)
    assert (oracle.partial_eval_lsb(packed, rs) == res.folded).all()
    n_leaves = 1 << (lm - k + r)
    leaf_hashes = np.array([np.frombuffer(oracle.hash_leaf(row.astype("<u8").tobytes(),
                                                           oracle.BLAKE3), np.uint8)
                            for row in res.opened_rows])
    assert (leaf_hashes == tree[np.array(res.queries)]).all()
    assert oracle.verify_merkle_multi_proof(root, n_leaves, res.queries, leaf_hashes,
                                            res.merkle_proof, oracle.BLAKE3)
    assert res.alpha.shape == (4, 2)
    _, _, root1 = oracle.commit(res.folded, 2, 3, oracle.BLAKE3)
    assert root1 == res.root1


def test_oracle_full_prover_consistency(oracle):
    """The oracle's recursive Ligerito proof: every level's rows authenticate
    against that level's root, the final rows against the last root, the
    proof has the reference's per-level counts, and its bincode blob round
    trips."""
    from oracle import codec as OC
    from oracle.ligerito import LigeritoConfig, prove
    from oracle.transcript import Blake3Transcript, ZincChallenger

    lm, r0, k = 12, 2, 4
    packed = oracle.chacha_words(21, 1 << lm)
    basis = oracle.chacha_words(22, 1 << lm)
    cw, tree, root = oracle.commit(packed, r0, k, oracle.BLAKE3)
    cfg = LigeritoConfig(initial_k=k, recursive_ks=[3, 2], log_inv_rates=[r0, 2, 1],
                         queries=[10, 6, 5], grinding_bits=[4, 3, 2],
                         fold_grinding_bits=[3, 2, 0], ood_samples=[0, 1, 2])
    p = prove(ZincChallenger(Blake3Transcript()), cfg, packed, basis, [5, 6], cw, tree, root)
    assert len(p.recursive_roots) == 2 and len(p.recursive_proofs) == 1
    assert len(p.grinding_nonces) == 3 and len(p.ood_values) == 3
    # messages: 1 + initial_k folds + OOD intros + one intro per induced basis
    # (level 0 and each non-final level) + the recursive folds
    assert len(p.sumcheck_transcript) == 1 + k + 3 + 2 + 3 + 2
    # fold grinds: 3,2,1 bits at level 0 (j < 3), 2,1 bits at level 1
    assert len(p.fold_grinding_nonces) == 3 + 2
    assert len(p.final_proof.yr) == 1 << (lm - k - 3 - 2)

    trace = {}
    p_t = prove(ZincChallenger(Blake3Transcript()), cfg, packed, basis, [5, 6], cw, tree, root,
                trace=trace)
    opened = [p_t.initial_proof, *p_t.recursive_proofs, p_t.final_proof]
    assert [lv[0] for lv in trace["levels"]] == [root, *p_t.recursive_roots]
    for (lroot, block_len, qs), lev in zip(trace["levels"], opened):
        lh = np.array([np.frombuffer(oracle.hash_leaf(
            np.array(r, dtype=np.uint64).astype("<u8").tobytes(), oracle.BLAKE3), np.uint8)
            for r in lev.opened_rows])
        pr = np.frombuffer(b"".join(lev.merkle_proof), np.uint8).reshape(-1, 32)
        assert oracle.verify_merkle_multi_proof(lroot, block_len, qs, lh, pr, oracle.BLAKE3)
    # the transcript replays: rebuild queries from a second run's challenger
    p2 = prove(ZincChallenger(Blake3Transcript()), cfg, packed, basis, [5, 6], cw, tree, root)
    assert OC.encode_ligerito(p) == OC.encode_ligerito(p2)
    blob = OC.encode_ligerito(p)
    assert OC.encode_ligerito(OC.decode_ligerito(blob)) == blob
    assert len(p.initial_proof.opened_rows) == 10
    assert all(len(r) == 1 << k for r in p.initial_proof.opened_rows)
    assert all(len(r) == 1 << 3 for r in p.recursive_proofs[0].opened_rows)
    assert all(len(r) == 1 << 2 for r in p.final_proof.opened_rows)


def _bit_mle(packed, point):
    """MLE over the bits of the packed words at point (low 7 coordinates pick
    the bit of a word), by its definition."""
    from oracle import oracle as O

    eq_lo = O.build_eq_lsb(point[:7])
    eq_hi = O.build_eq_lsb(point[7:])
    bits = np.unpackbits(np.ascontiguousarray(packed, "<u8").view(np.uint8).reshape(-1, 16),
                         axis=1, bitorder="little")                     # [y, v]
    acc = np.zeros(2, np.uint64)
    for y in range(packed.shape[0]):
        sel = eq_lo[bits[y].astype(bool)]
        if sel.shape[0]:
            acc ^= O.gf_mul(np.bitwise_xor.reduce(sel, axis=0), eq_hi[y])
    return acc


def test_oracle_ring_switch_identities(oracle):
    """ring_switch_prove's debug identity (src/ligerito.rs:478-487):
    sum_y B(y) * P(y) = beta0, and the verifier's claim check (:510-516):
    sum_v eq(r_lo, v) * s_v = the bit-MLE value at the full point."""
    from oracle.binary_pcs import ring_switch_prove
    from oracle.transcript import Blake3Transcript

    rng = np.random.default_rng(3)
    m = 8
    packed = rng.integers(0, 2**64, (1 << m, 2), dtype=np.uint64)
    point = rng.integers(0, 2**64, (m + 7, 2), dtype=np.uint64)
    s, b, beta0 = ring_switch_prove(Blake3Transcript(), packed, point[7:])
    assert (np.bitwise_xor.reduce(oracle.gf_mul_many(b, packed), axis=0) == beta0).all()
    eq_lo = oracle.build_eq_lsb(point[:7])
    mu = np.bitwise_xor.reduce(oracle.gf_mul_many(s, eq_lo), axis=0)
    assert (mu == _bit_mle(packed, point)).all()


def test_oracle_round0_and_ood_basis(oracle):
    """ood_eval (split at 2^12-element blocks) equals <P, eq(point)> over the
    full eq table; round 0 grinds, draws and absorbs deterministically."""
    from oracle.binary_pcs import ood_eval, ood_point, prove_round0
    from oracle.transcript import Blake3Transcript

    rng = np.random.default_rng(4)
    for m in (0, 3, 12, 14):
        packed = rng.integers(0, 2**64, (1 << m, 2), dtype=np.uint64)
        pt = ood_point(rng.integers(0, 2**64, 2, dtype=np.uint64), m)
        full = oracle.build_eq_lsb(pt)
        expect = np.bitwise_xor.reduce(oracle.gf_mul_many(packed, full), axis=0)
        assert (ood_eval(packed, pt) == expect).all()
        if m:
            assert (pt[1] == oracle.gf_mul(pt[0], pt[0])).all()
    packed = rng.integers(0, 2**64, (1 << 10, 2), dtype=np.uint64)
    a, b = Blake3Transcript(), Blake3Transcript()
    ra, rb = prove_round0(a, packed, 6), prove_round0(b, packed, 6)
    assert ra.nonce == rb.nonce and ra.nonce is not None
    assert a.state_digest() == b.state_digest() and (ra.y == rb.y).all()
    assert prove_round0(Blake3Transcript(), packed, 0).nonce is None


def test_oracle_open_bit_mle_runs(oracle):
    from oracle import codec as OC
    from oracle.binary_pcs import open_bit_mle, prove_round0
    from oracle.ligerito import LigeritoConfig
    from oracle.transcript import Blake3Transcript

    m, k = 10, 5
    packed = oracle.chacha_words(8, 1 << m)
    cw, tree, root = oracle.commit(packed, 2, k, oracle.BLAKE3)
    t = Blake3Transcript()
    t.absorb_slice(root)
    r0 = prove_round0(t, packed, 4)
    point = np.random.default_rng(5).integers(0, 2**64, (m + 7, 2), dtype=np.uint64)
    cfg = LigeritoConfig(k, [3], [2, 2], [20, 10], [4, 2], [2, 1], [0, 1])
    s_v, lig = open_bit_mle(t, cfg, packed, cw, tree, root, r0, point)
    w = OC.Writer()
    w.round0(r0.y, r0.nonce)
    w.ring_switch(s_v)
    w.ligerito(lig)
    r = OC.Reader(bytes(w.buf))
    y, nonce = r.round0()
    assert list(y) == list(r0.y) and nonce == r0.nonce
    assert [tuple(g) for g in r.ring_switch()] == [tuple(int(x) for x in g) for g in s_v]
    assert OC.encode_ligerito(r.ligerito()) == OC.encode_ligerito(lig)
