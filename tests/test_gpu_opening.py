"""GPU proof-of-work search and the level-0 Ligerito opening against the oracle.

* bz_pow_first_nonce must return the serial scan's nonce (first_pow_nonce,
  src/utils/blake3x4.rs:42-69) for every prefix length the one-block message
  allows, for windows that start mid-range, and report an empty range.
* bz_transcript_grind_pow must leave the transcript where the oracle's
  ZincChallenger::grind_pow leaves it.
* bz_ligerito_open_l0 must reproduce the oracle's level-0 opening
  (oracle/ligerito_l0.py) bit for bit: every sumcheck message, fold and query
  nonce, fold challenge, level-1 root, query, alpha, opened row and
  multi-proof hash, the folded arrays, and the final transcript state.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bits", [1, 5, 8, 12, 16, 20])
@pytest.mark.parametrize("plen", [0, 3, 16, 24, 31, 32, 55, 56])
def test_pow_first_nonce(oracle, ctx, bits, plen):
    from bitz_gb300 import pow_first_nonce

    prefix = bytes((13 * i + 3 * bits + plen) & 0xFF for i in range(plen))
    got = pow_first_nonce(prefix, bits, ctx=ctx)
    assert got == oracle.pow_first_nonce(prefix, bits)


@pytest.mark.parametrize("bits", [4, 10, 14])
def test_pow_windows(oracle, ctx, bits):
    from bitz_gb300 import pow_first_nonce

    prefix = bytes(range(16))
    first = oracle.pow_first_nonce(prefix, bits)
    # start past the first hit: the next hit
    assert pow_first_nonce(prefix, bits, start=first + 1, ctx=ctx) == \
        oracle.pow_first_nonce(prefix, bits, start=first + 1)
    # a range that ends at the first hit holds none
    assert pow_first_nonce(prefix, bits, start=0, end=first, ctx=ctx) is None
    # start near the top of the nonce space (64-bit counter arithmetic)
    top = 2**64 - 2**20
    assert pow_first_nonce(prefix, bits, start=top, ctx=ctx) == \
        oracle.pow_first_nonce(prefix, bits, start=top)
    assert pow_first_nonce(prefix, 0, start=77, ctx=ctx) == 77
    assert pow_first_nonce(prefix, bits, start=5, end=5, ctx=ctx) is None


def test_pow_rejects_bad_arguments(ctx):
    from bitz_gb300 import BzError, pow_first_nonce

    with pytest.raises(BzError):
        pow_first_nonce(bytes(57), 4, ctx=ctx)
    with pytest.raises(BzError):
        pow_first_nonce(bytes(16), 257, ctx=ctx)


@pytest.mark.parametrize("bits", [0, 1, 9, 17])
def test_transcript_grind_pow(oracle, ctx, bits):
    from bitz_gb300 import Blake3Transcript, ZincChallenger
    from oracle.transcript import Blake3Transcript as OT, ZincChallenger as OZ

    p = ZincChallenger(Blake3Transcript(), ctx)
    o = OZ(OT())
    for ch in (p, o):
        ch.observe_label(b"grind")
        ch.observe_f128([bits, 1])
    assert p.grind_pow(bits) == o.grind_pow(bits)
    assert p.t.state_digest() == o.t.state_digest()


L0_CASES = [
    # (log_n, log_inv_rate0, initial_k, recursive_k0, log_inv_rate1, fold_bits, grind_bits,
    #  queries, hash_kind)
    (10, 1, 2, 2, 1, 0, 0, 4, 1),
    (12, 2, 4, 3, 2, 6, 8, 12, 1),
    (12, 2, 6, 2, 2, 10, 0, 40, 0),
    (14, 2, 7, 3, 3, 12, 12, 64, 1),
    (16, 2, 8, 4, 2, 14, 16, 148, 1),
    (18, 1, 9, 5, 2, 16, 14, 100, 1),
]


def _run_l0(oracle, ctx, case, seed):
    from bitz_gb300 import Blake3Transcript, DeviceArray, L0Config, PcsParams, commit, open_l0
    from oracle.ligerito_l0 import L0Config as OCfg, open_l0 as oopen
    from oracle.transcript import Blake3Transcript as OT, ZincChallenger as OZ

    lm, r0, k, k1, r1, fb, gb, q, kind = case
    packed = oracle.chacha_words(seed, 1 << lm)
    basis = oracle.chacha_words(seed + 100, 1 << lm)
    target = [seed * 7 + 1, seed * 11 + 3]
    cw, tree, root = oracle.commit(packed, r0, k, kind, n_threads=8)
    ores = oopen(OZ(OT()), packed, basis, target, cw, tree, root,
                 OCfg(k, k1, r0, r1, fb, gb, q, kind))

    c, pd = commit(packed, PcsParams(lm + 7, r0, k, kind), ctx)
    assert c.root == root
    dp = DeviceArray.from_host(packed, ctx)
    db = DeviceArray.from_host(basis, ctx)
    tr = Blake3Transcript()
    res = open_l0(tr, pd, dp, db, target, L0Config(k, k1, r1, fb, gb, q, kind), ctx)
    try:
        assert len(res.sumcheck) == len(ores.sumcheck)
        for (a0, a2), (b0, b2) in zip(res.sumcheck, ores.sumcheck):
            assert a0.tolist() == b0.tolist() and a2.tolist() == b2.tolist()
        assert res.fold_nonces == ores.fold_nonces
        assert res.fold_challenges.tolist() == np.array(ores.fold_challenges).reshape(-1, 2).tolist()
        assert res.root1 == ores.root1
        assert res.grinding_nonce == ores.grinding_nonce
        assert res.queries == ores.queries
        assert res.alpha.tolist() == ores.alpha.tolist()
        assert (res.opened_rows == ores.opened_rows).all()
        assert res.merkle_proof.shape == ores.merkle_proof.shape
        assert (res.merkle_proof == ores.merkle_proof).all()
        f1, b1 = res.folded_host()
        assert (f1 == ores.folded).all() and (b1 == ores.folded_basis).all()
    finally:
        res.free()
        pd.free()
        dp.free()
        db.free()


@pytest.mark.parametrize("case", L0_CASES)
def test_open_l0_matches_oracle(oracle, ctx, case):
    _run_l0(oracle, ctx, case, seed=case[0])


def test_open_l0_transcript_state(oracle, ctx):
    """The transcript is advanced in place: after the opening both sides draw
    the same next challenge."""
    from bitz_gb300 import Blake3Transcript, DeviceArray, L0Config, PcsParams, commit, open_l0
    from oracle.ligerito_l0 import L0Config as OCfg, open_l0 as oopen
    from oracle.transcript import Blake3Transcript as OT, ZincChallenger as OZ

    lm, r0, k = 12, 2, 4
    packed = oracle.chacha_words(5, 1 << lm)
    basis = oracle.chacha_words(6, 1 << lm)
    cw, tree, root = oracle.commit(packed, r0, k, 1)
    ot = OT()
    ot.absorb_slice(b"prior protocol state")
    oopen(OZ(ot), packed, basis, [1, 2], cw, tree, root, OCfg(k, 3, r0, 2, 5, 6, 10, 1))
    c, pd = commit(packed, PcsParams(lm + 7, r0, k, 1), ctx)
    dp, db = DeviceArray.from_host(packed, ctx), DeviceArray.from_host(basis, ctx)
    t = Blake3Transcript()
    t.absorb_slice(b"prior protocol state")
    res = open_l0(t, pd, dp, db, [1, 2], L0Config(k, 3, 2, 5, 6, 10, 1), ctx)
    try:
        assert t.state_digest() == ot.state_digest()
        assert t.challenge_bytes(16) == ot.challenge_bytes(16)
    finally:
        res.free()
        pd.free()
        dp.free()
        db.free()


def test_open_l0_rejects_bad_config(oracle, ctx):
    from bitz_gb300 import (Blake3Transcript, BzError, DeviceArray, L0Config, PcsParams, commit,
                            open_l0)

    lm, r0, k = 10, 2, 4
    packed = oracle.chacha_words(1, 1 << lm)
    c, pd = commit(packed, PcsParams(lm + 7, r0, k, 1), ctx)
    dp = DeviceArray.from_host(packed, ctx)
    try:
        for cfg in (L0Config(k + 1, 2, 2), L0Config(k, lm - k + 1, 2),
                    L0Config(k, 2, 2, queries0=(1 << (lm - k + r0)) + 1),
                    L0Config(k, 2, 2, hash_kind=7)):
            with pytest.raises(BzError):
                open_l0(Blake3Transcript(), pd, dp, dp, [0, 0], cfg, ctx)
        # the whole code length as queries is allowed (every position once)
        res = open_l0(Blake3Transcript(), pd, dp, dp, [0, 0],
                      L0Config(k, 2, 2, queries0=1 << (lm - k + r0)), ctx)
        assert res.queries == list(range(1 << (lm - k + r0)))
        assert len(res.merkle_proof) == 0
        res.free()
    finally:
        pd.free()
        dp.free()


def test_open_l0_c2_shape(oracle, ctx):
    """The 2^24-element witness (2^12 lanes x 2^12 columns, rate 1/4) opened
    with 12 lane folds, the shape of the benchmark's opening."""
    _run_l0(oracle, ctx, (24, 2, 12, 6, 2, 16, 16, 148, 1), seed=1)


PROVE_CASES = [
    # (log_n, rate0, initial_k, recursive_ks, log_inv_rates, queries, grinding, fold_grinding,
    #  ood, hash)
    (10, 1, 2, [2], [1, 1], [4, 3], [0, 0], None, None, 1),
    (12, 2, 4, [3, 2], [2, 2, 1], [10, 6, 5], [4, 3, 2], [3, 2, 0], [0, 1, 2], 1),
    (12, 2, 6, [2], [2, 2], [40, 12], [0, 6], [8, 0], [0, 1], 0),
    (14, 2, 7, [3, 2], [2, 2, 2], [64, 30, 12], [8, 6, 4], None, [0, 0, 1], 1),
    (16, 2, 8, [4], [2, 2], [148, 60], [12, 10], [10, 6], None, 1),
]


def _prove_both(oracle, ctx, case, seed):
    from bitz_gb300 import (Blake3Transcript, DeviceArray, LigeritoConfig, PcsParams, codec,
                            commit, prove)
    from oracle import codec as OC
    from oracle.ligerito import LigeritoConfig as OCfg, prove as oprove
    from oracle.transcript import Blake3Transcript as OT, ZincChallenger as OZ

    lm, r0, k, ks, rates, qs, gb, fb, ood, kind = case
    packed = oracle.chacha_words(seed, 1 << lm)
    basis = oracle.chacha_words(seed + 50, 1 << lm)
    target = [seed, seed * 3 + 1]
    cw, tree, root = oracle.commit(packed, r0, k, kind, n_threads=8)
    ot = OT()
    ot.absorb_slice(b"outer protocol")
    exp = oprove(OZ(ot), OCfg(k, ks, rates, qs, gb, fb, ood, kind), packed, basis, target, cw,
                 tree, root)
    c, pd = commit(packed, PcsParams(lm + 7, r0, k, kind), ctx)
    dp, db = DeviceArray.from_host(packed, ctx), DeviceArray.from_host(basis, ctx)
    t = Blake3Transcript()
    t.absorb_slice(b"outer protocol")
    try:
        got = prove(t, pd, dp, db, target, LigeritoConfig(k, ks, rates, qs, gb, fb, ood, kind),
                    ctx)
        blob = codec.encode_ligerito(got)
        assert blob == OC.encode_ligerito(exp)
        assert t.state_digest() == ot.state_digest()
        return blob
    finally:
        pd.free()
        dp.free()
        db.free()


@pytest.mark.parametrize("case", PROVE_CASES)
def test_prove_matches_oracle(oracle, ctx, case):
    _prove_both(oracle, ctx, case, seed=case[0] + 1)


def test_prove_rejects_bad_config(oracle, ctx):
    from bitz_gb300 import (Blake3Transcript, BzError, DeviceArray, LigeritoConfig, PcsParams,
                            commit, prove)

    lm, r0, k = 10, 2, 4
    packed = oracle.chacha_words(1, 1 << lm)
    c, pd = commit(packed, PcsParams(lm + 7, r0, k, 1), ctx)
    dp = DeviceArray.from_host(packed, ctx)
    bad = [
        LigeritoConfig(k, [2], [1, 1], [4, 4], [0, 0]),                  # rate 0 != commitment
        LigeritoConfig(k, [7], [2, 1], [4, 4], [0, 0]),                  # k exceeds folded length
        LigeritoConfig(k, [2], [2, 1], [4, 4], [0, 0], ood_samples=[1, 0]),  # OOD at level 0
        LigeritoConfig(k, [2], [2, 1], [4, 1000], [0, 0]),               # queries > block length
        LigeritoConfig(k + 1, [2], [2, 1], [4, 4], [0, 0]),              # initial_k != lanes
    ]
    try:
        for cfg in bad:
            with pytest.raises(BzError):
                prove(Blake3Transcript(), pd, dp, dp, [0, 0], cfg, ctx)
        with pytest.raises(ValueError):
            LigeritoConfig(k, [2], [2], [4, 4], [0, 0]).to_c()
    finally:
        pd.free()
        dp.free()


def test_prove_c2_shape(oracle, ctx):
    """The 2^24-element witness (2^12 lanes x 2^12 columns, rate 1/4) with a
    two-step recursion: the benchmark's full opening shape."""
    _prove_both(oracle, ctx, (24, 2, 12, [6, 3], [2, 2, 2], [148, 100, 30], [16, 10, 8],
                              [4, 2, 0], None, 1), seed=1)
