"""BitZ BinaryPcs opening on the GPU against the oracle (oracle/binary_pcs.py).

Round 0 (the out-of-domain sample with its grinding), the ring switch, and
the whole bit-MLE opening (ring switch + open_basis + the recursive Ligerito
proof) must leave identical transcripts and produce identical bytes:
write_round0 || write_ring_switch || write_ligerito.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,bits", [(0, 0), (1, 3), (6, 0), (12, 5), (13, 8), (16, 0), (20, 12)])
def test_round0_matches_oracle(oracle, ctx, m, bits):
    from bitz_gb300 import BinaryPcs, Blake3Transcript, DeviceArray, LigeritoConfig
    from oracle.binary_pcs import prove_round0
    from oracle.transcript import Blake3Transcript as OT

    packed = oracle.chacha_words(m + 3, 1 << m)
    ot = OT()
    ot.absorb_slice(b"root")
    exp = prove_round0(ot, packed, bits)
    pcs = BinaryPcs(m, LigeritoConfig(1, [0], [1, 1], [1, 1], [0, 0]), bits, ctx)
    t = Blake3Transcript()
    t.absorb_slice(b"root")
    d = DeviceArray.from_host(packed, ctx)
    try:
        got = pcs.prove_round0(t, d)
        assert got.y.tolist() == exp.y.tolist()
        assert got.nonce == exp.nonce
        assert got.point.tolist() == exp.point.tolist()
        assert t.state_digest() == ot.state_digest()
    finally:
        d.free()


@pytest.mark.parametrize("m", [0, 3, 7, 10, 16])
def test_ring_switch_matches_oracle(oracle, ctx, m):
    import ctypes

    from bitz_gb300 import Blake3Transcript, DeviceArray, lib
    from bitz_gb300._lib import check, ptr
    from oracle.binary_pcs import ring_switch_prove
    from oracle.transcript import Blake3Transcript as OT

    rng = np.random.default_rng(m)
    packed = rng.integers(0, 2**64, (1 << m, 2), dtype=np.uint64)
    r_hi = rng.integers(0, 2**64, (m, 2), dtype=np.uint64)
    s, b, beta0 = ring_switch_prove(OT(), packed, r_hi)
    t = Blake3Transcript()
    d = DeviceArray.from_host(packed, ctx)
    db = DeviceArray(1 << m, ctx)
    s_v = np.zeros((128, 2), np.uint64)
    target = np.zeros(2, np.uint64)
    try:
        check(ctx.handle, lib().bz_pcs_ring_switch(ctx.handle, t.handle, d.ptr, 1 << m,
                                                   ptr(r_hi) if m else None, ptr(s_v), db.ptr,
                                                   ptr(target)))
        assert (s_v == s).all() and (target == beta0).all()
        assert (db.to_host() == b).all()
    finally:
        d.free()
        db.free()
    del ctypes


BIT_MLE_CASES = [
    # (packed_log, initial_k, recursive_ks, rates, queries, grinding, fold, ood, round0 bits, hash)
    (10, 5, [3], [2, 2], [20, 10], [4, 2], [2, 1], [0, 1], 4, 1),
    (12, 6, [3, 2], [1, 1, 1], [30, 8, 4], [0, 0, 0], None, None, 0, 0),
    (14, 7, [4], [2, 2], [64, 20], [8, 6], None, [0, 2], 6, 1),
]


def _bit_mle_both(oracle, ctx, case, seed):
    from bitz_gb300 import BinaryPcs, Blake3Transcript, DeviceArray, LigeritoConfig, codec
    from oracle import codec as OC
    from oracle.binary_pcs import open_bit_mle, prove_round0
    from oracle.ligerito import LigeritoConfig as OCfg
    from oracle.transcript import Blake3Transcript as OT

    m, k, ks, rates, qs, gb, fb, ood, r0_bits, kind = case
    packed = oracle.chacha_words(seed, 1 << m)
    point = np.random.default_rng(seed).integers(0, 2**64, (m + 7, 2), dtype=np.uint64)
    cw, tree, root = oracle.commit(packed, rates[0], k, kind, n_threads=8)
    ot = OT()
    ot.absorb_slice(root)
    o_r0 = prove_round0(ot, packed, r0_bits)
    s_v, lig = open_bit_mle(ot, OCfg(k, ks, rates, qs, gb, fb, ood, kind), packed, cw, tree,
                            root, o_r0, point)
    ow = OC.Writer()
    ow.round0(o_r0.y, o_r0.nonce)
    ow.ring_switch(s_v)
    ow.ligerito(lig)

    pcs = BinaryPcs(m, LigeritoConfig(k, ks, rates, qs, gb, fb, ood, kind), r0_bits, ctx)
    c, pd = pcs.commit(packed)
    assert c.root == root
    d = DeviceArray.from_host(packed, ctx)
    t = Blake3Transcript()
    t.absorb_slice(c.root)
    try:
        r0 = pcs.prove_round0(t, d)
        op = pcs.open_bit_mle(t, d, pd, r0, point)
        w = codec.Writer()
        r0.write(w)
        op.write(w)
        assert w.into_bytes() == bytes(ow.buf)
        assert t.state_digest() == ot.state_digest()
    finally:
        pd.free()
        d.free()


@pytest.mark.parametrize("case", BIT_MLE_CASES)
def test_open_bit_mle_matches_oracle(oracle, ctx, case):
    _bit_mle_both(oracle, ctx, case, seed=case[0] + 7)


def test_open_bit_mle_c1_shape(oracle, ctx):
    """2^20 packed words (2^10 lanes x 2^10 columns, rate 1/4) opened at one
    random point: the C1 benchmark's opening."""
    _bit_mle_both(oracle, ctx, (20, 10, [5], [2, 2], [148, 64], [16, 8], [0, 2], [0, 1], 8, 1),
                  seed=0)


def test_open_basis_rejects_wrong_round0(oracle, ctx):
    from bitz_gb300 import BinaryPcs, Blake3Transcript, BzError, DeviceArray, LigeritoConfig

    m, k = 10, 5
    packed = oracle.chacha_words(2, 1 << m)
    small = oracle.chacha_words(2, 1 << 8)
    pcs = BinaryPcs(m, LigeritoConfig(k, [3], [2, 2], [8, 4], [0, 0]), 0, ctx)
    c, pd = pcs.commit(packed)
    d, ds = DeviceArray.from_host(packed, ctx), DeviceArray.from_host(small, ctx)
    try:
        r0_small = pcs.prove_round0(Blake3Transcript(), ds)     # 8 variables, not 10
        with pytest.raises(BzError):
            pcs.open_bit_mle(Blake3Transcript(), d, pd, r0_small,
                             np.zeros((m + 7, 2), np.uint64))
        r0 = pcs.prove_round0(Blake3Transcript(), d)
        with pytest.raises(BzError):                               # point of the wrong length
            pcs.open_bit_mle(Blake3Transcript(), d, pd, r0, np.zeros((m + 6, 2), np.uint64))
    finally:
        pd.free()
        d.free()
        ds.free()
