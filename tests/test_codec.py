"""Proof codec (src/proof_codec.rs, src/binary_pcs.rs:487-557) against the
oracle's restatement (host code in libbitzgpu.so; no GPU needed).

Covers: bincode LigeritoProof bytes identical to the oracle's for random
proofs (empty vectors, ragged rows, every field populated), the fixed layout
of the empty proof, round trips through both decoders, rejection of every
truncation, trailing bytes and oversized lengths, round-0 and ring-switch
framing with the non-canonical presence tag, and read_ligerito's bounds.
"""
import random
import struct

import numpy as np
import pytest

from oracle import codec as OC


@pytest.fixture(scope="module")
def C():
    from bitz_gb300 import codec

    return codec


def _rand_proof(rng: random.Random, small=False):
    def gf():
        return (rng.getrandbits(64), rng.getrandbits(64))

    def rows():
        n = rng.choice([0, 1, 3] if small else [0, 1, 2, 5, 17])
        same = rng.random() < 0.7
        L = rng.choice([0, 1, 4, 8])
        return [[gf() for _ in range(L if same else rng.choice([0, 1, 3, 8]))] for _ in range(n)]

    def hashes():
        return [rng.randbytes(32) for _ in range(rng.choice([0, 1, 7, 30]))]

    p = OC.LigeritoProof()
    p.initial_root = rng.randbytes(32)
    p.initial_proof = OC.RecursiveProof(rows(), hashes())
    nr = rng.choice([0, 1, 2, 3])
    p.recursive_roots = [rng.randbytes(32) for _ in range(nr)]
    p.recursive_proofs = [OC.RecursiveProof(rows(), hashes()) for _ in range(rng.choice([0, nr]))]
    p.final_proof = OC.FinalProof([gf() for _ in range(rng.choice([0, 1, 16]))], rows(), hashes())
    p.sumcheck_transcript = [(gf(), gf()) for _ in range(rng.choice([0, 1, 13]))]
    p.grinding_nonces = [rng.getrandbits(64) for _ in range(rng.choice([0, 1, 3]))]
    p.ood_values = [gf() for _ in range(rng.choice([0, 2]))]
    p.fold_grinding_nonces = [rng.getrandbits(64) for _ in range(rng.choice([0, 12]))]
    return p


def _to_product(C, p):
    rr = lambda rows: [np.array(r, dtype=np.uint64).reshape(-1, 2) for r in rows]  # noqa: E731
    return C.LigeritoProof(
        initial_root=p.initial_root,
        initial_proof=C.RecursiveProof(rr(p.initial_proof.opened_rows),
                                       p.initial_proof.merkle_proof),
        recursive_roots=p.recursive_roots,
        recursive_proofs=[C.RecursiveProof(rr(q.opened_rows), q.merkle_proof)
                          for q in p.recursive_proofs],
        final_proof=C.FinalProof(np.array(p.final_proof.yr, dtype=np.uint64).reshape(-1, 2),
                                 rr(p.final_proof.opened_rows), p.final_proof.merkle_proof),
        sumcheck_transcript=np.array(p.sumcheck_transcript, dtype=np.uint64).reshape(-1, 2, 2),
        grinding_nonces=np.array(p.grinding_nonces, dtype=np.uint64),
        ood_values=np.array(p.ood_values, dtype=np.uint64).reshape(-1, 2),
        fold_grinding_nonces=np.array(p.fold_grinding_nonces, dtype=np.uint64))


def _same(C, a, o):
    """product LigeritoProof a equals oracle LigeritoProof o."""
    def rows_eq(x, y):
        return len(x) == len(y) and all(
            np.array(r, np.uint64).reshape(-1, 2).tolist() == [list(g) for g in s]
            for r, s in zip(x, y))

    def hs_eq(x, y):
        if isinstance(x, np.ndarray):
            x = [bytes(h) for h in x.reshape(-1, 32)]
        return [bytes(h) for h in x] == [bytes(h) for h in y]

    assert bytes(a.initial_root) == o.initial_root
    assert rows_eq(a.initial_proof.opened_rows, o.initial_proof.opened_rows)
    assert hs_eq(a.initial_proof.merkle_proof, o.initial_proof.merkle_proof)
    assert hs_eq(a.recursive_roots, o.recursive_roots)
    assert len(a.recursive_proofs) == len(o.recursive_proofs)
    for x, y in zip(a.recursive_proofs, o.recursive_proofs):
        assert rows_eq(x.opened_rows, y.opened_rows) and hs_eq(x.merkle_proof, y.merkle_proof)
    assert a.final_proof.yr.tolist() == [list(g) for g in o.final_proof.yr]
    assert rows_eq(a.final_proof.opened_rows, o.final_proof.opened_rows)
    assert hs_eq(a.final_proof.merkle_proof, o.final_proof.merkle_proof)
    assert a.sumcheck_transcript.tolist() == [[list(u), list(v)] for u, v in o.sumcheck_transcript]
    assert a.grinding_nonces.tolist() == o.grinding_nonces
    assert a.ood_values.tolist() == [list(g) for g in o.ood_values]
    assert a.fold_grinding_nonces.tolist() == o.fold_grinding_nonces


def test_empty_proof_layout(C):
    p = OC.LigeritoProof()
    blob = OC.encode_ligerito(p)
    # root + 11 empty Vec lengths (initial rows, initial hashes, recursive roots,
    # recursive proofs, yr, final rows, final hashes, sumcheck, grinding nonces,
    # ood values, fold nonces)
    assert blob == bytes(32) + bytes(8 * 11)
    assert C.encode_ligerito(_to_product(C, p)) == blob


def test_small_proof_layout():
    p = OC.LigeritoProof(initial_root=bytes(range(32)))
    p.initial_proof = OC.RecursiveProof([[(1, 2)]], [b"\xaa" * 32])
    p.sumcheck_transcript = [((3, 4), (5, 6))]
    p.grinding_nonces = [7]
    blob = OC.encode_ligerito(p)
    q = lambda *v: struct.pack("<" + "Q" * len(v), *v)  # noqa: E731
    expect = (bytes(range(32)) + q(1, 1, 1, 2) + q(1) + b"\xaa" * 32 + q(0, 0, 0, 0, 0)
              + q(1, 3, 4, 5, 6) + q(1, 7) + q(0, 0))
    assert blob == expect


@pytest.mark.parametrize("seed", range(12))
def test_encode_matches_oracle_and_round_trips(C, seed):
    rng = random.Random(seed)
    p = _rand_proof(rng)
    blob = OC.encode_ligerito(p)
    prod = _to_product(C, p)
    assert C.encode_ligerito(prod) == blob
    _same(C, C.decode_ligerito(blob), p)
    _same(C, prod, OC.decode_ligerito(blob))
    assert C.encode_ligerito(C.decode_ligerito(blob)) == blob


@pytest.mark.parametrize("seed", range(4))
def test_decode_rejects_truncation_and_trailing(C, seed):
    rng = random.Random(100 + seed)
    blob = OC.encode_ligerito(_rand_proof(rng, small=True))
    for cut in range(len(blob)):
        with pytest.raises(C.BzError) as e:
            C.decode_ligerito(blob[:cut])
        assert e.value.status == 11
        with pytest.raises(OC.CodecError):
            OC.decode_ligerito(blob[:cut])
    for extra in (b"\x00", b"\x01" * 9):
        with pytest.raises(C.BzError):
            C.decode_ligerito(blob + extra)
        with pytest.raises(OC.CodecError):
            OC.decode_ligerito(blob + extra)


def test_decode_rejects_oversized_lengths(C):
    base = bytearray(OC.encode_ligerito(OC.LigeritoProof()))
    for field_idx in range(11):
        for big in (1, 2**32, 2**63, 2**64 - 1):
            b = bytearray(base)
            struct.pack_into("<Q", b, 32 + 8 * field_idx, big)
            with pytest.raises(C.BzError):
                C.decode_ligerito(bytes(b))
            with pytest.raises(OC.CodecError):
                OC.decode_ligerito(bytes(b))


def test_stream_round0_ring_switch_ligerito(C):
    rng = random.Random(7)
    p = _rand_proof(rng)
    s_v = [(rng.getrandbits(64), rng.getrandbits(64)) for _ in range(128)]
    ow = OC.Writer()
    pw = C.Writer()
    for w in (ow, pw):
        w.round0((1, 2), None)
        w.round0((3, 4), 2**64 - 5)
        w.len(99)
        w.gf((5, 6))
        w.bytes(b"raw")
        w.ring_switch(s_v)
    ow.ligerito(p)
    pw.ligerito(_to_product(C, p))
    stream = bytes(ow.buf)
    assert pw.into_bytes() == stream
    r = C.Reader(stream)
    y, n = r.round0()
    assert y.tolist() == [1, 2] and n is None
    y, n = r.round0()
    assert y.tolist() == [3, 4] and n == 2**64 - 5
    assert r.len() == 99 and r.gf().tolist() == [5, 6] and r.take(3) == b"raw"
    assert r.ring_switch().tolist() == [list(g) for g in s_v]
    _same(C, r.ligerito(), p)
    assert r.remaining() == 0
    with pytest.raises(C.BzError) as e:
        r.len()
    assert e.value.status == 9


def test_round0_noncanonical_tag(C):
    for tag in (2, 3, 2**64 - 1):
        b = struct.pack("<QQQ", 1, 2, tag) + struct.pack("<Q", 5)
        with pytest.raises(C.BzError) as e:
            C.Reader(b).round0()
        assert e.value.status == 10
        with pytest.raises(OC.CodecError) as oe:
            OC.Reader(b).round0()
        assert oe.value.kind == "noncanonical"
    # a present nonce that is cut off is truncated, not non-canonical
    with pytest.raises(C.BzError) as e:
        C.Reader(struct.pack("<QQQ", 1, 2, 1)).round0()
    assert e.value.status == 9


def test_read_ligerito_bounds(C):
    blob = OC.encode_ligerito(OC.LigeritoProof())
    # declared length beyond the bytes left
    b = struct.pack("<Q", len(blob) + 1) + blob
    with pytest.raises(C.BzError) as e:
        C.Reader(b).ligerito()
    assert e.value.status == 9
    with pytest.raises(OC.CodecError) as oe:
        OC.Reader(b).ligerito()
    assert oe.value.kind == "truncated"
    # declared length above the 64 MiB cap
    b = struct.pack("<Q", (64 << 20) + 1) + blob
    with pytest.raises(C.BzError) as e:
        C.Reader(b).ligerito()
    assert e.value.status == 9
    # a blob with a trailing byte inside its frame is a bincode error
    b = struct.pack("<Q", len(blob) + 1) + blob + b"\x00"
    with pytest.raises(C.BzError) as e:
        C.Reader(b).ligerito()
    assert e.value.status == 11
    with pytest.raises(OC.CodecError) as oe:
        OC.Reader(b).ligerito()
    assert oe.value.kind == "bincode"


def test_ring_switch_needs_128(C):
    with pytest.raises(ValueError):
        C.Writer().ring_switch(np.zeros((127, 2), np.uint64))
    with pytest.raises(C.BzError) as e:
        C.Reader(bytes(16 * 127)).ring_switch()
    assert e.value.status == 9


def test_benchmark_size_proof_round_trip_is_linear_time(C):
    """A proof of the 2^24 opening's size (148 rows of 4096 elements, 9.9 MB)
    encodes, decodes and round-trips; the decoder appends row after row, so
    its time must stay linear in the blob (well under a second here)."""
    import time

    rng = np.random.default_rng(17)
    rows = [rng.integers(0, 2**64, (4096, 2), dtype=np.uint64) for _ in range(148)]
    p = C.LigeritoProof(
        initial_root=bytes(range(32)),
        initial_proof=C.RecursiveProof(rows, rng.integers(0, 256, (1500, 32), dtype=np.uint8)),
        recursive_roots=np.zeros((1, 32), np.uint8),
        recursive_proofs=[],
        final_proof=C.FinalProof(rng.integers(0, 2**64, (64, 2), dtype=np.uint64),
                                 [rng.integers(0, 2**64, (64, 2), dtype=np.uint64)
                                  for _ in range(148)],
                                 rng.integers(0, 256, (600, 32), dtype=np.uint8)),
        sumcheck_transcript=rng.integers(0, 2**64, (19, 2, 2), dtype=np.uint64),
        grinding_nonces=np.array([1, 2], np.uint64),
        ood_values=np.zeros((0, 2), np.uint64),
        fold_grinding_nonces=np.zeros(0, np.uint64))
    blob = C.encode_ligerito(p)
    assert len(blob) > 9_800_000
    t0 = time.perf_counter()
    q = C.decode_ligerito(blob)
    assert time.perf_counter() - t0 < 1.0
    assert all((a == b).all() for a, b in zip(q.initial_proof.opened_rows, rows))
    assert C.encode_ligerito(q) == blob
