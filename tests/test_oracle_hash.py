"""SHA-256 and BLAKE3 in the oracle, and the Merkle structure of
flock-core/src/merkle.rs (its tests at :825-1400 restated)."""
import hashlib
import os

import numpy as np
import pytest

# Published BLAKE3 digests (BLAKE3 specification test vectors; input byte i is
# i mod 251).  They cover single-block, multi-block and multi-chunk trees.
BLAKE3_KAT = {
    0: "af1349b9f5f9a1a6a0404dea36dcc9499bcb25c9adc112b7cc9a93cae41f3262",
    1: "2d3adedff11b61f14c886e35afa036736dcd87a74d27b5c1510225d0f592e213",
    63: "e9bc37a594daad83be9470df7f7b3798297c3d834ce80ba85d6e207627b7db7b",
    64: "4eed7141ea4a5cd4b788606bd23f46e212af9cacebacdc7d1f4c6dc7f2511b98",
    65: "de1e5fa0be70df6d2be8fffd0e99ceaa8eb6e8c93a63f2d8d1c30ecb6b263dee",
    1023: "10108970eeda3eb932baac1428c7a2163b0e924c9a9e25b35bba72b28f70bd11",
    1024: "42214739f095a406f3fc83deb889744ac00df831c10daa55189b5d121c855af7",
    1025: "d00278ae47eb27b34faecf67b4fe263f82d5412916c1ffd97c8cb7fb814b8444",
    2048: "e776b6028c7cd22a4d0ba182a8bf62205d2ef576467e838ed6f2529b85fba24a",
    3072: "b98cb0ff3623be03326b373de6b9095218513e64f1ee2edd2525c7ad1e5cffd2",
}


def _pat(n):
    return bytes(i % 251 for i in range(n))


@pytest.mark.parametrize("n", sorted(BLAKE3_KAT))
def test_blake3_known_answers(oracle, n):
    assert oracle.blake3(_pat(n)).hex() == BLAKE3_KAT[n]


def test_blake3_abc(oracle):
    assert oracle.blake3(b"abc").hex() == \
        "6437b3ac38465133ffb63b75273a8db548c558465d79db03fd359c6cd5bd9d85"


@pytest.mark.parametrize("n", [0, 1, 3, 55, 56, 63, 64, 65, 119, 120, 1000, 3000, 16384])
def test_sha256_matches_hashlib(oracle, n):
    d = os.urandom(n)
    assert oracle.sha256(d) == hashlib.sha256(d).digest()


def test_leaf_cv_is_non_root(oracle):
    data = bytes(range(256)) * 12
    data = data[:3000]
    assert oracle.hash_leaf(data, oracle.BLAKE3) != oracle.blake3(data)
    assert oracle.hash_leaf(data, oracle.SHA256) == hashlib.sha256(data).digest()


def test_pair_hashes(oracle):
    l, r = bytes([7]) * 32, bytes([9]) * 32
    assert oracle.hash_pair(l, r, oracle.SHA256) == hashlib.sha256(l + r).digest()
    # BLAKE3's PARENT flag separates the domains (merkle.rs blake3_separates_...)
    assert oracle.hash_pair(l, r, oracle.BLAKE3) != oracle.hash_leaf(l + r, oracle.BLAKE3)


@pytest.mark.parametrize("kind", [0, 1])
def test_two_leaves_by_hand(oracle, kind):
    data = bytes(range(16))
    tree = oracle.merkle_tree(data, 2, kind)
    h0 = oracle.hash_leaf(data[:8], kind)
    h1 = oracle.hash_leaf(data[8:], kind)
    assert tree[0].tobytes() == h0 and tree[1].tobytes() == h1
    assert tree[2].tobytes() == oracle.hash_pair(h0, h1, kind)


@pytest.mark.parametrize("kind", [0, 1])
def test_one_leaf_root_is_leaf_hash(oracle, kind):
    data = bytes(range(32))
    assert oracle.merkle_tree(data, 1, kind)[-1].tobytes() == oracle.hash_leaf(data, kind)


@pytest.mark.parametrize("kind", [0, 1])
def test_parallel_matches_sequential(oracle, kind):
    data = os.urandom(1024 * 64)
    a = oracle.merkle_tree(data, 1024, kind, n_threads=1)
    b = oracle.merkle_tree(data, 1024, kind, n_threads=4)
    assert (a == b).all()


def test_kinds_differ(oracle):
    data = os.urandom(64 * 32)
    assert (oracle.merkle_tree(data, 64, 0)[-1] != oracle.merkle_tree(data, 64, 1)[-1]).any()


@pytest.mark.parametrize("kind", [0, 1])
def test_multiproof_round_trip_and_tamper(oracle, kind):
    rng = np.random.default_rng(3)
    n_leaves, leaf = 256, 48
    data = rng.integers(0, 256, n_leaves * leaf, dtype=np.uint8).tobytes()
    tree = oracle.merkle_tree(data, n_leaves, kind)
    root = tree[-1].tobytes()
    for q in (1, 2, 7, 40, 256):
        pos = sorted(set(rng.integers(0, n_leaves, q).tolist()))
        proof = oracle.merkle_multi_proof(tree, n_leaves, pos)
        lh = tree[np.array(pos)]
        assert oracle.verify_merkle_multi_proof(root, n_leaves, pos, lh, proof, kind)
        if len(proof):
            bad = proof.copy()
            bad[0, 0] ^= 1
            assert not oracle.verify_merkle_multi_proof(root, n_leaves, pos, lh, bad, kind)
        # a proof must be consumed exactly
        extra = np.vstack([proof, proof[:1]]) if len(proof) else np.zeros((1, 32), np.uint8)
        assert not oracle.verify_merkle_multi_proof(root, n_leaves, pos, lh, extra, kind)
    # all leaves opened: empty proof
    allp = list(range(n_leaves))
    assert len(oracle.merkle_multi_proof(tree, n_leaves, allp)) == 0
    assert len(oracle.merkle_multi_proof(tree, n_leaves, [])) == 0
