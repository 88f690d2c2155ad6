"""The oracle's restatement of BitZ's dense grand-product GKR (src/bitz/gkr.rs)
against the reference's own checks (src/bitz/forest_tests.rs:42-123): the
proof verifies, the terminal claim is the leaves' multilinear value at the
terminal point, and a changed round message is rejected."""
import numpy as np
import pytest

from oracle import gkr as G


def _field(rng, n):
    return rng.integers(0, 2**64, (n, 2), dtype=np.uint64)


def _zeta(rng, s):
    # coordinates 0, 1 and random, as the reference's parity test picks them
    out = []
    for c in range(s):
        out.append(G.ZERO.copy() if c % 3 == 0 else G.ONE.copy() if c % 3 == 1
                   else _field(rng, 1)[0])
    return out


def _prove_and_verify(leaves, s, rng):
    roots, wit = G.batched_eval(leaves, 1 << s)
    zeta = _zeta(rng, s)
    root_claim = G.mle(roots, zeta)
    tr = G.HashChallenges(b"oracle-gkr")
    point, claim = G.prove(tr.send, tr.challenge, zeta, wit)
    return roots, zeta, root_claim, tr, point, claim, len(wit)


@pytest.mark.parametrize("t,s", [(1, 0), (3, 0), (2, 2), (4, 3), (5, 1), (3, 5), (6, 4)])
def test_dense_gkr_verifies_and_ends_at_the_leaf_mle(t, s):
    rng = np.random.default_rng(100 * t + s)
    leaves = _field(rng, 1 << (t + s))
    roots, zeta, root_claim, tr, point, claim, layers = _prove_and_verify(leaves, s, rng)
    assert layers == t
    assert len(point) == t + s
    assert G.gf_key(claim) == G.gf_key(G.mle(leaves, point))
    # the transcript: one message per round and one per close
    assert len(tr.messages) == sum(k + 1 for k in range(s, s + t))
    vt = G.HashChallenges(b"oracle-gkr")
    vt.messages = tr.messages
    got = G.verify(vt.recv, vt.challenge, root_claim, zeta, t)
    assert got is not None
    assert [G.gf_key(x) for x in got[0]] == [G.gf_key(x) for x in point]
    assert G.gf_key(got[1]) == G.gf_key(claim)


@pytest.mark.parametrize("which", [0, 1, -1])
def test_changed_message_is_rejected(which):
    rng = np.random.default_rng(7)
    t, s = 4, 2
    leaves = _field(rng, 1 << (t + s))
    _, zeta, root_claim, tr, _, _, _ = _prove_and_verify(leaves, s, rng)
    msgs = list(tr.messages)
    st, b = msgs[which]
    msgs[which] = (st, bytes([b[0] ^ 1]) + b[1:])
    vt = G.HashChallenges(b"oracle-gkr")
    vt.messages = msgs
    got = G.verify(vt.recv, vt.challenge, root_claim, zeta, t)
    assert got is None or G.gf_key(got[1]) != G.gf_key(G.mle(leaves, got[0]))


def test_forest_leaves_grid():
    rng = np.random.default_rng(3)
    t, s = 3, 7
    packed = rng.integers(0, 2**64, (2, 8), dtype=np.uint64)
    images = _field(rng, 8)
    leaves = G.forest_leaves(packed, images, t, s)
    for row in range(8):
        for col in range(128):
            bit = (int(packed[col // 64, row]) >> (col % 64)) & 1
            want = images[row] if bit else G.ONE
            assert G.gf_key(leaves[row * 128 + col]) == G.gf_key(want)


def test_product_layers_and_padding():
    rng = np.random.default_rng(4)
    leaves = _field(rng, 13)           # padded with ones to 16
    roots, wit = G.batched_eval(leaves, 2)
    assert [w.shape[0] for w in wit] == [16, 8, 4]
    full = np.concatenate([leaves, np.tile(G.ONE, (3, 1))])
    for g in range(2):
        acc = G.ONE.copy()
        for i in range(g, 16, 2):
            acc = G._mul(acc, full[i])
        assert G.gf_key(acc) == G.gf_key(roots[g])
