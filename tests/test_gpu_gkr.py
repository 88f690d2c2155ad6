"""The GPU grand-product GKR prover (bz_gkr_*) against the oracle's
restatement of BitZ's dense prover (src/bitz/gkr.rs): every round message,
the roots, the leaf point and the leaf claim are identical for the same
transcript, the oracle's verifier accepts the GPU's transcript, and the leaf
claim is the leaves' multilinear value at the leaf point.  The forest shapes
are the reference's own parity cases (src/bitz/forest_tests.rs:131-157)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _next_word(state):
    # the reference tests' xorshift (forest_tests.rs:14-19)
    x = state[0]
    x ^= (x << 13) & (2**64 - 1)
    x ^= x >> 7
    x ^= (x << 17) & (2**64 - 1)
    state[0] = x
    return x


def _forest_case(t, s, bits="mixed"):
    """The leaf grid, images and zeta of forest_tests.rs:42-80."""
    from oracle import gkr as G

    rows, cols = 1 << t, 1 << s
    st = [(0x9E3779B97F4A7C15 ^ (t << 32) ^ s) & (2**64 - 1)]
    images = np.zeros((rows, 2), np.uint64)
    for row in range(rows):
        if row % 7 == 0:
            images[row] = G.ONE
        else:
            images[row] = [_next_word(st), _next_word(st)]
    groups = (cols + 63) // 64
    packed = np.zeros((groups, rows), np.uint64)
    for g in range(groups):
        for row in range(rows):
            packed[g, row] = {"mixed": lambda: _next_word(st), "zero": lambda: 0,
                              "one": lambda: 2**64 - 1}[bits]()
    zeta = []
    for c in range(s):
        zeta.append(G.ZERO.copy() if c % 3 == 0 else G.ONE.copy() if c % 3 == 1
                    else np.array([_next_word(st), _next_word(st)], np.uint64))
    return packed, images, zeta


def _oracle_run(leaves, groups, zeta, seed):
    from oracle import gkr as G

    roots, wit = G.batched_eval(leaves, groups)
    tr = G.HashChallenges(seed)
    point, claim = G.prove(tr.send, tr.challenge, zeta, wit)
    return roots, point, claim, tr


def _same(a, b):
    return [tuple(int(v) for v in x) for x in a] == [tuple(int(v) for v in x) for x in b]


@pytest.mark.parametrize("t,s,bits", [(4, 6, "mixed"), (5, 6, "mixed"), (6, 9, "mixed"),
                                      (6, 10, "mixed"), (7, 12, "mixed"), (10, 10, "mixed"),
                                      (7, 0, "mixed"), (7, 3, "mixed"), (7, 10, "zero"),
                                      (7, 10, "one")])
def test_forest_prove_matches_oracle(ctx, t, s, bits):
    from bitz_gb300 import gkr as K
    from oracle import gkr as G

    packed, images, zeta = _forest_case(t, s, bits)
    leaves = G.forest_leaves(packed, images, t, s)
    roots, point, claim, otr = _oracle_run(leaves, 1 << s, zeta, b"forest")
    gtr = G.HashChallenges(b"forest")
    groots, gpoint, gclaim = K.forest_prove(packed, images, t, s, zeta, gtr, ctx)
    assert gtr.messages == otr.messages
    assert _same(groots, roots)
    assert _same(gpoint, point)
    assert G.gf_key(gclaim) == G.gf_key(claim)
    assert G.gf_key(gclaim) == G.gf_key(G.mle(leaves, gpoint))
    vt = G.HashChallenges(b"forest")
    vt.messages = gtr.messages
    got = G.verify(vt.recv, vt.challenge, G.mle(groots, zeta), zeta, t)
    assert got is not None and G.gf_key(got[1]) == G.gf_key(gclaim)


@pytest.mark.parametrize("log_n,log_g", [(1, 0), (2, 0), (2, 1), (5, 2), (9, 0), (12, 3),
                                         (16, 5), (18, 1)])
@pytest.mark.parametrize("device", [False, True])
def test_prove_random_leaves_matches_oracle(ctx, log_n, log_g, device):
    from bitz_gb300 import DeviceArray
    from bitz_gb300 import gkr as K
    from oracle import gkr as G

    rng = np.random.default_rng(1000 * log_n + log_g)
    leaves = rng.integers(0, 2**64, (1 << log_n, 2), dtype=np.uint64)
    zeta = [rng.integers(0, 2**64, 2, dtype=np.uint64) for _ in range(log_g)]
    roots, point, claim, otr = _oracle_run(leaves, 1 << log_g, zeta, b"rand")
    gtr = G.HashChallenges(b"rand")
    arg = DeviceArray.from_host(leaves, ctx) if device else leaves
    try:
        groots, gpoint, gclaim = K.prove(arg, 1 << log_g, zeta, gtr, ctx)
    finally:
        if device:
            arg.free()
    assert gtr.messages == otr.messages
    assert _same(groots, roots) and _same(gpoint, point)
    assert G.gf_key(gclaim) == G.gf_key(claim)


def test_gkr_errors_and_callback_failure(ctx):
    from bitz_gb300 import BzError, commit, PcsParams
    from bitz_gb300 import gkr as K
    from oracle import gkr as G

    leaves = np.ones((6, 2), np.uint64)
    with pytest.raises(BzError) as e:
        K.prove(leaves, 1, [], G.HashChallenges(), ctx)        # not a power of two
    assert e.value.status == 2
    with pytest.raises(BzError):
        K.prove(np.ones((8, 2), np.uint64), 8, [G.ONE] * 3, G.HashChallenges(), ctx)

    class Boom(G.HashChallenges):
        def challenge(self, stage):
            if len(self.messages) == 3:
                raise ValueError("transcript refused")
            return super().challenge(stage)

    with pytest.raises(ValueError):
        K.prove(np.ones((64, 2), np.uint64), 2, [G.ONE], Boom(), ctx)
    # the context still works after the aborted proof
    m = np.arange(2 << 10, dtype=np.uint64).reshape(-1, 2)
    c, pd = commit(m, PcsParams(10 + 7, 2, 5, 1), ctx)
    pd.free()
    assert len(c.root) == 32
