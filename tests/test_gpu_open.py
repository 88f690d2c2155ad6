"""Opening-side parity: rows, multi-proofs, folds and ring-switch passes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(rng, n):
    return rng.integers(0, 2**64, (n, 2), dtype=np.uint64)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("lm,r,lb", [(12, 2, 6), (16, 2, 8), (10, 1, 0)])
def test_rows_and_multiproof(oracle, ctx, kind, lm, r, lb):
    from bitz_gb300 import PcsParams, commit

    msg = oracle.chacha_words(17, 1 << lm)
    cw, tree, root = oracle.commit(msg, r, lb, kind)
    c, pd = commit(msg, PcsParams(lm + 7, r, lb, kind), ctx)
    n_leaves = 1 << (lm - lb + r)
    rng = np.random.default_rng(lm)
    try:
        for q in (1, 5, 37, 148):
            pos = sorted(set(rng.integers(0, n_leaves, min(q, n_leaves)).tolist()))
            rows = pd.rows(pos)
            L = 1 << lb
            for i, p in enumerate(pos):
                assert (rows[i] == cw[p * L:(p + 1) * L]).all()
            proof = pd.multi_proof(pos)
            exp = oracle.merkle_multi_proof(tree, n_leaves, pos)
            assert proof.shape == exp.shape and (proof == exp).all()
            leaf_hashes = tree[np.array(pos)]
            assert oracle.verify_merkle_multi_proof(root, n_leaves, pos, leaf_hashes, proof, kind)
        assert len(pd.multi_proof([])) == 0
    finally:
        pd.free()


@pytest.mark.parametrize("n", [2, 4, 8, 1024, 1 << 16, 1 << 20])
def test_fold_and_msg(oracle, ctx, n):
    from bitz_gb300 import DeviceArray
    from bitz_gb300.ligerito import fold_and_msg_lsb, round_msg_lsb

    rng = np.random.default_rng(n)
    f, b, r = _rand(rng, n), _rand(rng, n), _rand(rng, 1)[0]
    df, db = DeviceArray.from_host(f, ctx), DeviceArray.from_host(b, ctx)
    nf, nb, (u0, u2) = fold_and_msg_lsb(df, db, r)
    ef, eb, e0, e2 = oracle.fold_and_msg_lsb(f, b, r)
    assert (nf.to_host() == ef).all() and (nb.to_host() == eb).all()
    assert (u0 == e0).all() and (u2 == e2).all()
    m0, m2 = round_msg_lsb(df, db)
    o0, o2 = oracle.round_msg_lsb(f, b)
    assert (m0 == o0).all() and (m2 == o2).all()


@pytest.mark.parametrize("n", [2, 64, 1 << 12, 1 << 16])
def test_armed_fold_gate(oracle, ctx, n):
    """The armed fold of the prover's small rounds: opened it equals the
    oracle's fold; cancelled it writes nothing; left without a challenge its
    bounded wait runs out (a gate that nothing opens) and the context keeps
    working."""
    from bitz_gb300 import DeviceArray
    from bitz_gb300._lib import BzError
    from bitz_gb300.ligerito import fold_and_msg_lsb, fold_gate_check

    rng = np.random.default_rng(n + 5)
    f, b, r = _rand(rng, n), _rand(rng, n), _rand(rng, 1)[0]
    df, db = DeviceArray.from_host(f, ctx), DeviceArray.from_host(b, ctx)
    ef, eb, e0, e2 = oracle.fold_and_msg_lsb(f, b, r)
    nf, nb, (u0, u2) = fold_gate_check(df, db, r, 0)
    assert (nf.to_host() == ef).all() and (nb.to_host() == eb).all()
    assert (u0 == e0).all() and (u2 == e2).all()
    fold_gate_check(df, db, r, 1)
    with pytest.raises(BzError) as e:
        fold_gate_check(df, db, r, 2, limit_ns=20_000_000)
    assert e.value.status == 6  # BZ_ERR_TIMEOUT
    for _ in range(2):
        nf, nb, (u0, u2) = fold_and_msg_lsb(df, db, r)
        assert (nf.to_host() == ef).all() and (u0 == e0).all() and (u2 == e2).all()
        nf, nb, (u0, u2) = fold_gate_check(df, db, r, 0)
        assert (nb.to_host() == eb).all() and (u0 == e0).all() and (u2 == e2).all()


def test_sumcheck_prover_chain(oracle, ctx):
    """SumcheckProver.new + k folds (the initial_k L0 loop of
    ligerito.rs:3621-3657) against the oracle's chain."""
    from bitz_gb300 import DeviceArray
    from bitz_gb300.ligerito import SumcheckProver

    rng = np.random.default_rng(77)
    n, k = 1 << 14, 12
    f, b = _rand(rng, n), _rand(rng, n)
    prover, msg0 = SumcheckProver.new(DeviceArray.from_host(f, ctx), DeviceArray.from_host(b, ctx), 0)
    e0, e2 = oracle.round_msg_lsb(f, b)
    assert (msg0[0] == e0).all() and (msg0[1] == e2).all()
    cf, cb = f, b
    for i in range(k):
        r = _rand(rng, 1)[0]
        u0, u2 = prover.fold(r)
        cf, cb, x0, x2 = oracle.fold_and_msg_lsb(cf, cb, r)
        assert (u0 == x0).all() and (u2 == x2).all(), i
    assert (prover.f.to_host() == cf).all()


@pytest.mark.parametrize("n,k", [(1024, 1), (1024, 10), (1 << 16, 12), (1 << 20, 3)])
def test_partial_eval(oracle, ctx, n, k):
    from bitz_gb300 import DeviceArray
    from bitz_gb300.ligerito import partial_eval_lsb

    rng = np.random.default_rng(k)
    f, rs = _rand(rng, n), _rand(rng, k)
    out = partial_eval_lsb(DeviceArray.from_host(f, ctx), rs)
    assert (out.to_host() == oracle.partial_eval_lsb(f, rs)).all()


@pytest.mark.parametrize("k", [0, 1, 6, 7, 12, 13, 20, 22, 23])
def test_build_eq(oracle, ctx, k):
    """eq tables: doubling rounds (k <= 6, k > 22) and the split launch
    (lo x hi half tables) give the oracle's entries."""
    from bitz_gb300.ligerito import build_eq_lsb

    pt = _rand(np.random.default_rng(300 + k), k)
    assert (build_eq_lsb(pt, ctx).to_host() == oracle.build_eq_lsb(pt)).all()


@pytest.mark.parametrize("k", [1, 5, 12])
def test_ring_switch_passes(oracle, ctx, k):
    from bitz_gb300 import DeviceArray
    from bitz_gb300.ligerito import build_eq_lsb, phi_from_words, sv_fold

    rng = np.random.default_rng(100 + k)
    pt = _rand(rng, k)
    eq = build_eq_lsb(pt, ctx)
    eq_h = oracle.build_eq_lsb(pt)
    assert (eq.to_host() == eq_h).all()
    P = _rand(rng, 1 << k)
    sv = sv_fold(DeviceArray.from_host(P, ctx), eq)
    assert (sv == oracle.sv_fold(P, eq_h)).all()
    eq_r2 = oracle.build_eq_lsb(_rand(rng, 7))
    phi = phi_from_words(eq, eq_r2)
    assert (phi.to_host() == oracle.phi_from_words(eq_h, eq_r2)).all()
