"""Oracle folds and ring-switch passes, restating the reference identities
(flock-core/src/pcs/ligerito.rs fold tests; BitZ src/ligerito.rs:881-894 and
the recombination identity asserted at src/ligerito.rs:488-494)."""
import numpy as np
import pytest


def _rand(rng, n):
    return rng.integers(0, 2**64, (n, 2), dtype=np.uint64)


@pytest.mark.parametrize("n", [2, 4, 8, 64, 1024])
def test_fold_and_msg_matches_unfused(oracle, n):
    rng = np.random.default_rng(n)
    f, b, r = _rand(rng, n), _rand(rng, n), _rand(rng, 1)[0]
    nf, nb, u0, u2 = oracle.fold_and_msg_lsb(f, b, r)
    assert (nf == oracle.partial_eval_lsb(f, r.reshape(1, 2))).all()
    assert (nb == oracle.partial_eval_lsb(b, r.reshape(1, 2))).all()
    if n >= 4:
        e0, e2 = oracle.round_msg_lsb(nf, nb)
        assert (u0 == e0).all() and (u2 == e2).all()
    else:
        assert (u0 == 0).all() and (u2 == 0).all()


def test_partial_eval_composes(oracle):
    rng = np.random.default_rng(9)
    f = _rand(rng, 256)
    rs = _rand(rng, 5)
    once = oracle.partial_eval_lsb(f, rs)
    step = f
    for i in range(5):
        step = oracle.partial_eval_lsb(step, rs[i:i + 1])
    assert (once == step).all()
    # full evaluation equals <f, eq(point)>
    full = oracle.partial_eval_lsb(f, _rand(rng, 8))
    assert full.shape == (1, 2)


def test_mle_eval_is_inner_product_with_eq(oracle):
    rng = np.random.default_rng(11)
    f, pt = _rand(rng, 64), _rand(rng, 6)
    v = oracle.partial_eval_lsb(f, pt)[0]
    eq = oracle.build_eq_lsb(pt)
    acc = np.zeros(2, np.uint64)
    for i in range(64):
        acc ^= oracle.gf_mul(f[i], eq[i])
    assert (acc == v).all()


def test_round_msg_sum_check(oracle):
    # u(0) + u(1) = sum f*b, with u(1) = u0 + u1 + u2 and u1 recovered by the
    # sumcheck constraint; here check u0 and u2 against their definitions.
    rng = np.random.default_rng(4)
    f, b = _rand(rng, 32), _rand(rng, 32)
    u0, u2 = oracle.round_msg_lsb(f, b)
    a0 = np.zeros(2, np.uint64)
    a2 = np.zeros(2, np.uint64)
    for j in range(16):
        a0 ^= oracle.gf_mul(f[2 * j], b[2 * j])
        a2 ^= oracle.gf_mul(f[2 * j] ^ f[2 * j + 1], b[2 * j] ^ b[2 * j + 1])
    assert (u0 == a0).all() and (u2 == a2).all()


def test_ring_switch_recombination_identity(oracle):
    """sum_y Phi(eq_hi[y]) * P[y] == sum_u eq_r2[u] * s_u where s_u is the
    bit transpose of s_v (src/ligerito.rs:462-494)."""
    rng = np.random.default_rng(21)
    k = 6
    P = _rand(rng, 1 << k)
    eq_hi = oracle.build_eq_lsb(_rand(rng, k))
    sv = oracle.sv_fold(P, eq_hi)
    eq_r2 = oracle.build_eq_lsb(_rand(rng, 7))
    phi = oracle.phi_from_words(eq_hi, eq_r2)
    lhs = np.zeros(2, np.uint64)
    for y in range(1 << k):
        lhs ^= oracle.gf_mul(phi[y], P[y])
    # s_u[u] has bit v = bit u of s_v[v]
    su = np.zeros((128, 2), np.uint64)
    for u in range(128):
        val = 0
        for v in range(128):
            w = int(sv[v][u >> 6])
            if (w >> (u & 63)) & 1:
                val |= 1 << v
        su[u] = [val & (2**64 - 1), val >> 64]
    rhs = np.zeros(2, np.uint64)
    for u in range(128):
        rhs ^= oracle.gf_mul(eq_r2[u], su[u])
    assert (lhs == rhs).all()
