"""The oracle's NTT and commit codeword against the Reed-Solomon definition.

`oracle/lch_definition.py` evaluates the message polynomial in the
Lin-Chung-Han novel basis at every point of span{1, X, .., X^(ell-1)} from the
definitions alone (subspace polynomials, normalisation, basis products).  The
reference's additive NTT (flock-core/src/ntt/additive_ntt_f128.rs) computes
that encoding; agreement here pins the oracle's transform, its replicate-fill
start at layer r and the interleaved layout to the definition, not only to
self-consistency."""
import numpy as np
import pytest

from oracle import lch_definition as D


def _ints(words):
    return [int(w[0]) | (int(w[1]) << 64) for w in np.asarray(words, np.uint64).reshape(-1, 2)]


def _words(ints):
    return np.array([[x & (2**64 - 1), x >> 64] for x in ints], np.uint64)


def test_definition_field_matches_oracle(oracle):
    rng = np.random.default_rng(11)
    for _ in range(50):
        a, b = _ints(rng.integers(0, 2**64, (2, 2), dtype=np.uint64))
        assert D.mul(a, b) == oracle.gf_int(oracle.gf_mul(a, b))
    a = (1 << 127) | 12345
    assert D.mul(a, D.inv(a)) == 1


def test_subspace_polynomial_vanishes_on_its_subspace():
    for i in range(1, 5):
        for u in range(1 << i):
            assert D.subspace_poly(i, u) == 0
        assert D.subspace_poly(i, 1 << i) != 0


@pytest.mark.parametrize("k,r", [(0, 1), (1, 1), (2, 1), (3, 2), (4, 2), (5, 1), (3, 3), (6, 2)])
def test_ntt_equals_novel_basis_evaluation(oracle, k, r):
    rng = np.random.default_rng(0x1C4 + 16 * k + r)
    msg = rng.integers(0, 2**64, (1 << k, 2), dtype=np.uint64)
    padded = np.zeros((1 << (k + r), 2), np.uint64)
    padded[: 1 << k] = msg
    got = _ints(oracle.ntt_forward(padded))
    assert got == D.codeword(_ints(msg), r)


@pytest.mark.parametrize("m,r,lb", [(3, 1, 1), (5, 2, 2), (6, 1, 3), (6, 2, 4), (4, 3, 1)])
def test_commit_codeword_equals_definition(oracle, m, r, lb):
    msg = oracle.chacha_words(300 + 10 * m + r, 1 << m)
    cw, _, _ = oracle.commit(msg, r, lb, 1)
    assert _ints(cw) == D.interleaved_codeword(_ints(msg), lb, r)
