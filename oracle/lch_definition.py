"""The Reed-Solomon codeword of the commit, computed from its definition.

Test infrastructure only: nothing in the library imports this module.

This restates the definitions of Lin, Chung and Han, "Novel polynomial basis
and its application to Reed-Solomon erasure codes" (FOCS 2014), not the
reference's code.  It is a second derivation, independent of the reference,
of what the additive NTT of the commit computes
(flock-core/src/ntt/additive_ntt_f128.rs:63-156, 243-274 with the basis
{1, x, .., x^(ell-1)} of :136-140):

* the field is GF(2)[X] / (X^128 + X^7 + X^2 + X + 1); element bit i is the
  coefficient of X^i;
* the evaluation subspace V_ell = span{1, X, .., X^(ell-1)}, so the point
  omega_p of codeword position p is the element whose bits are those of p;
* subspace polynomial W_i(y) = prod_{u in V_i} (y - u), normalised
  What_i(y) = W_i(y) / W_i(X^i);
* novel basis X_j(y) = prod_{i : bit i of j} What_i(y);
* a message m_0 .. m_{2^k - 1} is the polynomial P(y) = sum_j m_j X_j(y), and
  its codeword at rate 2^-r is P(omega_p) for p < 2^(k + r).

Everything is Python integers and loops: sizes up to a few hundred points.
"""
from __future__ import annotations

_MOD = (1 << 128) | 0x87


def mul(a: int, b: int) -> int:
    """Shift-and-add product in GF(2^128)."""
    r = 0
    while b:
        if b & 1:
            r ^= a
        b >>= 1
        a <<= 1
        if a >> 128:
            a ^= _MOD
    return r


def inv(a: int) -> int:
    """a^(2^128 - 2)."""
    if a == 0:
        raise ZeroDivisionError("0 has no inverse")
    r, e = 1, (1 << 128) - 2
    while e:
        if e & 1:
            r = mul(r, a)
        a = mul(a, a)
        e >>= 1
    return r


def subspace_poly(i: int, y: int) -> int:
    """W_i(y): the product of (y + u) over the 2^i elements u of V_i."""
    r = 1
    for u in range(1 << i):
        r = mul(r, y ^ u)
    return r


def basis_matrix(k: int, ell: int) -> list[list[int]]:
    """X_j(omega_p) for p < 2^ell (rows) and j < 2^k (columns)."""
    norm = [inv(subspace_poly(i, 1 << i)) for i in range(k)]
    rows = []
    for p in range(1 << ell):
        what = [mul(subspace_poly(i, p), norm[i]) for i in range(k)]
        row = []
        for j in range(1 << k):
            x = 1
            for i in range(k):
                if (j >> i) & 1:
                    x = mul(x, what[i])
            row.append(x)
        rows.append(row)
    return rows


def codeword(message: list[int], log_inv_rate: int) -> list[int]:
    """P(omega_p) for every position p of the rate 2^-log_inv_rate code."""
    k = len(message).bit_length() - 1
    assert len(message) == 1 << k
    ell = k + log_inv_rate
    out = []
    for row in basis_matrix(k, ell):
        s = 0
        for mj, x in zip(message, row):
            s ^= mul(mj, x)
        out.append(s)
    return out


def interleaved_codeword(message: list[int], log_lanes: int, log_inv_rate: int) -> list[int]:
    """The commit's codeword of a message laid out msg[j * L + lane]: every
    lane is encoded on its own, output cw[p * L + lane]."""
    L = 1 << log_lanes
    n = len(message) // L
    k = n.bit_length() - 1
    assert n == 1 << k and n * L == len(message)
    mat = basis_matrix(k, k + log_inv_rate)
    out = [0] * (len(mat) * L)
    for lane in range(L):
        col = message[lane::L]
        for p, row in enumerate(mat):
            s = 0
            for mj, x in zip(col, row):
                s ^= mul(mj, x)
            out[p * L + lane] = s
    return out
