"""Oracle bit-matrix ingest against the definitions (CPU).

repack_leaf_bits: bit b of column c's row is cell (b, c); packed columns:
bit k of word i of group g is column 64g+k's bit i; rows_from_packed_cols
inverts it (the reference's round-trip property, src/ligerito.rs:690-717);
the packed message is {row[2i], row[2i+1]} column after column."""
import numpy as np
import pytest

from oracle import ingest as I

SHAPES = [(0, 0), (3, 2), (6, 6), (7, 5), (8, 7), (10, 3), (9, 8), (12, 1)]


def _cells(rng, rv, cv):
    cells = np.zeros((1 << (rv + cv), 2), np.uint64)
    cells[:, 0] = rng.integers(0, 2, 1 << (rv + cv))
    return cells


@pytest.mark.parametrize("rv,cv", SHAPES)
def test_repack_and_transposes(rv, cv):
    rng = np.random.default_rng(rv * 31 + cv)
    cells = _cells(rng, rv, cv)
    rows = I.repack_leaf_bits(cells, rv, cv)
    assert rows.shape == (1 << cv, max(((1 << rv) + 63) // 64, 1))
    for c in range(1 << cv):
        for b in range(1 << rv):
            assert (int(rows[c][b >> 6]) >> (b & 63)) & 1 == int(cells[(b << cv) | c, 0])
    pk = I.pack_columns_from_rows(rows, rv, cv)
    for g in range(pk.shape[0]):
        for i in range(1 << rv):
            for k in range(64):
                c = 64 * g + k
                exp = (int(rows[c][i >> 6]) >> (i & 63)) & 1 if c < (1 << cv) else 0
                assert (int(pk[g][i]) >> k) & 1 == exp
    assert (I.rows_from_packed_cols(pk, rv, cv) == rows).all()


def test_repack_rejects_non_binary_cells():
    cells = np.zeros((16, 2), np.uint64)
    cells[5, 0] = 2
    with pytest.raises(ValueError):
        I.repack_leaf_bits(cells, 2, 2)
    cells[5] = (0, 1)
    with pytest.raises(ValueError):
        I.repack_leaf_bits(cells, 2, 2)


def test_message_from_rows_layout():
    rng = np.random.default_rng(1)
    rv, cv = 9, 3
    rows = I.repack_leaf_bits(_cells(rng, rv, cv), rv, cv)
    msg = I.message_from_rows(rows, rv, cv)
    assert msg.shape == (1 << (rv - 7 + cv), 2)
    for c in range(1 << cv):
        for i in range(1 << (rv - 7)):
            assert msg[c * (1 << (rv - 7)) + i].tolist() == [rows[c][2 * i], rows[c][2 * i + 1]]
