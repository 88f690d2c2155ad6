"""Bit-matrix ingest on the GPU against the oracle (oracle/ingest.py), and the
commit of the rows (commit_rs_flock_from_rows) against the oracle commit of
the packed message they form."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(0, 0), (3, 2), (6, 6), (7, 5), (8, 7), (10, 3), (9, 8), (12, 1), (14, 10), (16, 6)]


@pytest.mark.parametrize("rv,cv", SHAPES)
def test_ingest_matches_oracle(ctx, rv, cv):
    from bitz_gb300 import ingest as G
    from oracle import ingest as I

    rng = np.random.default_rng(rv * 17 + cv)
    cells = np.zeros((1 << (rv + cv), 2), np.uint64)
    cells[:, 0] = rng.integers(0, 2, 1 << (rv + cv))
    exp_rows = I.repack_leaf_bits(cells, rv, cv)
    exp_pk = I.pack_columns_from_rows(exp_rows, rv, cv)
    d_cells = G.DeviceWords.from_host(cells, ctx)
    rows = G.repack_leaf_bits(d_cells, rv, cv)
    assert (rows.to_host().reshape(exp_rows.shape) == exp_rows).all()
    pk = G.pack_columns_from_rows(rows, rv, cv)
    assert (pk.to_host().reshape(exp_pk.shape) == exp_pk).all()
    back = G.rows_from_packed_cols(pk, rv, cv)
    assert (back.to_host().reshape(exp_rows.shape) == exp_rows).all()
    for a in (d_cells, rows, pk, back):
        a.free()


def test_repack_rejects_non_binary(ctx):
    from bitz_gb300 import BzError
    from bitz_gb300 import ingest as G

    cells = np.zeros((64, 2), np.uint64)
    cells[9, 0] = 3
    d = G.DeviceWords.from_host(cells, ctx)
    with pytest.raises(BzError):
        G.repack_leaf_bits(d, 3, 3)
    d.free()


@pytest.mark.parametrize("rv,cv,r,lb,kind", [(9, 6, 2, 4, 1), (11, 8, 1, 6, 0), (16, 8, 2, 8, 1)])
def test_commit_rows(oracle, ctx, rv, cv, r, lb, kind):
    from bitz_gb300 import ingest as G
    from oracle import ingest as I

    rng = np.random.default_rng(rv + cv)
    words = max(((1 << rv) + 63) // 64, 1)
    rows = rng.integers(0, 2**64, ((1 << cv), words), dtype=np.uint64)
    msg = I.message_from_rows(rows, rv, cv)
    _, _, root = oracle.commit(msg, r, lb, kind)
    d = G.DeviceWords.from_host(rows, ctx)
    c, pd = G.commit_rows(d, rv, cv, r, lb, kind)
    try:
        assert c.root == root
    finally:
        pd.free()
        d.free()
