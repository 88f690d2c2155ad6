"""Lane-sharded BLAKE3 commit on the GPU (bz_commit_shard, bz_merkle_from_shards).

One GPU plays every rank in turn (the ranks' kernels never wait on one
another; the exchange is a host-side concatenation here and an all-gather
between GPUs).  Checked against the CPU oracle and against the single commit:
each rank's codeword is its lanes of the whole codeword, its leaf CVs are the
oracle's chunk-run CVs, and the tree built from all ranks' CVs is the whole
commit's tree, so its root and multi-proofs are the single commit's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sharded(msg, params, world, ctx):
    from bitz_gb300 import shard as S

    shards = [S.commit_shard(S.lane_shard(msg, params, world, k), params, world, k, ctx)
              for k in range(world)]
    cvs = np.stack([S.leaf_cvs(pd) for pd in shards])
    c, tree = S.merkle_from_shards(cvs, params, ctx)
    return shards, cvs, c, tree


@pytest.mark.parametrize("lm,r,lb,world,seed", [(14, 2, 7, 2, 3), (16, 2, 8, 4, 1),
                                                (13, 1, 8, 2, 5), (18, 3, 9, 8, 2),
                                                (20, 2, 10, 2, 0), (17, 2, 15, 2, 4)])
def test_shard_commit_equals_single_commit(ctx, oracle, lm, r, lb, world, seed):
    import bitz_gb300 as bz
    from bitz_gb300 import shard as S

    params = bz.PcsParams(lm + 7, r, lb, bz.HashKind.BLAKE3)
    msg = oracle.chacha_words(seed, 1 << lm)
    shards, cvs, c, tree = _sharded(msg, params, world, ctx)
    full_c, full = bz.commit(msg, params, ctx)
    assert c.root == full_c.root
    assert (tree.merkle_tree == full.merkle_tree).all()
    cw = full.codeword.reshape(-1, 1 << lb, 2)
    ls = (1 << lb) // world
    for k, pd in enumerate(shards):
        assert (pd.codeword.reshape(-1, ls, 2) == cw[:, k * ls:(k + 1) * ls]).all()
        if lm <= 16:
            _, want = oracle.commit_lane_shard(S.lane_shard(msg, params, world, k), r, lb, world, k)
            assert (cvs[k] == want).all()
    pos = [1, 2, 9, params.n_leaves() - 1]
    assert (tree.multi_proof(pos) == full.multi_proof(pos)).all()
    rows = np.concatenate([pd.rows(pos) for pd in shards], axis=1)
    assert (rows == full.rows(pos)).all()
    for pd in shards:
        pd.free()
    tree.free()
    full.free()


def test_shard_commit_headline_shape(ctx):
    """2^24 elements (2^12 x 2^12, rate 1/4) over 4 ranks: the committed
    oracle root of the single commit."""
    import json
    import os

    import bitz_gb300 as bz
    from bitz_gb300 import shard as S

    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "roots.json")) as fh:
        roots = json.load(fh)["roots"]
    want = [e["root"] for e in roots if e["log_msg_len"] == 24 and e["hash"] == "blake3"][0]
    params = bz.PcsParams(31, 2, 12, bz.HashKind.BLAKE3)
    msg = bz.DeviceArray.chacha(1, 1 << 24, ctx).to_host()
    shards, _, c, tree = _sharded(msg, params, 4, ctx)
    assert c.root.hex() == want
    for pd in shards:
        pd.free()
    tree.free()


def test_shard_errors(ctx):
    import ctypes

    import bitz_gb300 as bz
    from bitz_gb300 import _lib

    L = _lib.lib()
    msg = np.zeros((1 << 13, 2), np.uint64)
    h = ctypes.c_void_p()
    for params, world, rank, code in [
            (bz.PcsParams(21, 2, 7, bz.HashKind.SHA256), 2, 0, 2),   # SHA-256: not sharded
            (bz.PcsParams(21, 2, 7, bz.HashKind.BLAKE3), 4, 0, 2),   # 32 lanes per rank
            (bz.PcsParams(21, 2, 8, bz.HashKind.BLAKE3), 3, 0, 1),   # world not a power of two
            (bz.PcsParams(21, 2, 8, bz.HashKind.BLAKE3), 2, 2, 1)]:  # rank >= world
        p = params.to_c()
        n = (1 << params.log_msg_len()) // world
        assert L.bz_commit_shard(ctx.handle, _lib.ptr(msg), n, ctypes.byref(p), world, rank,
                                 ctypes.byref(h)) == code
    # a tree-only handle has no codeword to open rows from
    params = bz.PcsParams(21, 2, 7, bz.HashKind.BLAKE3)
    cvs = np.zeros((2, params.n_leaves(), 32), np.uint8)
    from bitz_gb300 import shard as S

    _, tree = S.merkle_from_shards(cvs, params, ctx)
    with pytest.raises(bz.BzError) as e:
        tree.rows([0])
    assert e.value.status == 7
    tree.free()
