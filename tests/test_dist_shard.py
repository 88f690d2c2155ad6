"""The lane-sharded BLAKE3 commit's data path on CPU ranks (gloo, world 2 and 4).

Each rank encodes its lane shard and reduces every row to the CV of its run of
chunks with the CPU oracle (no GPU here), then runs the library's own exchange
code (bitz_gb300.shard: all-gather of per-position CVs in rank order, gather of
opened-row slices).  The tree built from the gathered CVs must be the
single-process commit's tree, and the gathered rows its rows: the sharded
commit is the same commit (flock-core/src/pcs/commit.rs:180-315), split by
lanes.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, {repo!r})
sys.path.insert(0, os.path.join({repo!r}, "bitz-poc_gb300"))
import numpy as np
import torch.distributed as dist
from oracle import oracle as O
from bitz_gb300 import shard as S
from bitz_gb300.pcs import PcsParams, HashKind

dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
lm, r, lb, seed = {lm}, {r}, {lb}, {seed}
params = PcsParams(lm + 7, r, lb, HashKind.BLAKE3)
msg = O.chacha_words(seed, 1 << lm)
shard_msg = S.lane_shard(msg, params, world, rank)
assert (shard_msg == O.lane_shard(msg, lb, world, rank)).all()
cw, cvs = O.commit_lane_shard(shard_msg, r, lb, world, rank)
tree, root = S.sharded_root(cvs, combine=O.merkle_from_shard_cvs)
pos = [0, 3, 5, (1 << (lm - lb + r)) - 1]
ls = (1 << lb) // world
rows = S.gather_rows(np.ascontiguousarray(cw.reshape(-1, ls, 2)[pos]))
with open(os.path.join({out!r}, "rank%d.json" % rank), "w") as fh:
    json.dump({{"root": root.hex(), "tree_sum": int(tree.astype(np.uint64).sum()),
               "rows": rows.tolist()}}, fh)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world,shape", [(2, (14, 2, 7, 3)), (4, (16, 2, 8, 1)),
                                         (2, (13, 1, 8, 5))])
def test_lane_sharded_commit_equals_single_commit(tmp_path, oracle, world, shape):
    pytest.importorskip("torch")
    lm, r, lb, seed = shape
    script = tmp_path / "worker.py"
    script.write_text(WORKER.format(repo=REPO, out=str(tmp_path), lm=lm, r=r, lb=lb, seed=seed))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node",
           str(world), "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(script)]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=REPO,
                         env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert res.returncode == 0, res.stderr[-3000:]
    msg = oracle.chacha_words(seed, 1 << lm)
    cw, tree, root = oracle.commit(msg, r, lb, oracle.BLAKE3)
    pos = [0, 3, 5, (1 << (lm - lb + r)) - 1]
    want_rows = cw.reshape(-1, 1 << lb, 2)[pos]
    for k in range(world):
        got = json.loads((tmp_path / f"rank{k}.json").read_text())
        assert got["root"] == root.hex()                       # every rank has the root
        assert got["tree_sum"] == int(tree.astype(np.uint64).sum())
        assert (np.array(got["rows"], dtype=np.uint64) == want_rows).all()


def test_shard_shapes_are_checked():
    from bitz_gb300 import shard as S
    from bitz_gb300.pcs import HashKind, PcsParams

    with pytest.raises(ValueError):
        S.shard_params(PcsParams(21, 2, 7, HashKind.SHA256), 2)   # SHA-256: replicas only
    with pytest.raises(ValueError):
        S.shard_params(PcsParams(21, 2, 7, HashKind.BLAKE3), 4)   # 32 lanes per rank
    with pytest.raises(ValueError):
        S.shard_params(PcsParams(21, 2, 8, HashKind.BLAKE3), 3)   # not a power of two
    p = S.shard_params(PcsParams(31, 2, 12, HashKind.BLAKE3), 4)
    assert (p.log_msg_len(), p.log_batch_size, p.k_code()) == (22, 10, 14)
