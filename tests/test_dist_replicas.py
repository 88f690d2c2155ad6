"""The multi-rank host paths of bench.py on CPU (gloo, world size 2).

The commit shards as independent replicas (one polynomial per rank, no
data-path collective); what is collective is the timing: a barrier around
the timed region and the maximum of the per-rank totals.  These tests run
that logic with the gloo backend on two CPU processes, two replica ranks that
each commit their own polynomial (with the CPU oracle) and gather the roots,
and the reference arm under torchrun (rank 0 times and prints one line, rank
1 exits without work).  The lane-sharded single commit is tested in
test_dist_shard.py.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys
sys.path.insert(0, {repo!r})
import bench
ws, rank, local = bench._dist()
d = bench._Dist(ws, local)
d.barrier()
m = d.max(float(10 * (rank + 1)))
d.barrier()
with open(os.path.join({out!r}, "rank%d.txt" % rank), "w") as fh:
    fh.write("rank %d max %s" % (rank, m))
d.close()
"""


REPLICA_WORKER = r"""
import os, sys
sys.path.insert(0, {repo!r})
sys.path.insert(0, os.path.join({repo!r}, "bitz-poc_gb300"))
import bench
from oracle import oracle as O
from bitz_gb300 import shard as S
ws, rank, local = bench._dist()
d = bench._Dist(ws, local)
# each replica commits its own polynomial (seed 1 + rank), as bench.py does
msg = O.chacha_words(1 + rank, 1 << 14)
_, _, root = O.commit(msg, 2, 7, O.BLAKE3)
import numpy as np
roots = S._all_gather(np.frombuffer(root, np.uint8))
if rank == 0:
    with open(os.path.join({out!r}, "roots.txt"), "w") as fh:
        fh.write(" ".join(r.tobytes().hex() for r in roots))
d.close()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=REPO, env=env)


def test_barrier_and_max_over_ranks(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "worker.py"
    script.write_text(WORKER.format(repo=REPO, out=str(tmp_path)))
    r = _torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [(tmp_path / f"rank{i}.txt").read_text() for i in range(2)]
    assert lines == ["rank 0 max 20.0", "rank 1 max 20.0"]


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--log-n", "14",
                   "--steps", "1", "--warmup", "1"])
    assert r.returncode == 0, r.stderr[-3000:]
    out = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(out) == 1                      # rank 0 only
    line = out[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_replica_ranks_commit_their_own_polynomials(tmp_path, oracle):
    """Two ranks each commit their own polynomial (seed 1 + rank) and the
    gathered roots are the single-process roots of those polynomials."""
    pytest.importorskip("torch")
    script = tmp_path / "replicas.py"
    script.write_text(REPLICA_WORKER.format(repo=REPO, out=str(tmp_path)))
    r = _torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-3000:]
    got = (tmp_path / "roots.txt").read_text().split()
    want = [oracle.commit(oracle.chacha_words(1 + k, 1 << 14), 2, 7, oracle.BLAKE3)[2].hex()
            for k in range(2)]
    assert got == want and got[0] != got[1]
