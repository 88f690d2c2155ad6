"""Process exit with live device objects: a script that commits, opens and
leaves every handle (context, device arrays, commitments, an opening, a batch
plan, a server) for interpreter shutdown must exit cleanly, in either order of
explicit context close and implicit teardown."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
sys.path.insert(0, {repo!r}); sys.path.insert(0, {pkg!r})
import numpy as np
import bitz_gb300 as bz

ctx = bz.Context(0)
msg = bz.DeviceArray.chacha(1, 1 << 12, ctx)
basis = bz.DeviceArray.chacha(2, 1 << 12, ctx)
c, pd = bz.commit(msg, bz.PcsParams(19, 2, 6, 1), ctx)
op = bz.open_l0(bz.Blake3Transcript(), pd, msg, basis, [1, 2], bz.L0Config(6, 3, 2, queries0=8), ctx)
proof = bz.prove(bz.Blake3Transcript(), pd, msg, basis, [1, 2],
                 bz.LigeritoConfig(6, [3], [2, 2], [8, 4], [0, 0]), ctx)
plan = bz.BatchPlan([msg], [bz.PcsParams(19, 2, 6, 1)], ctx=ctx)
plan.launch()
from bitz_gb300 import serve
srv = serve.Server(ctx, n_slots=2)
t = bz.Blake3Transcript()
if {close_first}:
    ctx.close()                       # children released first, then the context
    pd.free(); msg.free(); op.free()  # stale handles after close are ignored
print("done")
"""


@pytest.mark.parametrize("close_first", [False, True])
def test_exit_with_live_handles(close_first):
    code = SCRIPT.format(repo=REPO, pkg=os.path.join(REPO, "bitz-poc_gb300"),
                         close_first=close_first)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    assert "done" in r.stdout
