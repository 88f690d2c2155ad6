"""Batched CUDA-graph commits and the error contract of the C ABI."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_single(oracle, ctx):
    from bitz_gb300 import DeviceArray, PcsParams, commit, commit_batch

    rng = np.random.default_rng(3)
    params, msgs = [], []
    for i in range(12):
        n = int(rng.integers(10, 19))
        a, b = n // 2, n - n // 2
        params.append(PcsParams(n + 7, 2, a, 1))
        msgs.append(DeviceArray.chacha(1000 + i, 1 << n, ctx))
    for use_graph in (True, False):
        res = commit_batch(msgs, params, use_graph=use_graph, ctx=ctx)
        for (c, pd), m, p in zip(res, msgs, params):
            c1, pd1 = commit(m, p, ctx)
            assert c.root == c1.root
            assert (pd.codeword == pd1.codeword).all()
            pd.free()
            pd1.free()


def test_bad_shapes_and_state(ctx):
    from bitz_gb300 import BzError, DeviceArray, PcsParams, commit
    from bitz_gb300 import _lib

    with pytest.raises(ValueError):
        commit(np.zeros((16, 2), np.uint64), PcsParams(11, 0, 2), ctx)
    L = _lib.lib()
    p = _lib.Params(4, 1, 6, 0)                   # log_batch_size > log_msg_len
    h = ctypes.c_void_p()
    buf = np.zeros((16, 2), np.uint64)
    root = (ctypes.c_uint8 * 32)()
    assert L.bz_commit(ctx.handle, _lib.ptr(buf), 16, ctypes.byref(p), ctypes.byref(h), root) == 2
    p = _lib.Params(4, 1, 2, 7)                   # bad hash kind
    assert L.bz_commit(ctx.handle, _lib.ptr(buf), 16, ctypes.byref(p), ctypes.byref(h), root) == 1
    p = _lib.Params(4, 1, 2, 0)                   # wrong length
    assert L.bz_commit(ctx.handle, _lib.ptr(buf), 15, ctypes.byref(p), ctypes.byref(h), root) == 2
    c, pd = commit(buf, PcsParams(11, 1, 2, 0), ctx)
    pd.free()
    assert L.bz_commitment_free(pd.handle or h) in (1, 7)


def test_memory_budget_admission():
    from bitz_gb300 import BzError, Context, DeviceArray, PcsParams, commit

    small = Context(0, mem_budget_bytes=64 << 20)
    p = PcsParams(20 + 7, 2, 10, 1)               # 64 MiB codeword + tree > budget
    msg = DeviceArray.chacha(1, 1 << 20, small)
    with pytest.raises(BzError) as e:
        commit(msg, p, small)
    assert e.value.status == 4
    used, budget = small.memory()
    assert used == 0 and budget == 64 << 20
    p2 = PcsParams(16 + 7, 2, 8, 1)               # 4 MiB fits
    c, pd = commit(DeviceArray.chacha(1, 1 << 16, small), p2, small)
    assert small.memory()[0] > 0
    pd.free()
    assert small.memory()[0] == 0
    msg.free()
    small.close()


def test_autotune_picks_a_valid_schedule(oracle, ctx):
    from bitz_gb300 import PcsParams, commit

    p = PcsParams(16 + 7, 2, 8, 1)
    s = ctx.autotune(p, reps=2)
    assert ctx.schedule(p) == s
    msg = oracle.chacha_words(8, 1 << 16)
    _, _, root = oracle.commit(msg, 2, 8, 1, n_threads=8)
    c, pd = commit(msg, p, ctx)
    assert c.root == root
    pd.free()
