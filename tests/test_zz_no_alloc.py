"""The allocation-free fold entry point (bz_fold_and_msg_lsb_static).

It serves callers that cannot allocate device memory -- a prover host whose
runtime reserved the GPU's memory for its own pool, or a fold loop that
cannot pay for cudaMalloc's synchronisation -- by keeping the fold's per-block
scratch in a fixed device array.  This test calls it through the C ABI and
checks it against the allocating entry point (bz_fold_and_msg_lsb) on calls
in a row, so stale scratch from an earlier call would show up in a later one,
and against the CPU oracle's fold_and_msg_lsb directly, so a fault the two
GPU paths shared would show up too.  Results are exact (bit-identical) field
values.

The file name sorts last so that a run stopping at its first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alloc(L, ctx, nbytes):
    p = ctypes.c_void_p()
    assert L.bz_device_alloc(ctx.handle, nbytes, ctypes.byref(p)) == 0
    return p


def _run_pair(L, ctx, f, b, r):
    from bitz_gb300 import _lib

    n = f.shape[0]
    half = n // 2
    d_f, d_b = _alloc(L, ctx, f.nbytes), _alloc(L, ctx, b.nbytes)
    assert L.bz_memcpy_h2d(ctx.handle, d_f, _lib.ptr(f), f.nbytes) == 0
    assert L.bz_memcpy_h2d(ctx.handle, d_b, _lib.ptr(b), b.nbytes) == 0
    outs = [_alloc(L, ctx, half * 16) for _ in range(4)]
    d_msg = _alloc(L, ctx, 32)
    u0, u2 = np.zeros(2, np.uint64), np.zeros(2, np.uint64)
    # allocating entry point
    assert L.bz_fold_and_msg_lsb(ctx.handle, d_f, d_b, n, _lib.ptr(r), outs[0], outs[1],
                                 _lib.ptr(u0), _lib.ptr(u2)) == 0
    # allocation-free entry point, on the context's stream
    rc = L.bz_fold_and_msg_lsb_static(d_f, d_b, n, _lib.ptr(r), outs[2], outs[3], d_msg,
                                      L.bz_ctx_stream(ctx.handle))
    assert rc == 0
    assert L.bz_ctx_synchronize(ctx.handle) == 0
    host = []
    for o in outs:
        a = np.zeros((half, 2), np.uint64)
        assert L.bz_memcpy_d2h(ctx.handle, _lib.ptr(a), o, a.nbytes) == 0
        host.append(a)
    msg = np.zeros(4, np.uint64)
    assert L.bz_memcpy_d2h(ctx.handle, _lib.ptr(msg), d_msg, 32) == 0
    for p in [d_f, d_b, d_msg, *outs]:
        L.bz_device_free(ctx.handle, p)
    return host, u0, u2, msg


def test_static_fold_matches_allocating_fold_twice(ctx, oracle):
    from bitz_gb300 import _lib

    L = _lib.lib()
    rng = np.random.default_rng(2024)
    # calls in a row: a large fold, then smaller ones whose few blocks must
    # not pick up an earlier call's partial sums; n = 2 folds one pair (one
    # thread, empty message), n = 4 leaves a single folded pair
    for n in (1 << 18, 1 << 10, 2, 4):
        f = rng.integers(0, 2**64, (n, 2), dtype=np.uint64)
        b = rng.integers(0, 2**64, (n, 2), dtype=np.uint64)
        r = rng.integers(0, 2**64, 2, dtype=np.uint64)
        (nf, nb, nf_s, nb_s), u0, u2, msg = _run_pair(L, ctx, f, b, r)
        assert (nf_s == nf).all() and (nb_s == nb).all()
        assert (msg[:2] == u0).all() and (msg[2:] == u2).all()
        if n <= 1 << 10:
            # the CPU oracle, independently of either GPU path
            ef, eb, e0, e2 = oracle.fold_and_msg_lsb(f, b, r)
            assert (nf_s == ef).all() and (nb_s == eb).all()
            assert (msg[:2] == e0).all() and (msg[2:] == e2).all()


def test_static_fold_rejects_bad_sizes(ctx):
    from bitz_gb300 import _lib

    L = _lib.lib()
    r = np.zeros(2, np.uint64)
    dummy = ctypes.c_void_p(16)
    for n in (0, 1, 3, 1000, (1 << 40) * 2):
        assert L.bz_fold_and_msg_lsb_static(dummy, dummy, n, _lib.ptr(r), dummy, dummy, dummy,
                                            None) == 2
