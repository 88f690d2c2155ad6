"""Persistent batch plans: every commit of a batch runs as work items of one
persistent kernel; each root, tree and codeword must equal the commit made
alone (and the oracle's)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def own_ctx():
    """A private context, so schedules set here reach no other test."""
    from bitz_gb300.pcs import Context

    c = Context(0)
    yield c
    c.close()


# (log_msg_len, log_inv_rate, log_batch_size, hash): radix-8 shapes (>= 512
# lanes, leftover layers first or last), table passes + deep pass (256 lanes),
# short BLAKE3 leaves (< 64 lanes), SHA-256 trees, shapes small enough for the
# single-launch NTT (generic layers here), rates 1/2 .. 1/8.
MIX = [(20, 2, 10, 1), (18, 2, 9, 1), (16, 2, 8, 1), (17, 2, 8, 1), (19, 2, 9, 1),
       (21, 2, 10, 1), (14, 2, 7, 1), (12, 1, 6, 1), (13, 3, 4, 1), (15, 2, 7, 0),
       (12, 2, 9, 1), (10, 2, 5, 0), (19, 1, 10, 1), (16, 3, 8, 1), (11, 2, 2, 1)]


def _single(ctx, msgs, params):
    from bitz_gb300 import commit

    out = []
    for m, p in zip(msgs, params):
        c, pd = commit(m, p, ctx)
        out.append((c.root, pd.codeword))
        pd.free()
    return out


def test_persistent_plan_matches_single(ctx):
    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams

    params = [PcsParams(lm + 7, r, lb, h) for (lm, r, lb, h) in MIX]
    msgs = [DeviceArray.chacha(300 + i, 1 << lm, ctx) for i, (lm, _, _, _) in enumerate(MIX)]
    single = _single(ctx, msgs, params)
    plan = BatchPlan(msgs, params, ctx=ctx, persistent=True)
    try:
        for rep in range(3):  # the graph resets the scheduler state every launch
            plan.launch()
            roots = plan.roots()
            for i in range(len(msgs)):
                assert roots[i] == single[i][0], (rep, MIX[i])
        for i in range(len(msgs)):
            assert (plan.codeword(i) == single[i][1]).all(), MIX[i]
    finally:
        plan.close()
        for m in msgs:
            m.free()


@pytest.mark.parametrize("schedule", [0x8000, 0x18000, 3, 2, 0x13, 2 | (1 << 7), 0x5000,
                                      0x5001, 0x1002, 0x20, 0x42, (2 << 10) | 0x200 | 2,
                                      0x208000, 0x4010])
def test_persistent_plan_follows_schedules(oracle, own_ctx, schedule):
    """The context's schedule per shape picks the plan's passes; every
    schedule the library accepts gives the oracle's roots."""
    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams

    shapes = [(18, 2, 9), (17, 2, 8), (14, 1, 7), (19, 3, 9)]
    params = [PcsParams(lm + 7, r, lb, 1) for (lm, r, lb) in shapes]
    hosts = [oracle.chacha_words(700 + i, 1 << lm) for i, (lm, _, _) in enumerate(shapes)]
    msgs = [DeviceArray.from_host(h, own_ctx) for h in hosts]
    for p in params:
        own_ctx.set_schedule(p, schedule)
    plan = BatchPlan(msgs, params, ctx=own_ctx, persistent=True)
    try:
        plan.launch()
        roots = plan.roots()
        for i, (lm, r, lb) in enumerate(shapes):
            cw, _, root = oracle.commit(hosts[i], r, lb, 1, n_threads=8)
            assert roots[i] == root, shapes[i]
            assert (plan.codeword(i) == cw).all(), shapes[i]
    finally:
        plan.close()
        for m in msgs:
            m.free()


def test_persistent_plan_mixed_sizes_like_the_batched_benchmark(own_ctx):
    """Square-ish 2^floor(n/2) x 2^ceil(n/2) matrices, n uniform on [16, 21],
    autotuned schedules: roots equal the one-at-a-time commits."""
    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams

    rng = np.random.default_rng(3)
    sizes = [int(x) for x in rng.integers(16, 22, 24)]
    params = [PcsParams(n + 7, 2, n // 2, 1) for n in sizes]
    for p in {(p.m, p.log_batch_size): p for p in params}.values():
        own_ctx.autotune(p, reps=1)
    msgs = [DeviceArray.chacha(3000 + i, 1 << n, own_ctx) for i, n in enumerate(sizes)]
    single = _single(own_ctx, msgs, params)
    plan = BatchPlan(msgs, params, ctx=own_ctx, persistent=True)
    try:
        for _ in range(2):
            plan.launch()
        roots = plan.roots()
        assert roots == [s[0] for s in single]
    finally:
        plan.close()
        for m in msgs:
            m.free()


def test_persistent_plan_rejects_unsupported_shapes(ctx):
    from bitz_gb300 import BatchPlan, BzError, DeviceArray, PcsParams

    ok = DeviceArray.chacha(1, 1 << 12, ctx)
    wide = DeviceArray.chacha(2, 1 << 16, ctx)
    try:
        for m, p in ((wide, PcsParams(16 + 7, 2, 15, 1)),   # BLAKE3 leaves of 512 chunks
                     (ok, PcsParams(12 + 7, 2, 12, 1))):     # one column: no NTT layer
            with pytest.raises(BzError) as e:
                BatchPlan([ok, m], [PcsParams(12 + 7, 2, 6, 1), p], ctx=ctx, persistent=True)
            assert e.value.status == 2
    finally:
        ok.free()
        wide.free()


def test_persistent_plan_single_commit_2e22(ctx):
    """One 2^22-element commit (2^11 x 2^11, rate 1/4) as a persistent plan,
    launched three times: the root equals the plain commit's (the workload of
    the persistent kernel's ncu profile)."""
    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams, commit

    p = PcsParams(22 + 7, 2, 11, 1)
    m = DeviceArray.chacha(100, 1 << 22, ctx)
    plan = BatchPlan([m], [p], ctx=ctx, persistent=True)
    try:
        for _ in range(3):
            plan.launch()
        root = plan.roots()[0]
        c, pd = commit(m, p, ctx)
        pd.free()
        assert root == c.root
    finally:
        plan.close()
        m.free()


def test_persistent_plan_bounded_wait_reports_and_recovers(ctx):
    """A launch that waits for a step no item completes: every CTA gives up
    after the 30 ms limit, the host reads BZ_ERR_TIMEOUT, and the plan's next
    launches still give the single commits' roots."""
    import ctypes

    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams, _lib, commit

    L = _lib.lib()
    L.bz_batch_plan_stall_check.restype = ctypes.c_int
    L.bz_batch_plan_stall_check.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
    params = [PcsParams(18 + 7, 2, 9, 1), PcsParams(14 + 7, 2, 7, 1)]
    msgs = [DeviceArray.chacha(900 + i, 1 << (p.m - 7), ctx) for i, p in enumerate(params)]
    plan = BatchPlan(msgs, params, ctx=ctx, persistent=True)
    graph_plan = BatchPlan(msgs, params, ctx=ctx)
    try:
        assert L.bz_batch_plan_stall_check(plan.h, 30) == 6          # BZ_ERR_TIMEOUT
        assert L.bz_batch_plan_stall_check(graph_plan.h, 30) == 1    # not persistent
        plan.launch()
        roots = plan.roots()
        for m, p, r in zip(msgs, params, roots):
            c, pd = commit(m, p, ctx)
            pd.free()
            assert r == c.root
    finally:
        plan.close()
        graph_plan.close()
        for m in msgs:
            m.free()


@pytest.mark.parametrize("persistent", [True, False])
def test_plan_recommits_changed_messages(oracle, ctx, persistent):
    """A plan recommits its device messages at every launch: after the
    messages are overwritten in place, the next launch's roots are the new
    messages' (the persistent kernel's scheduler state restarts each launch)."""
    import ctypes

    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams, _lib

    L = _lib.lib()
    shapes = [(16, 2, 8), (18, 2, 9)]
    params = [PcsParams(lm + 7, r, lb, 1) for (lm, r, lb) in shapes]
    msgs = [DeviceArray.from_host(oracle.chacha_words(40 + i, 1 << lm), ctx)
            for i, (lm, _, _) in enumerate(shapes)]
    plan = BatchPlan(msgs, params, ctx=ctx, persistent=persistent)
    try:
        plan.launch()
        first = plan.roots()
        for seed in (50, 60):
            new = [oracle.chacha_words(seed + i, 1 << lm) for i, (lm, _, _) in enumerate(shapes)]
            for m, h in zip(msgs, new):
                _lib.check(ctx.handle, L.bz_memcpy_h2d(ctx.handle, ctypes.c_void_p(m.ptr.value),
                                                       h.ctypes.data_as(ctypes.c_void_p),
                                                       h.nbytes))
            plan.launch()
            roots = plan.roots()
            for i, (lm, r, lb) in enumerate(shapes):
                assert roots[i] == oracle.commit(new[i], r, lb, 1, n_threads=8)[2]
                assert roots[i] != first[i]
    finally:
        plan.close()
        for m in msgs:
            m.free()
