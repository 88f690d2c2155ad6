"""Serving and batch plans: every result is the same alone and in the mix."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shapes(rng, n, lo=10, hi=18):
    out = []
    for _ in range(n):
        k = int(rng.integers(lo, hi + 1))
        out.append((k, k // 2))
    return out


def test_server_results_equal_alone_and_in_the_mix(oracle, ctx):
    from bitz_gb300 import PcsParams, commit
    from bitz_gb300.serve import COMMITTED, OPENED, Server

    rng = np.random.default_rng(5)
    shapes = _shapes(rng, 24)
    msgs = [oracle.chacha_words(500 + i, 1 << k) for i, (k, _) in enumerate(shapes)]
    params = [PcsParams(k + 7, 2, a, 1) for (k, a) in shapes]
    queries = []
    with Server(ctx, n_slots=4) as srv:
        ids = []
        for i, (m, p) in enumerate(zip(msgs, params)):
            ids.append(srv.submit_commit(m, p))
        for i, rid in enumerate(ids):
            srv.wait(rid, COMMITTED, 120000)
            n_leaves = params[i].n_leaves()
            q = sorted(set(rng.integers(0, n_leaves, 9).tolist()))
            queries.append(q)
            srv.submit_open(rid, q)
        for i, rid in enumerate(ids):
            srv.wait(rid, OPENED, 120000)
            root = srv.root(rid)
            rows, proof = srv.open_result(rid, params[i].num_ntts())
            # alone: the plain commit path and the oracle
            c, pd = commit(msgs[i], params[i], ctx)
            assert root == c.root
            assert (rows == pd.rows(queries[i])).all()
            assert (proof == pd.multi_proof(queries[i])).all()
            pd.free()
            srv.release(rid)
        st = srv.stats()
        assert st["committed"] == 24 and st["opened"] == 24 and st["failed"] == 0
        assert st["in_use"] == 0


def test_commit_open_requests_and_completion_queue(oracle, ctx):
    """submit_commit_open queues the opening itself; the completion queue
    reports every request's COMMITTED and OPENED, and the results equal the
    plain path's."""
    from bitz_gb300 import PcsParams, commit
    from bitz_gb300.serve import COMMITTED, FAILED, OPENED, Server

    rng = np.random.default_rng(9)
    shapes = _shapes(rng, 20, 10, 18)
    msgs = [oracle.chacha_words(900 + i, 1 << k) for i, (k, _) in enumerate(shapes)]
    params = [PcsParams(k + 7, 2, a, 1) for (k, a) in shapes]
    qs = [sorted(set(rng.integers(0, p.n_leaves(), 5).tolist())) for p in params]
    with Server(ctx, n_slots=4) as srv:
        assert srv.next_done(16, 0) == []
        ids = [srv.submit_commit_open(m, p, q) for m, p, q in zip(msgs, params, qs)]
        seen = {rid: [] for rid in ids}
        opened = 0
        deadline = time.time() + 120
        while opened < len(ids) and time.time() < deadline:
            for rid, st in srv.next_done(64, 100000):
                assert st != FAILED
                seen[rid].append(st)
                opened += st == OPENED
        assert opened == len(ids)
        for i, rid in enumerate(ids):
            assert seen[rid] == [COMMITTED, OPENED]
            rows, proof = srv.open_result(rid, params[i].num_ntts())
            c, pd = commit(msgs[i], params[i], ctx)
            assert srv.root(rid) == c.root
            assert (rows == pd.rows(qs[i])).all()
            assert (proof == pd.multi_proof(qs[i])).all()
            pd.free()
            srv.release(rid)
        st = srv.stats()
        assert st["committed"] == 20 and st["opened"] == 20 and st["in_use"] == 0


def test_server_admission_by_memory(oracle, ctx):
    """With a budget that holds one request, the second waits until the first
    is opened (its codeword freed), then runs."""
    from bitz_gb300 import PcsParams
    from bitz_gb300.serve import COMMITTED, OPENED, QUEUED, Server

    p = PcsParams(18 + 7, 2, 9, 1)
    need = (16 << 18) + (16 << 20) + 32 * (2 * (1 << 11) - 1)
    m1, m2 = oracle.chacha_words(1, 1 << 18), oracle.chacha_words(2, 1 << 18)
    with Server(ctx, n_slots=4, mem_budget_bytes=int(need * 1.5)) as srv:
        a = srv.submit_commit(m1, p)
        srv.wait(a, COMMITTED, 60000)
        b = srv.submit_commit(m2, p)
        time.sleep(0.2)
        assert srv.state(b) == QUEUED          # not admitted: memory held by a
        srv.submit_open(a, [0, 5])
        srv.wait(a, OPENED, 60000)
        srv.wait(b, COMMITTED, 60000)          # admitted once a freed its HBM
        _, _, root = oracle.commit(m2, 2, 9, 1)
        assert srv.root(b) == root
        srv.submit_open(b, [1])
        srv.wait(b, OPENED, 60000)


@pytest.mark.parametrize("order", ["smallest", "fifo"])
def test_server_admission_order(oracle, ctx, order):
    """One slot: while a large commit runs, a large and then a small request
    queue up.  Smallest-first admits the small one first; arrival order (or
    an aging bound already passed) the large one.  Results are unchanged."""
    from bitz_gb300 import PcsParams
    from bitz_gb300.serve import ADMIT_FIFO, ADMIT_SMALLEST, OPENED, Server

    big, small = PcsParams(22 + 7, 2, 11, 1), PcsParams(12 + 7, 2, 6, 1)
    m_big = [oracle.chacha_words(40 + i, 1 << 22) for i in range(2)]
    m_small = oracle.chacha_words(42, 1 << 12)
    with Server(ctx, n_slots=1) as srv:
        srv.set_policy(ADMIT_SMALLEST if order == "smallest" else ADMIT_FIFO, 10000, 20)
        a = srv.submit_commit_open(m_big[0], big, [0, 3])
        b = srv.submit_commit_open(m_big[1], big, [1])
        c = srv.submit_commit_open(m_small, small, [2, 5])
        for rid in (a, b, c):
            srv.wait(rid, OPENED, 120000)
        tb, tc = srv.times(b)[1], srv.times(c)[1]
        assert (tc < tb) == (order == "smallest")
        for rid, m, p, q in ((b, m_big[1], big, [1]), (c, m_small, small, [2, 5])):
            cw, tree, root = oracle.commit(m, 2, p.log_batch_size, 1, n_threads=8)
            assert srv.root(rid) == root
            rows, proof = srv.open_result(rid, p.num_ntts())
            want = cw.reshape(-1, p.num_ntts(), 2)[q]
            assert (rows == want).all()
    with Server(ctx, n_slots=1) as srv:
        with pytest.raises(Exception):
            srv.set_policy(7, 10, 20)
        with pytest.raises(Exception):
            srv.set_policy(ADMIT_FIFO, 10, 63)


def test_server_bounded_wait_times_out(ctx):
    from bitz_gb300 import BzError, PcsParams
    from bitz_gb300.serve import OPENED, Server

    with Server(ctx, n_slots=1) as srv:
        m = np.zeros((1 << 12, 2), np.uint64)
        rid = srv.submit_commit(m, PcsParams(12 + 7, 2, 6, 1))
        with pytest.raises(BzError) as e:
            srv.wait(rid, OPENED, 200)         # never opened: the wait must end
        assert e.value.status == 6


def test_batch_plan_matches_single(oracle, ctx):
    from bitz_gb300 import BatchPlan, DeviceArray, PcsParams, commit

    rng = np.random.default_rng(8)
    shapes = _shapes(rng, 16, 12, 20)
    params = [PcsParams(k + 7, 2, a, 1) for (k, a) in shapes]
    msgs = [DeviceArray.chacha(70 + i, 1 << k, ctx) for i, (k, _) in enumerate(shapes)]
    single = []
    for m, p in zip(msgs, params):
        c, pd = commit(m, p, ctx)
        single.append((c.root, pd.codeword))
        pd.free()
    for graph in (True, False):
        for branches in (1, 4):
            plan = BatchPlan(msgs, params, use_graph=graph, n_branches=branches, ctx=ctx)
            for _ in range(2):
                plan.launch()
            roots = plan.roots()
            for i in range(len(msgs)):
                assert roots[i] == single[i][0]
                assert (plan.codeword(i) == single[i][1]).all()
            plan.close()


def test_server_reused_buffers_give_the_same_results(oracle, ctx):
    """Requests of one size run back to back reuse the finished ones' device
    buffers (codeword, tree, message); a budget that holds one large request
    makes the spares go back to the pool for other sizes.  Every root, row and
    multi-proof still equals the oracle's."""
    from bitz_gb300 import PcsParams
    from bitz_gb300.serve import OPENED, Server

    def need(k):
        return (16 << k) + (16 << (k + 2)) + 32 * (2 * (1 << (k - k // 2 + 2)) - 1)

    sizes = [14, 14, 14, 16, 14, 16, 12, 16, 14]
    with Server(ctx, n_slots=2, mem_budget_bytes=int(need(16) * 1.1)) as srv:
        for i, k in enumerate(sizes):
            m = oracle.chacha_words(700 + i, 1 << k)
            p = PcsParams(k + 7, 2, k // 2, 1)
            q = [0, 3, (1 << (k - k // 2 + 2)) - 1]
            rid = srv.submit_commit_open(m, p, q)
            srv.wait(rid, OPENED, 60000)
            cw, tree, root = oracle.commit(m, 2, k // 2, 1)
            assert srv.root(rid) == root
            rows, proof = srv.open_result(rid, p.num_ntts())
            lanes = 1 << (k // 2)
            exp_rows = cw.reshape(-1, lanes, 2)[q].reshape(len(q), -1)
            assert (rows.reshape(len(q), -1) == exp_rows).all()
            assert (proof == oracle.merkle_multi_proof(tree, 1 << (k - k // 2 + 2), q)).all()
            srv.release(rid)
        st = srv.stats()
        assert st["opened"] == len(sizes) and st["failed"] == 0 and st["in_use"] == 0
