"""GPU commit parity with the oracle: codeword, Merkle tree and root must be
bit-identical (flock-core/src/pcs/commit.rs semantics)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

# (log_msg_len, log_inv_rate, log_batch_size): small and ragged shapes,
# every leaf-size regime (16 B .. 16 KiB), rates 1/2 .. 1/8.
SHAPES = [
    (1, 1, 0), (1, 1, 1), (4, 1, 0), (6, 2, 1), (8, 1, 2), (9, 2, 5), (10, 1, 5), (10, 2, 3),
    (12, 2, 6), (12, 3, 4), (13, 2, 7), (14, 2, 7), (14, 1, 10), (15, 2, 8), (16, 2, 9),
    (16, 1, 12), (17, 2, 14), (18, 2, 9), (18, 3, 2), (20, 2, 10),
]


def _gpu_commit(msg, r, lb, kind, ctx, schedule=None):
    from bitz_gb300 import PcsParams, commit

    p = PcsParams(msg.shape[0].bit_length() - 1 + 7, r, lb, kind)
    if schedule is not None:
        ctx.set_schedule(p, schedule)
    c, pd = commit(msg, p, ctx)
    return c, pd


@pytest.mark.parametrize("lm,r,lb", SHAPES)
@pytest.mark.parametrize("kind", [0, 1])
def test_commit_matches_oracle(oracle, ctx, lm, r, lb, kind):
    msg = oracle.chacha_words(lm * 100 + r * 10 + lb, 1 << lm)
    cw, tree, root = oracle.commit(msg, r, lb, kind, n_threads=8)
    c, pd = _gpu_commit(msg, r, lb, kind, ctx)
    try:
        assert (pd.codeword == cw).all(), "codeword"
        assert (pd.merkle_tree == tree).all(), "tree"
        assert c.root == root
    finally:
        pd.free()


@pytest.mark.parametrize("lm,r,lb", [(1, 1, 0), (4, 1, 0), (6, 2, 1), (8, 1, 2), (7, 3, 4)])
def test_commit_codeword_equals_rs_definition(ctx, lm, r, lb):
    """The device codeword against the Lin-Chung-Han novel-basis evaluation
    computed from its definition (oracle/lch_definition.py), lane by lane."""
    from oracle import lch_definition as D

    rng = np.random.default_rng(0xDEF + lm)
    msg = rng.integers(0, 2**64, (1 << lm, 2), dtype=np.uint64)
    c, pd = _gpu_commit(msg, r, lb, 1, ctx)
    try:
        ints = [int(w[0]) | (int(w[1]) << 64) for w in msg]
        got = [int(w[0]) | (int(w[1]) << 64) for w in pd.codeword.reshape(-1, 2)]
        assert got == D.interleaved_codeword(ints, lb, r)
    finally:
        pd.free()


SCHEDULES = [0, 1, 2, 3, 4, 0x10, 0x13, 0x20,
             2 | (1 << 7), 3 | (2 << 7), 0x42, 0x41, 0x43, 0x42 | (1 << 7), 0x42 | (2 << 7),
             0x52, 0x43 | (1 << 7), 0x44,
             0x200 | 2, (1 << 10) | 2, (2 << 10) | 0x200 | 2, (3 << 10) | 0x200 | 2,
             (2 << 10) | 0x200 | 3 | (1 << 7), (1 << 10) | 0x10 | 2, (3 << 10) | 0x200 | 0x11,
             0x1000 | 2, 0x1200 | 2, 0x1000 | (1 << 10) | 2, 0x1000 | 0, 0x3602, 0x3a03,
             (1 << 10), (2 << 10) | 0x200, (3 << 10) | 0x3200, 0x1200 | (1 << 10), 0x3200,
             0x4000, 0x5000, 0x5400, 0x5C00, 0x5001, 0x5002, 0x4010,
             0x8000, 0x18000, 0x208000, 0x205000]


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("lm,r,lb", [(14, 2, 7), (12, 1, 4), (18, 2, 9), (20, 2, 10),
                                     (16, 1, 9), (19, 3, 9)])
def test_every_schedule_gives_the_same_codeword(oracle, ctx, schedule, lm, r, lb):
    from bitz_gb300 import PcsParams

    msg = oracle.chacha_words(99, 1 << lm)
    cw, _, root = oracle.commit(msg, r, lb, 1, n_threads=8)
    c, pd = _gpu_commit(msg, r, lb, 1, ctx, schedule)
    try:
        assert (pd.codeword == cw).all()
        assert c.root == root
    finally:
        pd.free()
        ctx.set_schedule(PcsParams(lm + 7, r, lb, 1), 3)


def test_roots_fixture(ctx):
    """Committed oracle roots, including the 2^20 and 2^24 benchmark shapes."""
    from bitz_gb300 import DeviceArray, PcsParams, commit

    with open(os.path.join(GOLDEN, "roots.json")) as fh:
        roots = json.load(fh)["roots"]
    for e in roots:
        kind = 1 if e["hash"] == "blake3" else 0
        p = PcsParams(e["log_msg_len"] + 7, e["log_inv_rate"], e["log_batch_size"], kind)
        msg = DeviceArray.chacha(e["seed"], 1 << e["log_msg_len"], ctx)
        c, pd = commit(msg, p, ctx)
        pd.free()
        msg.free()
        assert c.root.hex() == e["root"], e


@pytest.mark.parametrize("schedule", [0x5000, 0x5400, 0x5001, 0x8000, 0x18000, 0x208000])
def test_compact_twiddle_tables_at_benchmark_shapes(ctx, schedule):
    """Compact tables for the narrow twiddles of the deepest radix-4 pass
    (all three twiddles at 2^20 and 2^24, the second layer's only at 2^28
    shapes), against the committed oracle roots of the benchmark shapes."""
    from bitz_gb300 import DeviceArray, PcsParams, commit

    with open(os.path.join(GOLDEN, "roots.json")) as fh:
        roots = json.load(fh)["roots"]
    for e in roots:
        if e["log_msg_len"] not in (20, 24, 28) or e["hash"] != "blake3":
            continue
        p = PcsParams(e["log_msg_len"] + 7, e["log_inv_rate"], e["log_batch_size"], 1)
        ctx.set_schedule(p, schedule)
        msg = DeviceArray.chacha(e["seed"], 1 << e["log_msg_len"], ctx)
        try:
            c, pd = commit(msg, p, ctx)
            pd.free()
            assert c.root.hex() == e["root"], (hex(schedule), e)
        finally:
            msg.free()
            ctx.set_schedule(p, 3)


@pytest.mark.parametrize("schedule", [0x5000, 0x5400])
def test_compact_twiddle_tables_two_word(oracle, ctx, schedule):
    """2^22 words at rate 1/8 (ell = 16, passes from layer 3): the pass at
    layer 13 has t_o of 53 bits and t_a, t_b of 29 bits, both in two-word
    compact tables; the codeword root must equal the oracle's."""
    from bitz_gb300 import PcsParams

    msg = oracle.chacha_words(5, 1 << 22)
    _, _, root = oracle.commit(msg, 3, 9, 1, n_threads=16)
    try:
        c, pd = _gpu_commit(msg, 3, 9, 1, ctx, schedule)
        pd.free()
        assert c.root == root
    finally:
        ctx.set_schedule(PcsParams(22 + 7, 3, 9, 1), 3)


def test_cmt1_fixture(ctx):
    import struct

    from bitz_gb300 import PcsParams, commit

    with open(os.path.join(GOLDEN, "commit_cmt1_m16_r1_b5_sha256.bin"), "rb") as fh:
        buf = fh.read()
    _, m, r, lb, _, _, _, _, _, msg_len = struct.unpack_from("<10I", buf, 0)
    msg = np.frombuffer(buf, "<u8", msg_len * 2, 40).reshape(-1, 2).copy()
    off = 40 + msg_len * 16
    (cw_len,) = struct.unpack_from("<I", buf, off)
    cw = np.frombuffer(buf, "<u8", cw_len * 2, off + 4).reshape(-1, 2)
    root = buf[off + 4 + cw_len * 16: off + 4 + cw_len * 16 + 32]
    c, pd = commit(msg, PcsParams(m, r, lb, 0), ctx)
    try:
        assert (pd.codeword == cw).all()
        assert c.root == root
    finally:
        pd.free()


def test_device_input_equals_host_input(oracle, ctx):
    from bitz_gb300 import DeviceArray, PcsParams, commit

    p = PcsParams(20 + 7, 2, 10, 1)
    d = DeviceArray.chacha(5, 1 << 20, ctx)
    h = oracle.chacha_words(5, 1 << 20)
    assert (d.to_host() == h).all()
    c1, pd1 = commit(d, p, ctx)
    c2, pd2 = commit(h, p, ctx)
    assert c1.root == c2.root
    pd1.free(); pd2.free(); d.free()


def test_linearity_at_full_size(ctx):
    """RS encoding is linear: cw(a) ^ cw(b) == cw(a ^ b) at the 2^24-word,
    2^12 x 2^12 shape (checked on the device-copied codewords)."""
    from bitz_gb300 import DeviceArray, PcsParams, commit

    p = PcsParams(24 + 7, 2, 12, 1)
    a = DeviceArray.chacha(11, 1 << 24, ctx)
    b = DeviceArray.chacha(12, 1 << 24, ctx)
    ah, bh = a.to_host(), b.to_host()
    x = DeviceArray.from_host(ah ^ bh, ctx)
    _, pa = commit(a, p, ctx)
    _, pb = commit(b, p, ctx)
    _, px = commit(x, p, ctx)
    try:
        ca, cb, cx = pa.codeword, pb.codeword, px.codeword
        assert ((ca ^ cb) == cx).all()
        # replicate structure: the codeword of a constant message is constant per lane
    finally:
        for q in (pa, pb, px):
            q.free()
        for d in (a, b, x):
            d.free()


def test_determinism_and_sensitivity(oracle, ctx):
    from bitz_gb300 import PcsParams, commit

    p = PcsParams(14 + 7, 2, 7, 1)
    msg = oracle.chacha_words(3, 1 << 14)
    c1, d1 = commit(msg, p, ctx)
    c2, d2 = commit(msg, p, ctx)
    msg2 = msg.copy()
    msg2[7, 0] ^= 1
    c3, d3 = commit(msg2, p, ctx)
    assert c1.root == c2.root and c1.root != c3.root
    for d in (d1, d2, d3):
        d.free()


def test_async_host_commits_overlap_and_match(oracle, ctx):
    """bz_commit_async: several commits in flight; each root equals the
    synchronous commit's."""
    import ctypes

    from bitz_gb300 import PcsParams, commit
    from bitz_gb300 import _lib

    L = _lib.lib()
    p = PcsParams(18 + 7, 2, 9, 1)
    msgs = [oracle.chacha_words(40 + i, 1 << 18) for i in range(5)]
    pc = p.to_c()
    handles = []
    for m in msgs:
        h = ctypes.c_void_p()
        assert L.bz_commit_async(ctx.handle, _lib.ptr(m), m.shape[0], ctypes.byref(pc),
                                 ctypes.byref(h)) == 0
        handles.append(h)
    for m, h in zip(msgs, handles):
        root = (ctypes.c_uint8 * 32)()
        assert L.bz_commitment_root(h, root) == 0
        c, pd = commit(m, p, ctx)
        assert bytes(root) == c.root
        pd.free()
        L.bz_commitment_free(h)
