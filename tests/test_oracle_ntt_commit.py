"""Oracle NTT and commit, restating the reference's own self-consistency tests
(flock-core/src/ntt/additive_ntt_f128.rs:1055-1301, pcs/commit.rs:439-551) and
checking the committed fixtures."""
import json
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN


def _rand(rng, n):
    return rng.integers(0, 2**64, (n, 2), dtype=np.uint64)


def test_zero_dimensional_transform_is_identity(oracle):
    v = np.array([[2**64 - 1, 0x123456789ABCDEF0]], np.uint64)
    assert (oracle.ntt_forward(v) == v).all()


def test_twiddle_block_zero_is_zero(oracle):
    for ell in (3, 8, 14):
        for layer in range(ell):
            assert (oracle.ntt_twiddle(ell, layer, 0) == 0).all()


def test_deepest_layer_twiddles_are_shifted_block_index(oracle):
    # evals[0] is the basis {x^k}, so twiddle(ell-1, b) = b * x
    for ell in (4, 10, 16):
        for b in (1, 2, 3, 5, 77 % (1 << (ell - 1)), (1 << (ell - 1)) - 1):
            t = oracle.ntt_twiddle(ell, ell - 1, b)
            assert oracle.gf_int(t) == b << 1


@pytest.mark.parametrize("log_d", [3, 4, 8])
@pytest.mark.parametrize("num_ntts", [1, 2, 4, 8])
def test_interleaved_matches_per_lane(oracle, log_d, num_ntts):
    rng = np.random.default_rng(0xCC1 + log_d * 16 + num_ntts)
    x = _rand(rng, (1 << log_d) * num_ntts)
    inter = oracle.ntt_forward_interleaved(x, num_ntts)
    for lane in range(num_ntts):
        sub = oracle.ntt_forward(np.ascontiguousarray(x[lane::num_ntts]))
        assert (inter[lane::num_ntts] == sub).all()


@pytest.mark.parametrize("log_d,num_ntts", [(4, 2), (10, 8), (12, 32)])
def test_interleaved_parallel_matches_scalar(oracle, log_d, num_ntts):
    rng = np.random.default_rng(0xCC2)
    x = _rand(rng, (1 << log_d) * num_ntts)
    a = oracle.ntt_forward_interleaved(x, num_ntts, 0, 1)
    b = oracle.ntt_forward_interleaved(x, num_ntts, 0, 8)
    assert (a == b).all()


@pytest.mark.parametrize("m,r,lb", [(10, 1, 1), (12, 1, 2), (12, 2, 1), (14, 2, 3), (15, 3, 4)])
@pytest.mark.parametrize("kind", [0, 1])
def test_commit_matches_full_ntt(oracle, m, r, lb, kind):
    rng = np.random.default_rng(0xFEED + m)
    lm = m - 7
    z = _rand(rng, 1 << lm)
    cw, tree, root = oracle.commit(z, r, lb, kind)
    full = np.zeros(((1 << lm) << r, 2), np.uint64)
    full[: 1 << lm] = z
    full = oracle.ntt_forward_interleaved(full, 1 << lb, 0)
    assert (cw == full).all()
    k_code = lm - lb + r
    t2 = oracle.merkle_tree(full.tobytes(), 1 << k_code, kind)
    assert t2[-1].tobytes() == root
    assert (t2 == tree).all()


def test_rs_encoding_is_linear(oracle):
    rng = np.random.default_rng(123)
    z1, z2 = _rand(rng, 1 << 9), _rand(rng, 1 << 9)
    c1, _, _ = oracle.commit(z1, 1, 1, 0)
    c2, _, _ = oracle.commit(z2, 1, 1, 0)
    cx, _, _ = oracle.commit(z1 ^ z2, 1, 1, 0)
    assert ((c1 ^ c2) == cx).all()


def test_commit_rejects_bad_shapes(oracle):
    z = np.zeros((16, 2), np.uint64)
    with pytest.raises(ValueError):
        oracle.commit(z, 0, 1, 0)        # log_inv_rate < 1
    with pytest.raises(ValueError):
        oracle.commit(z, 1, 5, 0)        # log_batch_size > log_msg_len


def _splitmix(seed, n):
    s, out, M = seed, [], 2**64 - 1
    for _ in range(n):
        s = (s + 0x9E3779B97F4A7C15) & M
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        out.append(z ^ (z >> 31))
    return out


def test_cmt1_fixture(oracle):
    """The CMT1 file (dump_commit_vectors.rs layout) round-trips through the
    oracle; its witness is the dumper's SplitMix64(0xC0FFEE) stream."""
    with open(os.path.join(GOLDEN, "commit_cmt1_m16_r1_b5_sha256.bin"), "rb") as fh:
        buf = fh.read()
    hdr = struct.unpack_from("<10I", buf, 0)
    magic, m, r, lb, k_code, num_ntts, n_pos, n_leaves, leaf_sz, msg_len = hdr
    assert magic == 0x434D5431 and (m, r, lb) == (16, 1, 5)
    assert k_code == m - 7 - lb + r and num_ntts == 32 and n_leaves == n_pos == 1 << k_code
    off = 40
    msg = np.frombuffer(buf, "<u8", msg_len * 2, off).reshape(-1, 2)
    off += msg_len * 16
    (cw_len,) = struct.unpack_from("<I", buf, off)
    off += 4
    cw = np.frombuffer(buf, "<u8", cw_len * 2, off).reshape(-1, 2)
    off += cw_len * 16
    root = buf[off:off + 32]
    assert list(msg.reshape(-1)) == _splitmix(0xC0FFEE, msg_len * 2)
    cw2, _, root2 = oracle.commit(np.ascontiguousarray(msg), r, lb, 0)
    assert (cw2 == cw).all() and root2 == root


def test_roots_fixture_small(oracle):
    with open(os.path.join(GOLDEN, "roots.json")) as fh:
        roots = json.load(fh)["roots"]
    for e in roots:
        if e["log_msg_len"] > 16:
            continue
        z = oracle.chacha_words(e["seed"], 1 << e["log_msg_len"])
        kind = 1 if e["hash"] == "blake3" else 0
        _, _, root = oracle.commit(z, e["log_inv_rate"], e["log_batch_size"], kind, 4)
        assert root.hex() == e["root"], e


@pytest.mark.parametrize("ld,lanes,start,threads", [(6, 1, 0, 1), (8, 4, 2, 4), (12, 64, 2, 8),
                                                    (10, 512, 1, 3), (14, 128, 2, 16),
                                                    (16, 32, 3, 8), (9, 4096, 2, 8)])
def test_blocked_parallel_ntt_equals_per_layer(ld, lanes, start, threads):
    """The oracle's parallel form (top layers fused in pairs, deep layers per
    cache-resident sub-group, persistent thread pool: the structure of the
    reference's parallel path) equals the per-layer scalar form."""
    from oracle import oracle as O

    d = O.chacha_words(ld * 7 + lanes, lanes << ld)
    a = O.ntt_forward_interleaved(d, lanes, start, 1)
    b = O.ntt_forward_interleaved_blocked(d, lanes, start, threads)
    assert (a == b).all()
