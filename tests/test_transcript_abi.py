"""The library's host-side transcript against the oracle's (no GPU needed).

bz_transcript_* and bz_blake3_xof run on the host inside libbitzgpu.so (the
transcript absorbs a few bytes per protocol message); these tests load the
library and compare every operation byte for byte with oracle/transcript.py.
"""
import random

import numpy as np
import pytest


@pytest.fixture(scope="module")
def B():
    import bitz_gb300

    bitz_gb300.lib()
    return bitz_gb300


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 1023, 1024, 1025, 2047, 2048, 2049, 3072,
                               4097, 70000, 300000])
def test_xof_matches_oracle(oracle, B, n):
    d = np.random.default_rng(n).integers(0, 256, n, dtype=np.uint8).tobytes()
    for L in (1, 32, 64, 65, 200):
        assert B.blake3_xof(d, L) == oracle.blake3_xof(d, L)


def test_xof_empty_kat(B):
    from test_oracle_transcript import EMPTY_XOF_131

    assert B.blake3_xof(b"", 131).hex() == EMPTY_XOF_131


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_transcript_random_ops(oracle, B, seed):
    from oracle.transcript import Blake3Transcript as OT

    rng = random.Random(seed)
    a, b = B.Blake3Transcript(), OT()
    for i in range(250):
        op = rng.randrange(6)
        if op == 0:
            d = rng.randbytes(rng.choice([0, 1, 16, 100, 1500, 3000]))
            a.absorb(d)
            b.absorb(d)
        elif op == 1:
            d = rng.randbytes(rng.choice([0, 8, 16, 32, 2000]))
            a.absorb_slice(d)
            b.absorb_slice(d)
        elif op == 2:
            n = rng.choice([1, 16, 32, 100])
            assert a.challenge_bytes(n) == b.challenge_bytes(n)
        elif op == 3:
            n = rng.choice([0, 16, 64, 130])
            assert a.fill_sampling_bytes(n) == b.fill_sampling_bytes(n)
        elif op == 4:
            assert a.get_field_challenge().tolist() == list(
                np.frombuffer(b.challenge_bytes(16), "<u8"))
        else:
            assert a.state_digest() == b.state_digest()
        if i == 120:
            c = a.clone()
            assert c.state_digest() == a.state_digest()
            c.absorb(b"x")
            assert c.state_digest() != a.state_digest()


def test_challenger_observations(oracle, B):
    from oracle.transcript import Blake3Transcript as OT, ZincChallenger as OZ

    p = B.ZincChallenger(B.Blake3Transcript())
    o = OZ(OT())
    for ch in (p, o):
        ch.observe_label(b"flock-ligerito-basis-v0")
        ch.observe_f128([2**64 - 1, 12345])
        ch.observe_bytes(bytes(range(32)))
        ch.observe_f128_slice(np.arange(10, dtype=np.uint64).reshape(5, 2))
    assert p.t.state_digest() == o.t.state_digest()
    assert p.sample_f128().tolist() == o.sample_f128().tolist()
    assert p.sample_f128_vec(3).tolist() == o.sample_f128_vec(3).tolist()


@pytest.mark.parametrize("bits", [0, 1, 6, 10])
def test_verify_pow_matches_oracle(oracle, B, bits):
    from oracle.transcript import Blake3Transcript as OT, ZincChallenger as OZ

    prover = OZ(OT())
    prover.observe_label(b"pow")
    nonce = prover.grind_pow(bits)
    for cand, expect in ((nonce, True), (nonce + 1, None)):
        v_prod = B.ZincChallenger(B.Blake3Transcript())
        v_orc = OZ(OT())
        for v in (v_prod, v_orc):
            v.observe_label(b"pow")
        got = v_prod.verify_pow(cand, bits)
        assert got == v_orc.verify_pow(cand, bits)
        if expect is not None:
            assert got is expect
        assert v_prod.t.state_digest() == v_orc.t.state_digest()
