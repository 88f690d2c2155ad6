"""The C-ABI library builds, loads without a GPU and exports every symbol the
public header declares; host-only entry points behave as documented."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_library_exports_every_declared_symbol():
    from bitz_gb300 import _lib

    L = _lib.lib()
    names = _lib.declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if getattr(L, n, None) is None]
    assert not missing, missing


def test_abi_version_and_status_strings():
    from bitz_gb300 import _lib

    L = _lib.lib()
    assert L.bz_abi_version() == 1
    for s in range(9):
        assert L.bz_status_string(s)
    assert L.bz_status_string(0) == b"ok"


def test_null_arguments_are_rejected_without_a_device():
    from bitz_gb300 import _lib

    L = _lib.lib()
    assert L.bz_ctx_create(0, 0, None) == 1            # BZ_ERR_ARG
    assert L.bz_ctx_destroy(None) == 1
    assert L.bz_commitment_free(None) == 1
    assert L.bz_commit(None, None, 0, None, None, None) == 1
    assert L.bz_last_error(None) == b"no context"


def test_host_chacha_matches_rfc8439_fixture():
    from bitz_gb300 import pcs

    with open(os.path.join(GOLDEN, "chacha_kat.json")) as fh:
        words = json.load(fh)["words"]
    for seed, w in words.items():
        exp = np.array(w, dtype=np.uint64)
        got = pcs.chacha_words(int(seed), len(w), n_threads=1)
        assert (got == exp).all(), seed
        # offsets and multithreaded fills agree
        got2 = pcs.chacha_words(int(seed), len(w) - 3, first_word=3, n_threads=1)
        assert (got2 == exp[3:]).all()


def test_host_chacha_threads_agree():
    from bitz_gb300 import pcs

    a = pcs.chacha_words(7, 1 << 17, n_threads=1)
    b = pcs.chacha_words(7, 1 << 17, n_threads=8)
    assert (a == b).all()


def test_oracle_chacha_matches_fixture(oracle):
    with open(os.path.join(GOLDEN, "chacha_kat.json")) as fh:
        words = json.load(fh)["words"]
    for seed, w in words.items():
        assert (oracle.chacha_words(int(seed), len(w)) == np.array(w, dtype=np.uint64)).all()


def test_pcs_params_geometry():
    from bitz_gb300 import PcsParams, HashKind

    # benchmark shapes: 2^a x 2^b, rate 1/4 -> m = a + b + 7
    for a, b in [(10, 10), (12, 12), (14, 14)]:
        p = PcsParams(a + b + 7, 2, a, HashKind.BLAKE3)
        assert p.k_code() == b + 2
        assert p.n_leaves() == 1 << (b + 2)
        assert p.leaf_size_bytes() == 16 << a
        assert p.codeword_len_f128() == 1 << (a + b + 2)
    with pytest.raises(ValueError):
        PcsParams(10, 1, 5).validate()
    with pytest.raises(ValueError):
        PcsParams(20, 0, 5).validate()
