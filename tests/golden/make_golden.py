"""Regenerates the committed golden fixtures in tests/golden/.

Run where the BitZ-PoC reference checkout and the ``cryptography`` package
are available, giving the checkout's root:

    python tests/golden/make_golden.py --reference <path to BitZ-PoC>

(the reference is read only for ``ghash``; the other fixtures need neither
it nor the flag).

Outputs (all small):

* ``ghash_kat.json`` -- NIST CAVP GCM (AES-128, 96-bit IV) cases from the
  reference's ``vendor/field/tests/vectors/gcm_encrypt_128.rsp``, reduced to
  GHASH known answers: the hash subkey H = AES_K(0) and the GHASH digest
  (tag XOR AES_K(IV || 0^31 || 1)), as the reference's
  ``vendor/field/tests/ghash_vectors.rs:128-163`` does.  AES is computed here
  with the ``cryptography`` package so the GPU machine needs neither AES nor the
  reference.
* ``chacha_kat.json`` -- RFC 8439 ChaCha20 keystream words for the synthetic
  input generator (key = seed as LE u64 zero-padded, nonce 0), from
  ``cryptography``.
* ``commit_cmt1_m16_r1_b5_sha256.bin`` -- a commit fixture in the reference's
  CMT1 layout (flock-prover/src/bin/dump_commit_vectors.rs:13-31) with the same
  SplitMix64(0xC0FFEE) witness; produced by the oracle.  A maintainer with a
  Rust toolchain can regenerate the reference's own file with
  ``cargo run --release --bin dump_commit_vectors -- out.bin 16 1 5`` and
  compare byte for byte.
* ``roots.json`` -- oracle commit roots for seeded ChaCha inputs at the test
  shapes and at the 2^20- and 2^24-word benchmark shapes (regression pins for
  full-size GPU runs).
"""
from __future__ import annotations

import json
import os
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

RSP_IN_REFERENCE = os.path.join("vendor", "field", "tests", "vectors", "gcm_encrypt_128.rsp")


def parse_rsp(text):
    cases, cur, tag_bytes, in_rec = [], None, 0, False
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            if in_rec:
                cases.append(cur)
                in_rec = False
            continue
        if line.startswith("[") and line.endswith("]"):
            p = line[1:-1]
            if p.startswith("Taglen = "):
                tag_bytes = int(p.split("=")[1]) // 8
            continue
        name, _, value = line.partition(" = ")
        if name == "Count":
            cur = {"tag_bytes": tag_bytes}
            in_rec = True
        elif name in ("Key", "IV", "AAD", "CT", "Tag"):
            cur[name.lower()] = value.strip()
    if in_rec:
        cases.append(cur)
    return cases


def make_ghash(reference_root):
    from cryptography.hazmat.primitives.ciphers import Cipher, algorithms, modes

    if not reference_root:
        raise SystemExit("ghash needs --reference <path to the BitZ-PoC checkout>")
    with open(os.path.join(reference_root, RSP_IN_REFERENCE)) as fh:
        cases = parse_rsp(fh.read())
    assert len(cases) == 525, len(cases)
    out = []
    for i, c in enumerate(cases):
        key = bytes.fromhex(c["key"])
        enc = Cipher(algorithms.AES(key), modes.ECB()).encryptor()
        h = enc.update(bytes(16))
        iv = bytes.fromhex(c["iv"])
        assert len(iv) == 12
        mask = enc.update(iv + b"\x00\x00\x00\x01")
        tag = bytes.fromhex(c["tag"])
        ghash = bytes(t ^ m for t, m in zip(tag, mask))
        out.append({"h": h.hex(), "aad": c.get("aad", ""), "ct": c.get("ct", ""),
                    "ghash_prefix": ghash.hex()})
    with open(os.path.join(HERE, "ghash_kat.json"), "w") as fh:
        json.dump({"source": "NIST CAVP gcmEncryptExtIV128.rsp subset shipped by the reference "
                             "(vendor/field/tests/vectors/gcm_encrypt_128.rsp)",
                   "bit_order": "NIST: most significant bit of byte 0 is X^0",
                   "cases": out}, fh, indent=0)


def make_chacha():
    from cryptography.hazmat.primitives.ciphers import Cipher, algorithms

    res = {}
    for seed in (0, 1, 2, 3, 0xC0FFEE):
        key = struct.pack("<Q", seed) + bytes(24)
        enc = Cipher(algorithms.ChaCha20(key, bytes(16)), mode=None).encryptor()
        ks = enc.update(bytes(16 * 40))
        words = [[struct.unpack("<Q", ks[16 * i:16 * i + 8])[0],
                  struct.unpack("<Q", ks[16 * i + 8:16 * i + 16])[0]] for i in range(40)]
        res[str(seed)] = words
    with open(os.path.join(HERE, "chacha_kat.json"), "w") as fh:
        json.dump({"generator": "RFC 8439 ChaCha20, key = seed LE u64 zero padded, nonce 0, "
                                "counter from 0; word i = keystream bytes [16i, 16i+16) as (lo, hi)",
                   "words": res}, fh)


def splitmix_words(seed, n):
    s = seed
    out = []
    M = 2**64 - 1
    for _ in range(n):
        s = (s + 0x9E3779B97F4A7C15) & M
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        out.append(z ^ (z >> 31))
    return out


def make_cmt1():
    import numpy as np
    from oracle import oracle as O

    m, r, lb = 16, 1, 5
    log_msg = m - 7
    words = splitmix_words(0xC0FFEE, 2 << log_msg)
    msg = np.array(words, dtype=np.uint64).reshape(-1, 2)
    cw, tree, root = O.commit(msg, r, lb, O.SHA256)
    k_code = log_msg - lb + r
    hdr = struct.pack("<10I", 0x434D5431, m, r, lb, k_code, 1 << lb, 1 << k_code, 1 << k_code,
                      16 << lb, msg.shape[0])
    with open(os.path.join(HERE, "commit_cmt1_m16_r1_b5_sha256.bin"), "wb") as fh:
        fh.write(hdr)
        fh.write(msg.astype("<u8").tobytes())
        fh.write(struct.pack("<I", cw.shape[0]))
        fh.write(cw.astype("<u8").tobytes())
        fh.write(root)


# (log_msg_len, log_inv_rate, log_batch_size, hash_kind, seed)
ROOT_SHAPES = [
    (10, 1, 5, 0, 7), (10, 1, 5, 1, 7), (12, 2, 6, 1, 5), (12, 2, 6, 0, 5),
    (14, 2, 7, 1, 9), (13, 1, 4, 1, 11), (16, 2, 8, 1, 3), (15, 3, 6, 1, 4),
    (20, 2, 10, 1, 0), (20, 2, 10, 0, 0), (24, 2, 12, 1, 1),
]


def make_roots():
    from oracle import oracle as O

    res = []
    for (lm, r, lb, kind, seed) in ROOT_SHAPES:
        msg = O.chacha_words(seed, 1 << lm)
        _, _, root = O.commit(msg, r, lb, kind, n_threads=os.cpu_count() or 1)
        res.append({"log_msg_len": lm, "log_inv_rate": r, "log_batch_size": lb,
                    "hash": "blake3" if kind else "sha256", "seed": seed, "root": root.hex()})
        print(res[-1], flush=True)
    with open(os.path.join(HERE, "roots.json"), "w") as fh:
        json.dump({"inputs": "ChaCha20 words of the given seed", "roots": res}, fh, indent=1)


def add_root(lm, r, lb, kind, seed):
    """Compute one more oracle root and merge it into roots.json."""
    from oracle import oracle as O

    path = os.path.join(HERE, "roots.json")
    with open(path) as fh:
        data = json.load(fh)
    msg = O.chacha_words(seed, 1 << lm)
    _, _, root = O.commit(msg, r, lb, kind, n_threads=os.cpu_count() or 1)
    entry = {"log_msg_len": lm, "log_inv_rate": r, "log_batch_size": lb,
             "hash": "blake3" if kind else "sha256", "seed": seed, "root": root.hex()}
    data["roots"] = [e for e in data["roots"] if (e["log_msg_len"], e["seed"], e["hash"]) !=
                     (lm, seed, entry["hash"])] + [entry]
    with open(path, "w") as fh:
        json.dump(data, fh, indent=1)
    print(entry)


if __name__ == "__main__":
    args = sys.argv[1:]
    reference = None
    if "--reference" in args:
        i = args.index("--reference")
        reference = args[i + 1]
        del args[i:i + 2]
    if args[:1] == ["root"]:
        add_root(*[int(x) for x in args[1:6]])
        sys.exit(0)
    which = args or ["ghash", "chacha", "cmt1", "roots"]
    if "ghash" in which:
        make_ghash(reference)
    if "chacha" in which:
        make_chacha()
    if "cmt1" in which:
        make_cmt1()
    if "roots" in which:
        make_roots()
