/*
 * CPU oracle for the BitZ / flock Ligerito commitment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (Rust crate flock-core vendored in BitZ-PoC, plus the GF(2^128)
 * field crate).  It is linked only by the test-suite, by the package smoke
 * check and by the CPU-baseline leg of bench.py, always as the checker or as
 * the timed CPU baseline -- never by the GPU library.
 *
 * Parity status: the field is pinned to NIST GCM/GHASH known answers, SHA-256
 * to Python's hashlib, ChaCha20 to the `cryptography` package, BLAKE3 to the
 * BLAKE3 specification's published digests (single- and multi-chunk inputs);
 * the NTT and the commit codeword to the Reed-Solomon encoding in the
 * Lin-Chung-Han novel basis evaluated from its definition (a second,
 * independent derivation in lch_definition.py).  The Merkle / fold code
 * follows the reference source (file:line cited beside each function) but
 * has no reference-produced golden file to compare with (the reference is
 * Rust and no Rust toolchain exists on either machine): for those functions
 * parity is "unpinned" beyond the reference's own self-consistency
 * identities, which the tests restate.
 *
 * Element layout everywhere: a GF(2^128) element is two little-endian uint64
 * words {lo, hi}; arrays of n elements are uint64_t[2n].
 */
#ifndef BITZ_ORACLE_H
#define BITZ_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- GF(2^128), X^128 = X^7 + X^2 + X + 1 ---- */
const char *orc_clmul_kind(void); /* "pmull" on aarch64+crypto, else "portable" */
void orc_gf_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]);
void orc_gf_mul_bitwise(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]);
void orc_gf_inv(const uint64_t a[2], uint64_t out[2]);
void orc_gf_mul_many(const uint64_t *a, const uint64_t *b, uint64_t *out, size_t n);
/* GHASH chain over 16-byte polynomial-bit-order blocks: x = (x + blk) * h */
void orc_ghash_chain(const uint64_t h[2], const uint64_t *blocks, size_t n, uint64_t out[2]);

/* ---- additive NTT (LCH novel basis, standard subspace {1,x,..}) ---- */
/* twiddle(layer, block) of AdditiveNttF128::standard(log_domain) */
void orc_ntt_twiddle(int log_domain, int layer, uint64_t block, uint64_t out[2]);
/* all normalized subspace-poly rows: out[i][k] at out + 2*(i*log_domain + k) */
void orc_ntt_evals(int log_domain, uint64_t *out);
/* interleaved forward transform from start_layer, in place, n_threads >= 1 */
void orc_ntt_forward_interleaved(uint64_t *data, size_t num_ntts, int log_d,
                                 int start_layer, int n_threads);
/* single-lane forward transform (log_d layers) */
/* the same transform, top layers fused in pairs, deep layers per cache-resident
 * sub-group, on a persistent thread pool (the reference's parallel path) */
void orc_ntt_forward_interleaved_blocked(uint64_t *data, size_t num_ntts, int log_d,
                                         int start_layer, int n_threads);
void orc_ntt_forward(uint64_t *data, int log_d);

/* ---- hashes ---- */
void orc_sha256(const uint8_t *data, size_t len, uint8_t out[32]);
/* BLAKE3 unkeyed hash (root), 32-byte output */
void orc_blake3_hash(const uint8_t *data, size_t len, uint8_t out[32]);
/* Hasher::new().update(data).finalize_non_root() */
void orc_blake3_leaf_cv(const uint8_t *data, size_t len, uint8_t out[32]);
/* Non-root CV of whole chunks starting at chunk `first_chunk` of a larger
 * input (len a power-of-two number of 1 KiB chunks) */
void orc_blake3_subtree_cv(const uint8_t *data, size_t len, uint64_t first_chunk,
                           uint8_t out[32]);
void orc_blake3_rows_subtree_cvs(const uint8_t *rows, size_t n_rows, size_t row_len,
                                 uint64_t first_chunk, uint8_t *out);
/* merge_subtrees_non_root(l, r, Mode::Hash) */
void orc_blake3_parent_cv(const uint8_t l[32], const uint8_t r[32], uint8_t out[32]);

/* BLAKE3 extended output (finalize_xof) of the whole input */
void orc_blake3_xof(const uint8_t *data, size_t len, uint8_t *out, size_t out_len);
/* proof of work: blake3(prefix || nonce_le) has >= bits leading zero bits */
int orc_pow_ok(const uint8_t *prefix, size_t plen, uint64_t nonce, unsigned bits);
uint64_t orc_pow_first_nonce(const uint8_t *prefix, size_t plen, uint64_t start, uint64_t end,
                             unsigned bits);

/* hash_kind: 0 = SHA-256, 1 = BLAKE3 */
void orc_hash_leaf(const uint8_t *data, size_t len, int kind, uint8_t out[32]);
void orc_hash_pair(const uint8_t l[32], const uint8_t r[32], int kind, uint8_t out[32]);

/* ---- Merkle (flat layout: leaves, then each level up, root last) ---- */
void orc_merkle_tree(const uint8_t *data, size_t data_len, size_t num_leaves, int kind,
                     uint8_t *tree /* (2*num_leaves-1)*32 */, int n_threads);
/* returns number of hashes written to out (caller sizes out for q*depth) */
/* parent levels above the leaves already in tree[0 .. num_leaves) */
void orc_merkle_tree_from_leaves(uint8_t *tree, size_t num_leaves, int kind);
size_t orc_merkle_multi_proof(const uint8_t *tree, size_t num_leaves,
                              const uint64_t *positions, size_t q, uint8_t *out);
int orc_verify_merkle_multi_proof(const uint8_t root[32], size_t num_leaves,
                                  const uint64_t *sorted_positions, const uint8_t *leaf_hashes,
                                  size_t q, const uint8_t *proof, size_t n_proof, int kind);

/* ---- commit ---- */
/* msg: 2^(log_msg_len) elements, codeword: 2^(log_msg_len+log_inv_rate) elements,
   tree: (2*n_leaves-1)*32 bytes, root: 32 bytes.  Returns 0 or -1 on bad shape. */
int orc_commit(const uint64_t *msg, int log_msg_len, int log_inv_rate, int log_batch_size,
               int hash_kind, uint64_t *codeword, uint8_t *tree, uint8_t root[32],
               int n_threads);

/* ---- sumcheck folds (LSB variable) ---- */
void orc_partial_eval_lsb(const uint64_t *evals, size_t n, const uint64_t *rs, size_t k,
                          uint64_t *out /* n >> k */);
void orc_round_msg_lsb(const uint64_t *f, const uint64_t *b, size_t n, uint64_t u0[2],
                       uint64_t u2[2]);
void orc_fold_and_msg_lsb(const uint64_t *f, const uint64_t *b, size_t n, const uint64_t r[2],
                          uint64_t *nf, uint64_t *nb, uint64_t u0[2], uint64_t u2[2]);

/* ---- ring switch helpers (BitZ src/ligerito.rs) ---- */
void orc_build_eq_lsb(const uint64_t *point, size_t k, uint64_t *out /* 2^k */);
void orc_sv_fold(const uint64_t *packed, size_t n, const uint64_t *eq, uint64_t *sv /* 128 */);
void orc_phi_from_words(const uint64_t *eq_hi, size_t n, const uint64_t *eq_r2 /* 128 */,
                        uint64_t *out);

/* ---- inputs ---- */
/* RFC 8439 ChaCha20 keystream, key = seed (LE u64, zero padded), nonce 0,
   block counter from `first_block`; writes n_words 16-byte words */
void orc_chacha_words(uint64_t seed, uint64_t first_word, uint64_t *out, size_t n_words);
void orc_chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3],
                        uint8_t out[64]);

/* ---- recursive opening ---- */
/* dense induced basis of a level's queries (ligerito.rs:1968-2072) */
void orc_induce_basis(int log_n, const uint64_t *queries, size_t nq, const uint64_t *w,
                      uint64_t *basis);

#ifdef __cplusplus
}
#endif
#endif
