// Level-0 Ligerito opening against a device-resident commitment.
//
// Drives recursive_prover_with_basis_initial_impl
// (flock-core/src/pcs/ligerito.rs:3566-3720) from its first observation up
// to the opened level-0 rows, with every array operation on the GPU and the
// Fiat-Shamir transcript on the host:
//
//   observe label "flock-ligerito-basis-v0", target, initial root (:3566-3571)
//   first sumcheck message round_msg_lsb(f, basis)             (:2998-3007)
//   initial_k lane folds, round j ground with fold_grinding_bits[0] - j
//   bits when positive, each message observed                  (:3621-3657)
//   ligero_commit of f^1 (recursive_ks[0] lanes, rate
//   log_inv_rates[1]); observe its root                        (:3662-3679)
//   grind_pow(grinding_bits[0]), sample_distinct_queries,
//   alpha_0 = sample_f128_vec(ceil_log2(queries[0]))           (:3713-3718)
//   open_initial: opened rows + Merkle multi-proof             (:3476-3481)
//
// The level-1 OOD rounds (:3686-3706) take ood_samples[1] samples; this driver
// covers configurations with none.  What follows in the reference (inducing
// the level-0 basis from the opened rows, the recursive levels) continues from
// the folded arrays and the level-1 commitment this driver leaves resident.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <set>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "runtime.h"
#include "transcript.h"

struct bz_l0_opening {
    bz_ctx *ctx = nullptr;
    std::vector<uint64_t> sumcheck;      // (1 + initial_k) x {u0.lo, u0.hi, u2.lo, u2.hi}
    std::vector<uint64_t> fold_nonces;
    std::vector<uint64_t> challenges;    // initial_k x {lo, hi}
    uint8_t root1[32] = {0};
    uint64_t grinding_nonce = 0;
    std::vector<uint64_t> queries;
    std::vector<uint64_t> alpha;         // ceil_log2(q) x {lo, hi}
    std::vector<uint64_t> rows;          // q x 2^initial_k x {lo, hi}
    std::vector<uint8_t> proof;          // n_hashes x 32
    bz_commitment *level1 = nullptr;
    void *fold_buf = nullptr;            // both ping-pong halves of the folds
    size_t fold_bytes = 0;
    const uint64_t *d_f1 = nullptr, *d_b1 = nullptr;
    size_t n1 = 0;
    uint32_t lanes = 0;
};

namespace {

void observe_u(bzh::Transcript &t, const uint64_t u0[2], const uint64_t u2[2]) {
    t.observe_f128(u0);
    t.observe_f128(u2);
}

uint32_t ceil_log2(uint64_t n) {
    uint32_t k = 0;
    while (((uint64_t)1 << k) < n) ++k;
    return k;
}

void free_opening(bz_l0_opening *o) {
    if (!o) return;
    if (o->level1) bz_commitment_free(o->level1);
    if (o->fold_buf) bz::dev_free(o->ctx, o->fold_buf, o->fold_bytes, false);
    delete o;
}

}  // namespace

extern "C" {

int bz_ligerito_open_l0(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                        const uint64_t *d_packed, const uint64_t *d_basis,
                        const uint64_t target[2], const bz_l0_config *cfg,
                        bz_l0_opening **out) {
    bzh::Transcript *tr = bz_transcript_inner(transcript);
    if (!ctx || !tr || !c0 || !d_packed || !d_basis || !target || !cfg || !out)
        return BZ_ERR_ARG;
    *out = nullptr;
    if (c0->ctx != ctx) return bz::set_msg(ctx, BZ_ERR_ARG, "commitment of another context");
    const bz::Shape &s = c0->shape;
    const uint32_t log_n = (uint32_t)s.log_msg_len, k = cfg->initial_k;
    if (k != (uint32_t)s.log_lanes)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "initial_k must equal the commitment's lanes");
    if (k == 0 || k > log_n) return bz::set_msg(ctx, BZ_ERR_SHAPE, "initial_k out of range");
    const uint32_t n1 = log_n - k;
    if (cfg->recursive_k0 > n1)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "recursive_ks[0] exceeds the folded length");
    const uint64_t block_len0 = s.n_leaves();
    if (cfg->queries0 > block_len0)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "queries[0] exceeds the level-0 block length");
    if (cfg->hash_kind > 1) return bz::set_msg(ctx, BZ_ERR_ARG, "bad hash kind");
    int rc = bz::fetch_root(c0);
    if (rc) return rc;

    bz_l0_opening *o = new (std::nothrow) bz_l0_opening();
    if (!o) return BZ_ERR_NOMEM;
    o->ctx = ctx;
    o->lanes = 1u << k;
    const size_t n = (size_t)1 << log_n;
    // ping-pong: round j writes n >> (j+1) elements of f and of b; even
    // rounds into half A (n/2 + n/2 elements), odd rounds into half B (n/4 +
    // n/4), so no round reads the buffer it writes
    o->fold_bytes = (n / 2) * 16 * 2 + (n / 4) * 16 * 2;
    rc = bz::dev_alloc(ctx, o->fold_bytes, &o->fold_buf, false);
    if (rc) {
        delete o;
        return rc;
    }
    uint4 *A = (uint4 *)o->fold_buf;
    uint4 *B = A + n;  // A holds n/2 f + n/2 b = n elements
    auto fail = [&](int code) {
        free_opening(o);
        return code;
    };

    static const char kLabel[] = "flock-ligerito-basis-v0";
    tr->absorb_slice((const uint8_t *)kLabel, sizeof kLabel - 1);
    tr->observe_f128(target);
    tr->absorb_slice(c0->root, 32);

    uint64_t u0[2], u2[2];
    rc = bz_round_msg_lsb(ctx, d_packed, d_basis, n, u0, u2);
    if (rc) return fail(rc);
    observe_u(*tr, u0, u2);
    o->sumcheck.insert(o->sumcheck.end(), {u0[0], u0[1], u2[0], u2[1]});

    const uint64_t *f = d_packed, *b = d_basis;
    size_t len = n;
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t bits = cfg->fold_grinding_bits0 > j ? cfg->fold_grinding_bits0 - j : 0;
        if (bits) {
            uint64_t nonce;
            rc = bz_transcript_grind_pow(ctx, transcript, bits, &nonce);
            if (rc) return fail(rc);
            o->fold_nonces.push_back(nonce);
        }
        uint64_t r[2];
        tr->sample_f128(r);
        o->challenges.insert(o->challenges.end(), {r[0], r[1]});
        uint4 *dst = (j & 1) ? B : A;
        uint64_t *nf = (uint64_t *)dst, *nb = (uint64_t *)(dst + len / 2);
        rc = bz_fold_and_msg_lsb(ctx, f, b, len, r, nf, nb, u0, u2);
        if (rc) return fail(rc);
        observe_u(*tr, u0, u2);
        o->sumcheck.insert(o->sumcheck.end(), {u0[0], u0[1], u2[0], u2[1]});
        f = nf;
        b = nb;
        len /= 2;
    }
    o->d_f1 = f;
    o->d_b1 = b;
    o->n1 = len;

    rc = bz_ligero_commit_device(ctx, f, n1 - cfg->recursive_k0, cfg->recursive_k0,
                                 cfg->log_inv_rate1, cfg->hash_kind, &o->level1, o->root1);
    if (rc) return fail(rc);
    tr->absorb_slice(o->root1, 32);

    rc = bz_transcript_grind_pow(ctx, transcript, cfg->grinding_bits0, &o->grinding_nonce);
    if (rc) return fail(rc);

    // sample_distinct_queries (ligerito.rs:3191-3221)
    std::set<uint64_t> seen;
    while (o->queries.size() < cfg->queries0) {
        uint64_t v[2];
        tr->sample_f128(v);
        const uint64_t q = v[0] % block_len0;
        if (seen.insert(q).second) o->queries.push_back(q);
    }
    std::sort(o->queries.begin(), o->queries.end());
    const uint32_t n_alpha = ceil_log2(cfg->queries0);
    for (uint32_t i = 0; i < n_alpha; ++i) {
        uint64_t a[2];
        tr->sample_f128(a);
        o->alpha.insert(o->alpha.end(), {a[0], a[1]});
    }

    const size_t q = o->queries.size();
    o->rows.resize(q * o->lanes * 2);
    rc = bz_commitment_rows(c0, o->queries.data(), q, o->rows.data());
    if (rc) return fail(rc);
    size_t n_hashes = 0;
    rc = bz_commitment_multiproof(c0, o->queries.data(), q, nullptr, 0, &n_hashes);
    if (rc) return fail(rc);
    o->proof.resize(n_hashes * 32);
    rc = bz_commitment_multiproof(c0, o->queries.data(), q, o->proof.data(), n_hashes, &n_hashes);
    if (rc) return fail(rc);
    *out = o;
    return BZ_OK;
}

int bz_l0_opening_sizes(const bz_l0_opening *o, bz_l0_sizes *sz) {
    if (!o || !sz) return BZ_ERR_ARG;
    sz->n_sumcheck = o->sumcheck.size() / 4;
    sz->n_fold_nonces = o->fold_nonces.size();
    sz->n_queries = o->queries.size();
    sz->n_alpha = o->alpha.size() / 2;
    sz->row_len = o->lanes;
    sz->n_proof_hashes = o->proof.size() / 32;
    sz->folded_len = o->n1;
    return BZ_OK;
}

int bz_l0_opening_copy(const bz_l0_opening *o, uint64_t *sumcheck, uint64_t *fold_nonces,
                       uint64_t *challenges, uint8_t root1[32], uint64_t *grinding_nonce,
                       uint64_t *queries, uint64_t *alpha, uint64_t *rows, uint8_t *proof) {
    if (!o) return BZ_ERR_ARG;
    auto cp = [](auto *dst, const auto &v) {
        if (dst && !v.empty()) std::copy(v.begin(), v.end(), dst);
    };
    cp(sumcheck, o->sumcheck);
    cp(fold_nonces, o->fold_nonces);
    cp(challenges, o->challenges);
    if (root1) std::copy(o->root1, o->root1 + 32, root1);
    if (grinding_nonce) *grinding_nonce = o->grinding_nonce;
    cp(queries, o->queries);
    cp(alpha, o->alpha);
    cp(rows, o->rows);
    cp(proof, o->proof);
    return BZ_OK;
}

bz_commitment *bz_l0_opening_level1(bz_l0_opening *o) { return o ? o->level1 : nullptr; }

int bz_l0_opening_folded(const bz_l0_opening *o, const uint64_t **d_f1, const uint64_t **d_b1,
                         size_t *n1) {
    if (!o) return BZ_ERR_ARG;
    if (d_f1) *d_f1 = o->d_f1;
    if (d_b1) *d_b1 = o->d_b1;
    if (n1) *n1 = o->n1;
    return BZ_OK;
}

int bz_l0_opening_free(bz_l0_opening *o) {
    if (!o) return BZ_ERR_ARG;
    free_opening(o);
    return BZ_OK;
}

}  // extern "C"
