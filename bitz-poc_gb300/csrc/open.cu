// Recursive Ligerito opening against a device-resident commitment.
//
// Drives recursive_prover_with_basis_initial_impl
// (flock-core/src/pcs/ligerito.rs:3524-3884) with every array operation on
// the GPU and the Fiat-Shamir transcript on the host:
//
// level 0 (bz_ligerito_open_l0 stops after it)
//   observe label "flock-ligerito-basis-v0", target, initial root (:3566-3571)
//   first sumcheck message round_msg_lsb(f, basis)             (:2998-3007)
//   initial_k lane folds, round j ground with fold_grinding_bits[0] - j
//   bits when positive, each message observed                  (:3621-3657)
//   ligero_commit of f^1 (recursive_ks[0] lanes, rate
//   log_inv_rates[1]); observe its root                        (:3662-3679)
//   ood_samples[1] out-of-domain introduce + glue rounds       (:3686-3706)
//   grind_pow(grinding_bits[0]), sample_distinct_queries,
//   alpha_0 = sample_f128_vec(ceil_log2(queries[0]))           (:3713-3718)
//   open_initial: opened rows + Merkle multi-proof             (:3476-3481)
// recursive levels (bz_ligerito_prove)
//   induce the level's basis from its queries, introduce + glue (:3734-3748)
//   per level i: recursive_ks[i] folds with fold grinding     (:3755-3774)
//   last level: yr = f observed, grind, queries, final rows    (:3776-3860)
//   else: ligero_commit of the next level, OOD rounds, grind, queries,
//   alpha, rows, induce, introduce + glue                      (:3863-3946)
//
// The lookahead fold schedule of the reference (:3606-3651) gives a
// bit-identical transcript (an exact polynomial identity) and is not
// restated.  The induced basis uses the transposed-NTT form
// (induce_sumcheck_poly_via_ntt, :2124-2184), byte-identical to the dense
// form the reference picks for small levels (:2186-2222).  The claimed sums
// of introduced polynomials enter no message or proof field, so they are
// not computed.
#include <cuda_runtime.h>

#include <future>

#include <string.h>

#include <algorithm>
#include <new>
#include <set>
#include <utility>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "proof.h"
#include "runtime.h"
#include "transcript.h"

namespace {

uint32_t ceil_log2(uint64_t n) {
    uint32_t k = 0;
    while (((uint64_t)1 << k) < n) ++k;
    return k;
}

uint4 to_u4(const uint64_t v[2]) {
    return make_uint4((uint32_t)v[0], (uint32_t)(v[0] >> 32), (uint32_t)v[1],
                      (uint32_t)(v[1] >> 32));
}

// The running sumcheck prover (SumcheckProver, ligerito.rs:2981-3182) with f
// and the combined basis on the device.  Folds ping-pong between two halves
// of one allocation: A holds up to n/2 + n/2 elements (f, b), B up to
// n/4 + n/4, and round j writes the half it does not read.
struct Sumcheck {
    bz_ctx *ctx = nullptr;
    bz_transcript *transcript = nullptr;
    bzh::Transcript *tr = nullptr;
    void *buf = nullptr;
    size_t buf_bytes = 0;
    uint4 *A = nullptr, *B = nullptr;
    const uint64_t *f = nullptr;  // current arrays (the inputs before the first fold)
    uint64_t *b = nullptr;        // null while b is still the caller's input
    const uint64_t *b_in = nullptr;
    size_t len = 0;
    bool next_in_B = false;       // where the next fold writes
    std::vector<uint64_t> msgs;   // 4 words per SumcheckMessage
    bz::ArmedFold armed;          // the next round's fold, enqueued ahead of its challenge

    const uint64_t *basis() const { return b ? b : b_in; }

    void record(const uint64_t u0[2], const uint64_t u2[2]) {
        tr->observe_f128(u0);
        tr->observe_f128(u2);
        msgs.insert(msgs.end(), {u0[0], u0[1], u2[0], u2[1]});
    }

    int init(bz_ctx *c, bz_transcript *t, const uint64_t *f0, const uint64_t *b0, size_t n) {
        ctx = c;
        transcript = t;
        tr = bz_transcript_inner(t);
        buf_bytes = (n / 2) * 16 * 2 + (n / 4) * 16 * 2;
        int rc = bz::dev_alloc(ctx, buf_bytes, &buf, false);
        if (rc) return rc;
        A = (uint4 *)buf;
        B = A + n;
        f = f0;
        b_in = b0;
        len = n;
        return BZ_OK;
    }

    void release() {
        if (armed.live) {
            bz::fold_cancel(ctx, &armed);
            bz::reset_msg_ticket(ctx);
        }
        if (buf) bz::dev_free(ctx, buf, buf_bytes, false);
        buf = nullptr;
    }

    // SumcheckProver::new: the first message over (f, basis)
    int first_message() {
        uint64_t u0[2], u2[2];
        int rc = bz_round_msg_lsb(ctx, f, basis(), len, u0, u2);
        if (rc) return rc;
        record(u0, u2);
        return BZ_OK;
    }

    // one fold round: optional grind, challenge, fold, observe.  With
    // arm_next (the caller's next step is another fold round without a
    // grind), the next round's fold is enqueued before this round's message
    // is read, so its launch overlaps the host's wait and transcript work.
    int fold_round(uint32_t bits, std::vector<uint64_t> &fold_nonces, uint64_t r_out[2],
                   bool arm_next = false) {
        if (bits) {
            if (armed.live) return bz::set_msg(ctx, BZ_ERR_STATE, "grind behind an armed fold");
            uint64_t nonce;
            int rc = bz_transcript_grind_pow(ctx, transcript, bits, &nonce);
            if (rc) return rc;
            fold_nonces.push_back(nonce);
        }
        tr->sample_f128(r_out);
        uint4 *dst = next_in_B ? B : A;
        uint64_t *nf = (uint64_t *)dst, *nb = (uint64_t *)(dst + len / 2);
        const uint64_t *in_f = f, *in_b = basis();
        const size_t in_len = len;
        const bool was_armed = armed.live;
        uint32_t seq = 0;
        int rc = BZ_OK;
        if (armed.live) {
            if (armed.f != f || armed.b != basis() || armed.n != len || armed.nf != nf ||
                armed.nb != nb) {
                bz::fold_cancel(ctx, &armed);
                bz::reset_msg_ticket(ctx);
                return bz::set_msg(ctx, BZ_ERR_STATE, "armed fold does not match the round");
            }
            seq = armed.msg_seq;
            bz::fold_open(ctx, &armed, r_out);
        } else if ((rc = bz::fold_launch(ctx, f, basis(), len, r_out, nf, nb, &seq))) {
            return rc;
        }
        f = nf;
        b = nb;
        len /= 2;
        next_in_B = !next_in_B;
        if (arm_next && bz::fold_armable(ctx, len)) {
            uint4 *nd = next_in_B ? B : A;
            rc = bz::fold_arm(ctx, f, b, len, (uint64_t *)nd, (uint64_t *)(nd + len / 2), &armed);
        }
        uint64_t u0[2], u2[2];
        int wrc = bz::msg_wait(ctx, seq, u0, u2);
        if (wrc && was_armed && !rc) {
            // the gate ran out before r arrived (a host stall, or a tool that
            // completes each launch before returning): run the round unarmed
            if (armed.live) bz::fold_cancel(ctx, &armed);
            if (bz::gate_gave_up(ctx)) {
                bz::reset_msg_ticket(ctx);
                wrc = bz::fold_launch(ctx, in_f, in_b, in_len, r_out, nf, nb, &seq);
                if (!wrc) wrc = bz::msg_wait(ctx, seq, u0, u2);
            }
        }
        if (rc || wrc) {
            if (armed.live) bz::fold_cancel(ctx, &armed);
            bz::reset_msg_ticket(ctx);
            return rc ? rc : wrc;
        }
        record(u0, u2);
        return BZ_OK;
    }

    // introduce_new(b_new) + observe + glue(beta) (:3099-3145)
    int introduce_glue(const uint4 *b_new) {
        uint64_t u0[2], u2[2];
        int rc = bz_round_msg_lsb(ctx, f, (const uint64_t *)b_new, len, u0, u2);
        if (rc) return rc;
        record(u0, u2);
        uint64_t beta[2];
        tr->sample_f128(beta);
        ctx->launches += bz::launch_glue((uint4 *)b, b_new, len, to_u4(beta), ctx->stream);
        BZ_CUDA(ctx, cudaGetLastError());
        return BZ_OK;
    }

    // `count` out-of-domain rounds over the current n variables
    // (:3686-3706): z = sample_f128_vec(n); eq(z); (msg, y) =
    // introduce_new_with_eval(eq(z)); observe y, u0, u2; glue(beta)
    int ood(uint32_t count, std::vector<uint64_t> &ood_values) {
        if (!count) return BZ_OK;
        uint32_t n = 0;
        while (((size_t)1 << n) < len) ++n;
        const size_t parts = bz::dot_partials_count(len, ctx->num_sms);
        void *scratch = nullptr;
        const size_t bytes = (len + n + 1 + parts) * 16;
        int rc = bz::dev_alloc(ctx, bytes, &scratch, false);
        if (rc) return rc;
        uint4 *d_eq = (uint4 *)scratch, *d_z = d_eq + len, *d_y = d_z + n,
              *d_part = d_y + 1;
        std::vector<uint64_t> z(2 * (size_t)n);
        for (uint32_t s = 0; s < count && !rc; ++s) {
            for (uint32_t i = 0; i < n; ++i) tr->sample_f128(&z[2 * i]);
            if (n) cudaMemcpyAsync(d_z, z.data(), 16 * (size_t)n, cudaMemcpyHostToDevice,
                                   ctx->stream);
            ctx->launches += bz::launch_build_eq(d_z, n, d_eq, ctx->stream, ctx->num_sms);
            uint64_t u0[2], u2[2], y[2];
            rc = bz_round_msg_lsb(ctx, f, (const uint64_t *)d_eq, len, u0, u2);
            if (rc) break;
            ctx->launches += bz::launch_dot((const uint4 *)f, d_eq, len, d_part, d_y,
                                            ctx->stream, ctx->num_sms);
            if (cudaMemcpyAsync(y, d_y, 16, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
                cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
                rc = bz::set_msg(ctx, BZ_ERR_CUDA, "out-of-domain evaluation");
                break;
            }
            tr->observe_f128(y);
            ood_values.insert(ood_values.end(), {y[0], y[1]});
            record(u0, u2);
            uint64_t beta[2];
            tr->sample_f128(beta);
            ctx->launches += bz::launch_glue((uint4 *)b, d_eq, len, to_u4(beta), ctx->stream);
        }
        bz::dev_free(ctx, scratch, bytes, false);
        if (!rc && cudaGetLastError() != cudaSuccess)
            rc = bz::set_msg(ctx, BZ_ERR_CUDA, "out-of-domain round");
        return rc;
    }
};

// sample_distinct_queries (ligerito.rs:3191-3221)
std::vector<uint64_t> sample_queries(bzh::Transcript *tr, uint64_t block_len, uint32_t count) {
    std::set<uint64_t> seen;
    std::vector<uint64_t> out;
    while (out.size() < count) {
        uint64_t v[2];
        tr->sample_f128(v);
        const uint64_t q = v[0] % block_len;
        if (seen.insert(q).second) out.push_back(q);
    }
    std::sort(out.begin(), out.end());
    return out;
}

std::vector<uint64_t> sample_vec(bzh::Transcript *tr, uint32_t n) {
    std::vector<uint64_t> v(2 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) tr->sample_f128(&v[2 * i]);
    return v;
}

// opened rows (each 2^log_lanes elements) and the multi-proof, on stream st
int open_rows_on(bz_commitment *c, const std::vector<uint64_t> &queries, bzp::Level &out,
                 cudaStream_t st) {
    const size_t q = queries.size();
    const size_t lanes = c->shape.leaf_bytes() / 16;
    out.rows.lens.assign(q, lanes);
    out.rows.data.resize(q * lanes * 2);
    int rc = bz::commitment_rows_on(c, queries.data(), q, out.rows.data.data(), st);
    if (rc) return rc;
    size_t n_hashes = 0;
    rc = bz::commitment_multiproof_on(c, queries.data(), q, nullptr, 0, &n_hashes, st);
    if (rc) return rc;
    out.hashes.resize(n_hashes * 32);
    return bz::commitment_multiproof_on(c, queries.data(), q, out.hashes.data(), n_hashes,
                                        &n_hashes, st);
}

int open_rows(bz_commitment *c, const std::vector<uint64_t> &queries, bzp::Level &out) {
    return open_rows_on(c, queries, out, c->ctx->stream);
}

// The same opening on the context's side stream from its helper thread, so its
// gather and its device-to-host copy of the rows (the bulk of a level-0
// opening) overlap the work that follows on the context stream.  The side
// stream first waits for the context stream's work enqueued so far.
std::future<int> open_rows_async(bz_commitment *c, std::vector<uint64_t> queries,
                                 bzp::Level &out) {
    bz_ctx *ctx = c->ctx;
    cudaEvent_t ready = nullptr;
    if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) == cudaSuccess) {
        cudaEventRecord(ready, ctx->stream);
        cudaStreamWaitEvent(ctx->side_stream, ready, 0);
        cudaEventDestroy(ready);
    } else {
        cudaGetLastError();
        cudaStreamSynchronize(ctx->stream);
    }
    return bz::side_async(ctx, [c, q = std::move(queries), &out]() {
        return open_rows_on(c, q, out, c->ctx->side_stream);
    });
}

// The basis a level's queries induce over its 2^log_msg_cols message columns,
// on the device (caller frees *d_basis with dev_free): eq(alpha) weights on
// the queries scattered over the 2^(log_msg_cols + rate) codeword domain,
// transposed NTT, low outputs.
int induce_basis(bz_ctx *ctx, uint32_t log_msg_cols, uint32_t rate,
                 const std::vector<uint64_t> &queries, const std::vector<uint64_t> &alpha,
                 uint4 **d_basis, size_t *bytes_out) {
    const int log_d = (int)(log_msg_cols + rate);
    const size_t q = queries.size();
    const size_t n_alpha = alpha.size() / 2;
    const size_t n_w = (size_t)1 << n_alpha;  // eq(alpha) has 2^n_alpha >= q entries
    const size_t bytes = (((size_t)1 << log_d) + n_w + n_alpha) * 16 + q * 8 + 16;
    void *mem = nullptr;
    int rc = bz::dev_alloc(ctx, bytes, &mem, false);
    if (rc) return rc;
    uint4 *d_dom = (uint4 *)mem, *d_w = d_dom + ((size_t)1 << log_d), *d_alpha = d_w + n_w;
    uint64_t *d_pos = (uint64_t *)(d_alpha + n_alpha);
    const uint4 *d_tw = nullptr;
    rc = bz::get_twiddles(ctx, log_d, &d_tw);
    if (rc) {
        bz::dev_free(ctx, mem, bytes, false);
        return rc;
    }
    if (n_alpha)
        cudaMemcpyAsync(d_alpha, alpha.data(), 16 * n_alpha, cudaMemcpyHostToDevice, ctx->stream);
    if (q) cudaMemcpyAsync(d_pos, queries.data(), 8 * q, cudaMemcpyHostToDevice, ctx->stream);
    ctx->launches += bz::launch_build_eq(d_alpha, n_alpha, d_w, ctx->stream, ctx->num_sms);
    ctx->launches += bz::launch_induce_basis(d_dom, log_d, d_pos, d_w, (int)q, d_tw, ctx->stream);
    if (cudaGetLastError() != cudaSuccess) {
        bz::dev_free(ctx, mem, bytes, false);
        return bz::set_msg(ctx, BZ_ERR_CUDA, "induce basis");
    }
    *d_basis = d_dom;
    *bytes_out = bytes;
    return BZ_OK;
}

}  // namespace

struct bz_l0_opening {
    bz_ctx *ctx = nullptr;
    Sumcheck sc;
    std::vector<uint64_t> fold_nonces;
    std::vector<uint64_t> challenges;  // initial_k x {lo, hi}
    std::vector<uint64_t> ood_values;
    uint8_t root1[32] = {0};
    uint64_t grinding_nonce = 0;
    std::vector<uint64_t> queries;
    std::vector<uint64_t> alpha;       // ceil_log2(q) x {lo, hi}
    bzp::Level initial;                // opened rows + multi-proof
    std::future<int> initial_done;     // the opening of `initial`, when still in flight
    bz_commitment *level1 = nullptr;
    uint32_t lanes = 0, log_msg_cols0 = 0, rate0 = 0;
};

namespace {

// Status of the level-0 row opening (waits for it when still in flight).
int initial_rows(bz_l0_opening *o) {
    return o->initial_done.valid() ? o->initial_done.get() : BZ_OK;
}

void free_opening(bz_l0_opening *o) {
    if (!o) return;
    initial_rows(o);  // the helper thread writes o->initial
    if (o->level1) bz_commitment_free(o->level1);
    o->sc.release();
    delete o;
}

int open_level0(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                const uint64_t *d_packed, const uint64_t *d_basis, const uint64_t target[2],
                const bz_l0_config *cfg, bz_l0_opening **out) {
    bzh::Transcript *tr = bz_transcript_inner(transcript);
    if (!ctx || !tr || !c0 || !d_packed || !d_basis || !target || !cfg || !out)
        return BZ_ERR_ARG;
    *out = nullptr;
    if (c0->ctx != ctx) return bz::set_msg(ctx, BZ_ERR_ARG, "commitment of another context");
    if (!c0->d_cw) return bz::set_msg(ctx, BZ_ERR_STATE, "tree-only commitment: no codeword");
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
    o->log_msg_cols0 = n1;
    o->rate0 = (uint32_t)s.log_inv_rate;
    rc = o->sc.init(ctx, transcript, d_packed, d_basis, (size_t)1 << log_n);
    if (rc) {
        delete o;
        return rc;
    }
    auto fail = [&](int code) {
        free_opening(o);
        return code;
    };

    static const char kLabel[] = "flock-ligerito-basis-v0";
    tr->absorb_slice((const uint8_t *)kLabel, sizeof kLabel - 1);
    tr->observe_f128(target);
    tr->absorb_slice(c0->root, 32);

    if ((rc = o->sc.first_message())) return fail(rc);
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t bits = cfg->fold_grinding_bits0 > j ? cfg->fold_grinding_bits0 - j : 0;
        const bool arm = j + 1 < k && cfg->fold_grinding_bits0 <= j + 1;
        uint64_t r[2];
        if ((rc = o->sc.fold_round(bits, o->fold_nonces, r, arm))) return fail(rc);
        o->challenges.insert(o->challenges.end(), {r[0], r[1]});
    }

    rc = bz_ligero_commit_device(ctx, o->sc.f, n1 - cfg->recursive_k0, cfg->recursive_k0,
                                 cfg->log_inv_rate1, cfg->hash_kind, &o->level1, o->root1);
    if (rc) return fail(rc);
    tr->absorb_slice(o->root1, 32);
    if ((rc = o->sc.ood(cfg->ood_samples1, o->ood_values))) return fail(rc);

    rc = bz_transcript_grind_pow(ctx, transcript, cfg->grinding_bits0, &o->grinding_nonce);
    if (rc) return fail(rc);
    o->queries = sample_queries(tr, block_len0, cfg->queries0);
    o->alpha = sample_vec(tr, ceil_log2(cfg->queries0));
    o->initial_done = open_rows_async(c0, o->queries, o->initial);
    *out = o;
    return BZ_OK;
}

}  // namespace

extern "C" {

int bz_ligerito_open_l0(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                        const uint64_t *d_packed, const uint64_t *d_basis,
                        const uint64_t target[2], const bz_l0_config *cfg,
                        bz_l0_opening **out) {
    int rc = open_level0(ctx, transcript, c0, d_packed, d_basis, target, cfg, out);
    if (rc) return rc;
    if ((rc = initial_rows(*out))) {
        free_opening(*out);
        *out = nullptr;
    }
    return rc;
}

int bz_l0_opening_sizes(const bz_l0_opening *o, bz_l0_sizes *sz) {
    if (!o || !sz) return BZ_ERR_ARG;
    sz->n_sumcheck = o->sc.msgs.size() / 4;
    sz->n_fold_nonces = o->fold_nonces.size();
    sz->n_queries = o->queries.size();
    sz->n_alpha = o->alpha.size() / 2;
    sz->row_len = o->lanes;
    sz->n_proof_hashes = o->initial.hashes.size() / 32;
    sz->folded_len = o->sc.len;
    sz->n_ood_values = o->ood_values.size() / 2;
    return BZ_OK;
}

int bz_l0_opening_copy(const bz_l0_opening *o, uint64_t *sumcheck, uint64_t *fold_nonces,
                       uint64_t *challenges, uint8_t root1[32], uint64_t *grinding_nonce,
                       uint64_t *queries, uint64_t *alpha, uint64_t *rows, uint8_t *proof) {
    if (!o) return BZ_ERR_ARG;
    auto cp = [](auto *dst, const auto &v) {
        if (dst && !v.empty()) std::copy(v.begin(), v.end(), dst);
    };
    cp(sumcheck, o->sc.msgs);
    cp(fold_nonces, o->fold_nonces);
    cp(challenges, o->challenges);
    if (root1) std::copy(o->root1, o->root1 + 32, root1);
    if (grinding_nonce) *grinding_nonce = o->grinding_nonce;
    cp(queries, o->queries);
    cp(alpha, o->alpha);
    cp(rows, o->initial.rows.data);
    cp(proof, o->initial.hashes);
    return BZ_OK;
}

struct bz_rows {
    std::vector<uint64_t, bzp::NoInitAlloc<uint64_t>> data;
};

int bz_l0_opening_take_rows(bz_l0_opening *o, bz_rows **rows, const uint64_t **data) {
    if (!o || !rows || !data) return BZ_ERR_ARG;
    *rows = nullptr;
    *data = nullptr;
    const int rc = initial_rows(o);  // the helper thread writes o->initial
    if (rc) return rc;
    // the rows move out once: a second take, or rows that never arrived,
    // find an array of the wrong size
    const size_t want = o->queries.size() * (size_t)o->lanes * 2;
    if (want && o->initial.rows.data.size() != want) return BZ_ERR_STATE;
    bz_rows *r = new (std::nothrow) bz_rows();
    if (!r) return BZ_ERR_NOMEM;
    r->data = std::move(o->initial.rows.data);
    o->initial.rows.data.clear();
    *rows = r;
    *data = r->data.data();
    return BZ_OK;
}

int bz_rows_free(bz_rows *rows) {
    delete rows;
    return BZ_OK;
}

int bz_l0_opening_ood_values(const bz_l0_opening *o, uint64_t *values) {
    if (!o) return BZ_ERR_ARG;
    if (values && !o->ood_values.empty())
        std::copy(o->ood_values.begin(), o->ood_values.end(), values);
    return BZ_OK;
}

bz_commitment *bz_l0_opening_level1(bz_l0_opening *o) { return o ? o->level1 : nullptr; }

int bz_l0_opening_folded(const bz_l0_opening *o, const uint64_t **d_f1, const uint64_t **d_b1,
                         size_t *n1) {
    if (!o) return BZ_ERR_ARG;
    if (d_f1) *d_f1 = o->sc.f;
    if (d_b1) *d_b1 = o->sc.basis();
    if (n1) *n1 = o->sc.len;
    return BZ_OK;
}

int bz_l0_opening_free(bz_l0_opening *o) {
    if (!o) return BZ_ERR_ARG;
    free_opening(o);
    return BZ_OK;
}

int bz_ligerito_prove(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                      const uint64_t *d_packed, const uint64_t *d_basis, const uint64_t target[2],
                      const bz_ligerito_config *cfg, bz_ligerito_proof **out) {
    if (!ctx || !cfg || !out || !c0) return BZ_ERR_ARG;
    *out = nullptr;
    const uint32_t r = cfg->recursive_steps;
    if (r < 1 || !cfg->recursive_ks || !cfg->log_inv_rates || !cfg->queries ||
        !cfg->grinding_bits)
        return bz::set_msg(ctx, BZ_ERR_ARG, "config needs recursive_steps >= 1 and its arrays");
    auto fold_bits = [&](uint32_t lvl) {
        return cfg->fold_grinding_bits ? cfg->fold_grinding_bits[lvl] : 0u;
    };
    auto ood_count = [&](uint32_t lvl) { return cfg->ood_samples ? cfg->ood_samples[lvl] : 0u; };
    if (ood_count(0) != 0) return bz::set_msg(ctx, BZ_ERR_SHAPE, "L0 must not take OOD samples");
    if (cfg->log_inv_rates[0] != (uint32_t)c0->shape.log_inv_rate)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "log_inv_rates[0] differs from the commitment");
    // every level's shape before any transcript work
    {
        uint32_t n = (uint32_t)c0->shape.log_msg_len - cfg->initial_k;
        for (uint32_t i = 0; i < r; ++i) {
            if (cfg->recursive_ks[i] > n)
                return bz::set_msg(ctx, BZ_ERR_SHAPE, "recursive_ks exceed the folded length");
            const uint32_t cols = n - cfg->recursive_ks[i];
            if (cols + cfg->log_inv_rates[i + 1] > 40)
                return bz::set_msg(ctx, BZ_ERR_SHAPE, "level shape too large");
            if (cfg->queries[i + 1] > ((uint64_t)1 << (cols + cfg->log_inv_rates[i + 1])))
                return bz::set_msg(ctx, BZ_ERR_SHAPE, "queries exceed a level's block length");
            n = cols;
        }
    }

    bz_l0_config l0;
    l0.initial_k = cfg->initial_k;
    l0.recursive_k0 = cfg->recursive_ks[0];
    l0.log_inv_rate1 = cfg->log_inv_rates[1];
    l0.fold_grinding_bits0 = fold_bits(0);
    l0.grinding_bits0 = cfg->grinding_bits[0];
    l0.queries0 = cfg->queries[0];
    l0.hash_kind = cfg->hash_kind;
    l0.ood_samples1 = ood_count(1);
    bz_l0_opening *o = nullptr;
    int rc = open_level0(ctx, transcript, c0, d_packed, d_basis, target, &l0, &o);
    if (rc) return rc;
    bzh::Transcript *tr = bz_transcript_inner(transcript);
    Sumcheck &sc = o->sc;

    bz_ligerito_proof *p = new (std::nothrow) bz_ligerito_proof();
    std::vector<bz_commitment *> levels{o->level1};
    o->level1 = nullptr;  // owned by `levels` from here
    auto finish = [&](int code) {
        for (bz_commitment *c : levels)
            if (c) bz_commitment_free(c);
        free_opening(o);
        if (code) delete p;
        return code;
    };
    if (!p) return finish(BZ_ERR_NOMEM);
    memcpy(p->initial_root, c0->root, 32);
    p->recursive_roots.insert(p->recursive_roots.end(), o->root1, o->root1 + 32);
    p->grinding_nonces.push_back(o->grinding_nonce);
    p->ood_values = o->ood_values;
    p->fold_grinding_nonces = o->fold_nonces;

    // basis induced by the level-0 queries over f^1's columns (:3722-3748)
    uint4 *d_ind = nullptr;
    size_t ind_bytes = 0;
    rc = induce_basis(ctx, o->log_msg_cols0, o->rate0, o->queries, o->alpha, &d_ind, &ind_bytes);
    if (rc) return finish(rc);
    rc = sc.introduce_glue(d_ind);
    bz::dev_free(ctx, d_ind, ind_bytes, false);
    if (rc) return finish(rc);

    for (uint32_t i = 0; i < r; ++i) {
        bz_commitment *prev = levels.back();
        const uint32_t prev_rate = cfg->log_inv_rates[i + 1];
        for (uint32_t j = 0; j < cfg->recursive_ks[i]; ++j) {
            const uint32_t bits = fold_bits(i + 1) > j ? fold_bits(i + 1) - j : 0;
            const bool arm = j + 1 < cfg->recursive_ks[i] && fold_bits(i + 1) <= j + 1;
            uint64_t ri[2];
            if ((rc = sc.fold_round(bits, p->fold_grinding_nonces, ri, arm))) return finish(rc);
        }
        const uint64_t block_len = prev->shape.n_leaves();
        if (i == r - 1) {
            // finish(): yr = f, every element observed (:3776-3790)
            p->yr.resize(2 * sc.len);
            if (cudaMemcpyAsync(p->yr.data(), sc.f, 16 * sc.len, cudaMemcpyDeviceToHost,
                                ctx->stream) != cudaSuccess ||
                cudaStreamSynchronize(ctx->stream) != cudaSuccess)
                return finish(bz::set_msg(ctx, BZ_ERR_CUDA, "final polynomial"));
            for (size_t e = 0; e < sc.len; ++e) tr->observe_f128(&p->yr[2 * e]);
            uint64_t nonce;
            rc = bz_transcript_grind_pow(ctx, transcript, cfg->grinding_bits[i + 1], &nonce);
            if (rc) return finish(rc);
            p->grinding_nonces.push_back(nonce);
            const std::vector<uint64_t> qs = sample_queries(tr, block_len, cfg->queries[i + 1]);
            if ((rc = open_rows(prev, qs, p->fin))) return finish(rc);
            p->sumcheck = sc.msgs;
            if ((rc = initial_rows(o))) return finish(rc);
            p->initial = std::move(o->initial);
            *out = p;
            return finish(BZ_OK);
        }
        // commit the next level (:3863-3882)
        uint32_t n_next = 0;
        while (((size_t)1 << n_next) < sc.len) ++n_next;
        const uint32_t k_next = cfg->recursive_ks[i + 1];
        bz_commitment *next = nullptr;
        uint8_t root_next[32];
        rc = bz_ligero_commit_device(ctx, sc.f, n_next - k_next, k_next, cfg->log_inv_rates[i + 2],
                                     cfg->hash_kind, &next, root_next);
        if (rc) return finish(rc);
        levels.push_back(next);
        tr->absorb_slice(root_next, 32);
        p->recursive_roots.insert(p->recursive_roots.end(), root_next, root_next + 32);
        if ((rc = sc.ood(ood_count(i + 2), p->ood_values))) return finish(rc);
        uint64_t nonce;
        rc = bz_transcript_grind_pow(ctx, transcript, cfg->grinding_bits[i + 1], &nonce);
        if (rc) return finish(rc);
        p->grinding_nonces.push_back(nonce);
        const std::vector<uint64_t> qs = sample_queries(tr, block_len, cfg->queries[i + 1]);
        const std::vector<uint64_t> alpha = sample_vec(tr, ceil_log2(cfg->queries[i + 1]));
        p->recursive.emplace_back();
        if ((rc = open_rows(prev, qs, p->recursive.back()))) return finish(rc);
        rc = induce_basis(ctx, n_next, prev_rate, qs, alpha, &d_ind, &ind_bytes);
        if (rc) return finish(rc);
        rc = sc.introduce_glue(d_ind);
        bz::dev_free(ctx, d_ind, ind_bytes, false);
        if (rc) return finish(rc);
    }
    return finish(bz::set_msg(ctx, BZ_ERR_STATE, "unreachable"));
}

}  // extern "C"
