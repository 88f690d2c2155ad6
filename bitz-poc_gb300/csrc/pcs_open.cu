// BitZ's BinaryPcs opening around the Ligerito prover (src/binary_pcs.rs):
//
//  * prove_round0 (:320-325 -> prove_ood_round_packed,
//    src/ligerito_flock.rs:1520-1557): bind the round's header, grind when
//    the difficulty is nonzero, draw zeta, evaluate the packed message's
//    multilinear extension at (zeta, zeta^2, zeta^4, ...) on the GPU, absorb
//    the value.
//  * ring switch (ring_switch_prove_with, src/ligerito.rs:445-496): eq of the
//    high point coordinates, the 128 bit-column sums s_v (absorbed), seven
//    challenges r'', the weight table B(y) = Phi_r''(eq_hi[y]) and its claimed
//    sum beta0 = sum_u eq(r'')[u] * transpose(s)_u.
//  * open_basis (:341-367): eta, basis += eta * eq(round-0 point)
//    (add_ood_basis, src/ligerito_flock.rs:1590-1650), target += eta * y,
//    then the recursive Ligerito proof.
//  * open_bit_mle (:413-431): ring switch on point[7..], then open_basis.
//
// The arrays (packed message, eq tables, basis) stay on the device; the
// transcript and the handful of scalars it binds (zeta's powers, beta0,
// eta * y) are computed on the host.
#include <cuda_runtime.h>

#include <string.h>

#include <new>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "runtime.h"
#include "transcript.h"

struct bz_round0 {
    uint32_t vars = 0;
    std::vector<uint64_t> point;  // vars x {lo, hi}
    uint64_t y[2] = {0, 0};
    int has_nonce = 0;
    uint64_t nonce = 0;
};

namespace {

constexpr int kOodBlockLog = 12;  // OOD_BLOCK_LOG, src/ligerito_flock.rs:1377

uint4 to_u4(const uint64_t v[2]) {
    return make_uint4((uint32_t)v[0], (uint32_t)(v[0] >> 32), (uint32_t)v[1],
                      (uint32_t)(v[1] >> 32));
}

void absorb_u64(bzh::Transcript *tr, uint64_t v) {
    uint8_t b[8];
    for (int i = 0; i < 8; ++i) b[i] = (uint8_t)(v >> (8 * i));
    tr->absorb_slice(b, 8);
}

void absorb_u32(bzh::Transcript *tr, uint32_t v) {
    uint8_t b[4];
    for (int i = 0; i < 4; ++i) b[i] = (uint8_t)(v >> (8 * i));
    tr->absorb_slice(b, 4);
}

void absorb_str(bzh::Transcript *tr, const char *s) {
    tr->absorb_slice((const uint8_t *)s, strlen(s));
}

// absorb_gf_slice (src/ligerito.rs:57-67): absorb_slice(tag || words LE)
void absorb_gf_slice(bzh::Transcript *tr, uint8_t tag, const uint64_t *v, size_t n) {
    std::vector<uint8_t> b(1 + 16 * n);
    b[0] = tag;
    for (size_t i = 0; i < 2 * n; ++i)
        for (int k = 0; k < 8; ++k) b[1 + 8 * i + k] = (uint8_t)(v[i] >> (8 * k));
    tr->absorb_slice(b.data(), b.size());
}

// grind_and_absorb_in_domain (src/piop/spartan/grinding.rs:139-172,
// 264-268): frame, 32-byte seed challenge, smallest nonce of
// blake3(seed || nonce), nonce frame.
int grind_in_domain(bz_ctx *ctx, bzh::Transcript *tr, const char *domain, uint64_t index,
                    uint32_t bits, uint64_t *nonce) {
    if (bits < 1 || bits > 256) return bz::set_msg(ctx, BZ_ERR_ARG, "grinding bits out of range");
    absorb_str(tr, "bitz/spartan/fiat-shamir-grinding/v1");
    absorb_str(tr, domain);
    absorb_u64(tr, index);
    absorb_u32(tr, bits);
    uint8_t seed[32];
    tr->challenge(seed, 32);
    int rc = bz_pow_first_nonce(ctx, seed, 32, bits, 0, ~0ull, nonce);
    if (rc) return rc;
    absorb_str(tr, "bitz/spartan/fiat-shamir-grinding/nonce/v1");
    absorb_u64(tr, *nonce);
    return BZ_OK;
}

// eq(point[0..lo)) and eq(point[lo..vars)) on the device, lo = min(vars, 12)
struct EqSplit {
    void *mem = nullptr;
    size_t bytes = 0;
    uint4 *tail = nullptr, *head = nullptr;
    int lo = 0;
    size_t n_head = 0;
    int build(bz_ctx *ctx, const std::vector<uint64_t> &point, uint32_t vars) {
        lo = (int)(vars < (uint32_t)kOodBlockLog ? vars : kOodBlockLog);
        const uint32_t hi_vars = vars - (uint32_t)lo;
        n_head = (size_t)1 << hi_vars;
        bytes = (((size_t)1 << lo) + n_head + vars + 1) * 16;
        int rc = bz::dev_alloc(ctx, bytes, &mem, false);
        if (rc) return rc;
        tail = (uint4 *)mem;
        head = tail + ((size_t)1 << lo);
        uint4 *d_pt = head + n_head;
        if (vars)
            cudaMemcpyAsync(d_pt, point.data(), 16 * (size_t)vars, cudaMemcpyHostToDevice,
                            ctx->stream);
        ctx->launches += bz::launch_build_eq(d_pt, (size_t)lo, tail, ctx->stream, ctx->num_sms);
        ctx->launches += bz::launch_build_eq(d_pt + lo, hi_vars, head, ctx->stream, ctx->num_sms);
        return cudaGetLastError() == cudaSuccess ? BZ_OK
                                                 : bz::set_msg(ctx, BZ_ERR_CUDA, "eq tables");
    }
    void release(bz_ctx *ctx) {
        if (mem) bz::dev_free(ctx, mem, bytes, false);
        mem = nullptr;
    }
};

bool pow2(size_t n) { return n && !(n & (n - 1)); }

uint32_t log2_exact(size_t n) {
    uint32_t k = 0;
    while (((size_t)1 << k) < n) ++k;
    return k;
}

// the 128 x 128 bit transpose of s (src/ligerito.rs:108-120)
void transpose_bits_128(const uint64_t *s, uint64_t *out) {
    memset(out, 0, 256 * 8);
    for (int v = 0; v < 128; ++v)
        for (int u = 0; u < 128; ++u)
            if ((s[2 * v + (u >> 6)] >> (u & 63)) & 1) out[2 * u + (v >> 6)] |= 1ull << (v & 63);
}

}  // namespace

extern "C" {

int bz_pcs_prove_round0(bz_ctx *ctx, bz_transcript *transcript, const uint64_t *d_packed,
                        size_t n, uint32_t grinding_bits, bz_round0 **out) {
    bzh::Transcript *tr = bz_transcript_inner(transcript);
    if (!ctx || !tr || !d_packed || !out) return BZ_ERR_ARG;
    *out = nullptr;
    if (!pow2(n) || n > ((size_t)1 << 40))
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "packed message length must be a power of two");
    bz_round0 *r = new (std::nothrow) bz_round0();
    if (!r) return BZ_ERR_NOMEM;
    r->vars = log2_exact(n);
    absorb_str(tr, "bitz/core/ood-round/v1");
    absorb_u64(tr, r->vars);
    absorb_u32(tr, grinding_bits);
    if (grinding_bits) {
        int rc = grind_in_domain(ctx, tr, "bitz/core/ood-round-grinding/v1", 0, grinding_bits,
                                 &r->nonce);
        if (rc) {
            delete r;
            return rc;
        }
        r->has_nonce = 1;
    }
    uint64_t cur[2];
    tr->sample_f128(cur);  // zeta
    r->point.resize(2 * (size_t)r->vars);
    for (uint32_t i = 0; i < r->vars; ++i) {
        r->point[2 * i] = cur[0];
        r->point[2 * i + 1] = cur[1];
        uint64_t sq[2];
        bz::hgf_mul(cur, cur, sq);
        cur[0] = sq[0];
        cur[1] = sq[1];
    }
    EqSplit eq;
    int rc = eq.build(ctx, r->point, r->vars);
    void *tmp = nullptr;
    const size_t parts = bz::split_dot_partials(eq.n_head, ctx->num_sms);
    if (!rc) rc = bz::dev_alloc(ctx, (parts + 1) * 16, &tmp, false);
    if (!rc) {
        uint4 *d_part = (uint4 *)tmp, *d_y = d_part + parts;
        ctx->launches += bz::launch_split_dot((const uint4 *)d_packed, eq.tail, eq.lo, eq.head,
                                              eq.n_head, d_part, d_y, ctx->stream, ctx->num_sms);
        if (cudaMemcpyAsync(r->y, d_y, 16, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
            rc = bz::set_msg(ctx, BZ_ERR_CUDA, "out-of-domain evaluation");
    }
    if (tmp) bz::dev_free(ctx, tmp, 0, false);
    eq.release(ctx);
    if (rc) {
        delete r;
        return rc;
    }
    absorb_gf_slice(tr, 0x50, r->y, 1);  // absorb_ood_value (src/ligerito.rs:69-73)
    *out = r;
    return BZ_OK;
}

int bz_round0_get(const bz_round0 *r, uint64_t y[2], int *has_nonce, uint64_t *nonce,
                  uint32_t *vars) {
    if (!r) return BZ_ERR_ARG;
    if (y) {
        y[0] = r->y[0];
        y[1] = r->y[1];
    }
    if (has_nonce) *has_nonce = r->has_nonce;
    if (nonce) *nonce = r->nonce;
    if (vars) *vars = r->vars;
    return BZ_OK;
}

int bz_round0_point(const bz_round0 *r, uint64_t *point) {
    if (!r || (r->vars && !point)) return BZ_ERR_ARG;
    std::copy(r->point.begin(), r->point.end(), point);
    return BZ_OK;
}

int bz_round0_free(bz_round0 *r) {
    delete r;
    return BZ_OK;
}

int bz_pcs_ring_switch(bz_ctx *ctx, bz_transcript *transcript, const uint64_t *d_packed, size_t n,
                       const uint64_t *r_hi, uint64_t s_v[256], uint64_t *d_basis,
                       uint64_t target[2]) {
    bzh::Transcript *tr = bz_transcript_inner(transcript);
    if (!ctx || !tr || !d_packed || !s_v || !d_basis || !target) return BZ_ERR_ARG;
    if (!pow2(n) || n > ((size_t)1 << 40))
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "packed message length must be a power of two");
    const uint32_t m = log2_exact(n);
    if (m && !r_hi) return BZ_ERR_ARG;
    void *d_eq = nullptr;  // eq(r_hi) (n entries), then eq(r'') (128 entries)
    int rc = bz::dev_alloc(ctx, (n + 128) * 16, &d_eq, false);
    if (rc) return rc;
    uint64_t *d_eq_r2 = (uint64_t *)d_eq + 2 * n;
    auto done = [&](int code) {
        bz::dev_free(ctx, d_eq, 0, false);
        return code;
    };
    if ((rc = bz_build_eq_lsb(ctx, r_hi, m, (uint64_t *)d_eq))) return done(rc);
    if ((rc = bz_sv_fold(ctx, d_packed, (const uint64_t *)d_eq, n, s_v))) return done(rc);
    absorb_gf_slice(tr, 0x20, s_v, 128);  // absorb_sv (src/ligerito.rs:248-250)
    uint64_t r2[14], eq_r2[256];
    for (int i = 0; i < 7; ++i) tr->sample_f128(r2 + 2 * i);
    // eq(r'') on the device (128 entries), copied back for beta0 and Phi
    if ((rc = bz_build_eq_lsb(ctx, r2, 7, d_eq_r2))) return done(rc);
    if ((rc = bz_memcpy_d2h(ctx, eq_r2, d_eq_r2, 128 * 16))) return done(rc);
    uint64_t s_u[256];
    transpose_bits_128(s_v, s_u);
    target[0] = target[1] = 0;
    for (int u = 0; u < 128; ++u) {
        uint64_t p[2];
        bz::hgf_mul(s_u + 2 * u, eq_r2 + 2 * u, p);
        target[0] ^= p[0];
        target[1] ^= p[1];
    }
    rc = bz_phi_from_words(ctx, (const uint64_t *)d_eq, n, eq_r2, d_basis);
    return done(rc);
}

int bz_pcs_open_basis(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                      const uint64_t *d_packed, const bz_round0 *round0, uint64_t *d_basis,
                      const uint64_t target[2], const bz_ligerito_config *cfg,
                      bz_ligerito_proof **out) {
    bzh::Transcript *tr = bz_transcript_inner(transcript);
    if (!ctx || !tr || !c0 || !d_packed || !round0 || !d_basis || !target || !cfg || !out)
        return BZ_ERR_ARG;
    const size_t n = (size_t)1 << c0->shape.log_msg_len;
    if (round0->vars != (uint32_t)c0->shape.log_msg_len)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "round-0 point dimension differs from the witness");
    uint64_t eta[2];
    tr->sample_f128(eta);
    EqSplit eq;
    int rc = eq.build(ctx, round0->point, round0->vars);
    if (rc) return rc;
    ctx->launches += bz::launch_eq_axpy((uint4 *)d_basis, eq.tail, eq.lo, eq.head, to_u4(eta), n,
                                        ctx->stream);
    eq.release(ctx);
    BZ_CUDA(ctx, cudaGetLastError());
    uint64_t ey[2], t2[2];
    bz::hgf_mul(eta, round0->y, ey);
    t2[0] = target[0] ^ ey[0];
    t2[1] = target[1] ^ ey[1];
    return bz_ligerito_prove(ctx, transcript, c0, d_packed, d_basis, t2, cfg, out);
}

int bz_pcs_open_bit_mle(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                        const uint64_t *d_packed, const bz_round0 *round0, const uint64_t *point,
                        size_t point_len, const bz_ligerito_config *cfg, uint64_t s_v[256],
                        bz_ligerito_proof **out) {
    if (!ctx || !c0 || !point || !s_v || !out) return BZ_ERR_ARG;
    const uint32_t m = (uint32_t)c0->shape.log_msg_len;
    if (point_len != (size_t)m + 7)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "bit-MLE point length must be packed_log + 7");
    const size_t n = (size_t)1 << m;
    void *d_b = nullptr;
    int rc = bz::dev_alloc(ctx, n * 16, &d_b, false);
    if (rc) return rc;
    uint64_t target[2];
    rc = bz_pcs_ring_switch(ctx, transcript, d_packed, n, point + 2 * 7, s_v, (uint64_t *)d_b,
                            target);
    if (!rc)
        rc = bz_pcs_open_basis(ctx, transcript, c0, d_packed, round0, (uint64_t *)d_b, target,
                               cfg, out);
    bz::dev_free(ctx, d_b, 0, false);
    return rc;
}

}  // extern "C"
