// Batched grand-product GKR prover on the GPU: BitZ's gpgkr_prove
// (src/bitz/gkr.rs:113-282) over GrandProductCircuit::batched_eval
// (gkr.rs:93-108), the dense rounds with the column-free weights.  The
// packed forest (src/bitz/forest.rs) proves the same transcript from packed
// bits and row images; bz_gkr_forest_prove takes those inputs, builds the
// leaf grid on the device and runs the same rounds.
//
// The reference's transcript (the spongefish crate) stays with the caller:
// every round hands its two field elements to a callback, which absorbs them
// and returns the next challenge, so a Rust prover keeps its own
// ProverState.  The product layers, the fold of each round by the previous
// challenge and the round sums run on the GPU; per round the kernel's last
// CTA posts the two reduced sums to mapped host memory, and the host
// multiplies them by the running eq factor and calls the transcript.
#include <cuda_runtime.h>

#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "runtime.h"

using namespace bz;

namespace {

struct Gf {
    uint64_t w[2] = {0, 0};
};

Gf gmul(const Gf &a, const Gf &b) {
    Gf o;
    hgf_mul(a.w, b.w, o.w);
    return o;
}
Gf gadd(const Gf &a, const Gf &b) {
    Gf o;
    o.w[0] = a.w[0] ^ b.w[0];
    o.w[1] = a.w[1] ^ b.w[1];
    return o;
}
bool gzero(const Gf &a) { return !a.w[0] && !a.w[1]; }
Gf gone() {
    Gf o;
    o.w[0] = 1;
    return o;
}
// eq(r, z) = r z + (1 - r)(1 - z) (src/bitz/mod.rs:328-331).
Gf eq_factor(const Gf &r, const Gf &z) {
    return gadd(gmul(r, z), gmul(gadd(gone(), r), gadd(gone(), z)));
}
// v0 + rho (v1 - v0)
Gf fold(const Gf &rho, const Gf &v0, const Gf &v1) { return gadd(v0, gmul(rho, gadd(v1, v0))); }

bool pow2(size_t n) { return n && !(n & (n - 1)); }
int log2u(size_t n) {
    int l = 0;
    while (((size_t)1 << l) < n) ++l;
    return l;
}

uint4 to_u4(const Gf &a) {
    return make_uint4((uint32_t)a.w[0], (uint32_t)(a.w[0] >> 32), (uint32_t)a.w[1],
                      (uint32_t)(a.w[1] >> 32));
}

struct DevBuf {
    bz_ctx *ctx;
    void *p = nullptr;
    explicit DevBuf(bz_ctx *c) : ctx(c) {}
    ~DevBuf() {
        if (p) dev_free(ctx, p, 0, false);
    }
};

// The whole proof from device leaves (n of them, overwritten: the leaf layer
// is folded in place as the rounds go).
int gkr_run(bz_ctx *ctx, uint4 *d_leaves, size_t n, size_t groups, const uint64_t *point,
            bz_gkr_transcript_fn fn, void *user, uint64_t *roots, uint64_t *out_point,
            uint64_t out_claim[2]) {
    cudaStream_t st = ctx->stream;
    const int L = log2u(n), S = log2u(groups), layers = L - S;
    // layers 1 .. layers above the leaves, each half the one below
    DevBuf upper(ctx), eqa(ctx), eqb(ctx), scratch(ctx);
    int rc = dev_alloc(ctx, n * 16, &upper.p, false);
    if (!rc) rc = dev_alloc(ctx, std::max<size_t>(n / 4, 1) * 16, &eqa.p, false);
    if (!rc) rc = dev_alloc(ctx, std::max<size_t>(n / 4, 1) * 16, &eqb.p, false);
    const size_t part_bytes = fold_partials_bytes(0);
    if (!rc) rc = dev_alloc(ctx, part_bytes + 64 * 16 + 64, &scratch.p, false);
    if (rc) return rc;
    uint64_t *d_partials = (uint64_t *)scratch.p;
    uint4 *d_point = (uint4 *)((uint8_t *)scratch.p + part_bytes);
    uint64_t *d_msg = (uint64_t *)((uint8_t *)scratch.p + part_bytes + 64 * 16);
    std::vector<uint4 *> layer(layers + 1);
    layer[0] = d_leaves;
    size_t off = 0;
    for (int j = 1; j <= layers; ++j) {
        layer[j] = (uint4 *)upper.p + off;
        off += n >> j;
        ctx->launches += launch_gkr_product(layer[j - 1], n >> j, layer[j], st, ctx->num_sms);
    }
    BZ_CUDA(ctx, cudaGetLastError());
    if (roots)
        BZ_CUDA(ctx, cudaMemcpyAsync(roots, layer[layers], groups * 16, cudaMemcpyDeviceToHost,
                                     st));
    // MSB-first point of the current layer (gkr.rs:113-119)
    std::vector<Gf> p(S);
    for (int i = 0; i < S; ++i) {
        p[S - 1 - i].w[0] = point[2 * i];
        p[S - 1 - i].w[1] = point[2 * i + 1];
    }
    Gf claim;
    for (int j = layers - 1; j >= 0; --j) {
        const int k = L - j - 1;  // coordinates of this layer's point
        uint4 *l = layer[j], *r = layer[j] + ((size_t)1 << k);
        Gf factor = gone(), rho;
        std::vector<Gf> next;
        bool pending = false;
        if (k > 0) {
            // weights of the first round: eq over the k - 1 lowest (little-endian) coordinates
            std::vector<uint64_t> ext(2 * (size_t)(k - 1) + 2, 0);
            for (int i = 0; i < k - 1; ++i) {
                ext[2 * i] = p[k - 1 - i].w[0];
                ext[2 * i + 1] = p[k - 1 - i].w[1];
            }
            if (k > 1)
                BZ_CUDA(ctx, cudaMemcpyAsync(d_point, ext.data(), (size_t)(k - 1) * 16,
                                             cudaMemcpyHostToDevice, st));
            ctx->launches += launch_build_eq(d_point, (size_t)(k - 1), (uint4 *)eqa.p, st,
                                             ctx->num_sms);
            uint4 *w = (uint4 *)eqa.p, *w_next = (uint4 *)eqb.p;
            for (int rnd = 0; rnd < k; ++rnd) {
                const int remaining = k - 1 - rnd;
                const size_t h = (size_t)1 << remaining;
                const Gf &z = p[rnd];
                // the round's last CTA posts the two sums to the mapped
                // mailbox: no finish kernel, copy or stream synchronisation
                const MsgPost post = next_msg_post(ctx);
                ctx->launches += launch_gkr_round(l, r, w, h, pending, to_u4(rho), gzero(z),
                                                  remaining ? w_next : nullptr, d_partials,
                                                  d_msg, st, ctx->num_sms, &post);
                BZ_CUDA(ctx, cudaGetLastError());
                Gf se, si;
                rc = msg_wait(ctx, post.seq_val, se.w, si.w);
                if (rc) {
                    reset_msg_ticket(ctx);
                    return rc;
                }
                se = gmul(factor, se);
                si = gmul(factor, si);
                const uint64_t msg[4] = {se.w[0], se.w[1], si.w[0], si.w[1]};
                Gf ch;
                if (fn(user, BZ_GKR_ROUND, msg, ch.w) != 0)
                    return set_msg(ctx, BZ_ERR_STATE, "the transcript callback failed");
                next.push_back(ch);
                rho = ch;
                pending = true;
                factor = gmul(factor, eq_factor(ch, z));
                std::swap(w, w_next);
            }
        }
        // the close (gkr.rs:270-281): the last fold of the two-entry halves
        // two entries per half still to fold, or (a layer without rounds) one
        uint64_t lr[8] = {0};
        const size_t take = pending ? 32 : 16;
        BZ_CUDA(ctx, cudaMemcpyAsync(lr, l, take, cudaMemcpyDeviceToHost, st));
        BZ_CUDA(ctx, cudaMemcpyAsync(lr + 4, r, take, cudaMemcpyDeviceToHost, st));
        BZ_CUDA(ctx, cudaStreamSynchronize(st));
        Gf l0, l1, r0, r1;
        l0.w[0] = lr[0], l0.w[1] = lr[1], l1.w[0] = lr[2], l1.w[1] = lr[3];
        r0.w[0] = lr[4], r0.w[1] = lr[5], r1.w[0] = lr[6], r1.w[1] = lr[7];
        if (pending) {
            l0 = fold(rho, l0, l1);
            r0 = fold(rho, r0, r1);
        }
        const uint64_t msg[4] = {l0.w[0], l0.w[1], r0.w[0], r0.w[1]};
        Gf rc;
        if (fn(user, BZ_GKR_CLOSE, msg, rc.w) != 0)
            return set_msg(ctx, BZ_ERR_STATE, "the transcript callback failed");
        claim = fold(rc, l0, r0);
        p.clear();
        p.push_back(rc);
        p.insert(p.end(), next.begin(), next.end());
    }
    for (int i = 0; i < L; ++i) {
        out_point[2 * i] = p[L - 1 - i].w[0];
        out_point[2 * i + 1] = p[L - 1 - i].w[1];
    }
    out_claim[0] = claim.w[0];
    out_claim[1] = claim.w[1];
    return BZ_OK;
}

int check_shape(bz_ctx *ctx, size_t n, size_t groups) {
    if (!pow2(n) || n < 2) return set_msg(ctx, BZ_ERR_SHAPE, "leaves: a power of two, at least 2");
    if (!pow2(groups) || groups >= n)
        return set_msg(ctx, BZ_ERR_SHAPE, "groups: a power of two below the leaf count");
    if (log2u(n) > 40) return set_msg(ctx, BZ_ERR_SHAPE, "too many leaves");
    return BZ_OK;
}

}  // namespace

extern "C" {

int bz_gkr_prove_device(bz_ctx *ctx, uint64_t *d_leaves, size_t n_leaves, size_t groups,
                        const uint64_t *point, bz_gkr_transcript_fn fn, void *user,
                        uint64_t *roots, uint64_t *out_point, uint64_t out_claim[2]) {
    if (!ctx || !d_leaves || !fn || !out_point || !out_claim || (groups > 1 && !point))
        return BZ_ERR_ARG;
    int rc = check_shape(ctx, n_leaves, groups);
    if (rc) return rc;
    return gkr_run(ctx, (uint4 *)d_leaves, n_leaves, groups, point, fn, user, roots, out_point,
                   out_claim);
}

int bz_gkr_prove(bz_ctx *ctx, const uint64_t *leaves, size_t n_leaves, size_t groups,
                 const uint64_t *point, bz_gkr_transcript_fn fn, void *user, uint64_t *roots,
                 uint64_t *out_point, uint64_t out_claim[2]) {
    if (!ctx || !leaves || !fn || !out_point || !out_claim || (groups > 1 && !point))
        return BZ_ERR_ARG;
    int rc = check_shape(ctx, n_leaves, groups);
    if (rc) return rc;
    DevBuf d(ctx);
    rc = dev_alloc(ctx, n_leaves * 16, &d.p, false);
    if (rc) return rc;
    BZ_CUDA(ctx, cudaMemcpyAsync(d.p, leaves, n_leaves * 16, cudaMemcpyHostToDevice,
                                 ctx->stream));
    return gkr_run(ctx, (uint4 *)d.p, n_leaves, groups, point, fn, user, roots, out_point,
                   out_claim);
}

int bz_gkr_forest_prove(bz_ctx *ctx, const uint64_t *packed, const uint64_t *images, int t,
                        int s, const uint64_t *zeta, bz_gkr_transcript_fn fn, void *user,
                        uint64_t *roots, uint64_t *out_point, uint64_t out_claim[2]) {
    if (!ctx || !packed || !images || !fn || !out_point || !out_claim || (s > 0 && !zeta))
        return BZ_ERR_ARG;
    if (t < 1 || s < 0 || t + s > 40)
        return set_msg(ctx, BZ_ERR_SHAPE, "forest: t >= 1 rows bits, t + s <= 40");
    const size_t rows = (size_t)1 << t, cols = (size_t)1 << s, n = rows * cols;
    const size_t groups64 = (cols + 63) / 64;
    DevBuf d_leaves(ctx), d_in(ctx);
    int rc = dev_alloc(ctx, n * 16, &d_leaves.p, false);
    if (!rc) rc = dev_alloc(ctx, groups64 * rows * 8 + rows * 16, &d_in.p, false);
    if (rc) return rc;
    uint64_t *d_packed = (uint64_t *)d_in.p;
    uint4 *d_images = (uint4 *)((uint8_t *)d_in.p + groups64 * rows * 8);
    BZ_CUDA(ctx, cudaMemcpyAsync(d_packed, packed, groups64 * rows * 8, cudaMemcpyHostToDevice,
                                 ctx->stream));
    BZ_CUDA(ctx, cudaMemcpyAsync(d_images, images, rows * 16, cudaMemcpyHostToDevice,
                                 ctx->stream));
    ctx->launches += launch_gkr_forest_leaves(d_packed, d_images, t, s, (uint4 *)d_leaves.p,
                                              ctx->stream, ctx->num_sms);
    BZ_CUDA(ctx, cudaGetLastError());
    return gkr_run(ctx, (uint4 *)d_leaves.p, n, cols, zeta, fn, user, roots, out_point,
                   out_claim);
}

}  // extern "C"
