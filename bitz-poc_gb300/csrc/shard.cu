// Lane-sharded BLAKE3 commit: one commit split over the lanes of its matrix.
//
// Every lane's NTT is independent (flock-core/src/ntt/additive_ntt_f128.rs:
// 176-191: the interleaved transform is the per-lane transform applied to
// each lane), and a BLAKE3 leaf is the non-root CV of the tree over the
// leaf's 1 KiB chunks, chunk i holding lanes 64 i .. 64 i + 63 of the
// position with i as its counter (flock-core/src/merkle.rs:160-201).  So rank
// `rank` of `world` (a power of two; L / world >= 64 lanes) commits lanes
// [rank L/world, (rank+1) L/world) as a commit of its own (a message shard in
// its own compact layout msg_shard[col * L/world + j] = msg[col * L + rank *
// L/world + j]), hashing its chunks with their global counters and reducing
// each of its rows to the CV of the aligned run of chunks it holds.  That CV
// is one node of every leaf's chunk tree.  After the ranks exchange those
// per-position CVs (32 bytes per position per rank; the only collective), any
// rank merges them into the leaf CVs and builds the Merkle tree: the root is
// the whole commit's root.
//
// The reference commits on one machine; these entry points have no
// counterpart there.  SHA-256 leaves hash each row sequentially across all
// lanes, so SHA-256 commits are not sharded (replicas only).
#include <cuda_runtime.h>

#include <string.h>

#include <string>

#include "../../include/bitz_gpu.h"
#include "runtime.h"

using namespace bz;

namespace {

bool pow2(uint64_t n) { return n && !(n & (n - 1)); }

// The shard shape of rank `rank` of `world` for the whole commit `full`.
int shard_shape(const bz_params *params, uint32_t world, uint32_t rank, Shape &out,
                std::string &why) {
    if (!params) {
        why = "params is null";
        return BZ_ERR_ARG;
    }
    if (params->hash_kind != 1) {
        why = "only BLAKE3 commits shard by lanes (SHA-256 leaves span every lane)";
        return BZ_ERR_SHAPE;
    }
    if (!pow2(world) || rank >= world) {
        why = "world must be a power of two and rank < world";
        return BZ_ERR_ARG;
    }
    uint32_t lw = 0;
    while ((1u << lw) < world) ++lw;
    if (params->log_batch_size < 6 + lw) {
        why = "each rank needs at least 64 lanes (one BLAKE3 chunk per position)";
        return BZ_ERR_SHAPE;
    }
    Shape full;
    int rc = shape_from_params(params, full, (size_t)1 << params->log_msg_len, why);
    if (rc) return rc;
    out = full;
    out.log_msg_len = full.log_msg_len - (int)lw;
    out.log_lanes = full.log_lanes - (int)lw;
    out.chunk0 = (uint64_t)rank << (out.log_lanes - 6);
    return BZ_OK;
}

}  // namespace

extern "C" {

int bz_commit_shard_device(bz_ctx *ctx, const uint64_t *d_msg_shard, size_t n_words,
                           const bz_params *params, uint32_t world, uint32_t rank,
                           bz_commitment **out) {
    if (!ctx || !d_msg_shard || !out) return BZ_ERR_ARG;
    *out = nullptr;
    Shape s;
    std::string why;
    int rc = shard_shape(params, world, rank, s, why);
    if (rc) return set_msg(ctx, rc, why);
    if (n_words != s.msg_words()) return set_msg(ctx, BZ_ERR_SHAPE, "shard length must be 2^log_msg_len / world");
    bz_commitment *c = nullptr;
    rc = alloc_commitment(ctx, s, &c);
    if (rc) return rc;
    rc = enqueue_commit(ctx, s, (const uint4 *)d_msg_shard, c, ctx->stream, schedule_for(ctx, s));
    if (rc) {
        bz_commitment_free(c);
        return rc;
    }
    *out = c;
    return BZ_OK;
}

int bz_commit_shard(bz_ctx *ctx, const uint64_t *msg_shard, size_t n_words,
                    const bz_params *params, uint32_t world, uint32_t rank,
                    bz_commitment **out) {
    if (!ctx || !msg_shard || !out) return BZ_ERR_ARG;
    *out = nullptr;
    void *d_msg = nullptr;
    const size_t bytes = n_words * 16;
    int rc = dev_alloc(ctx, bytes, &d_msg, true);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(d_msg, msg_shard, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        dev_free(ctx, d_msg, bytes, true);
        return set_err(ctx, BZ_ERR_CUDA, "H2D message shard", e);
    }
    rc = bz_commit_shard_device(ctx, (const uint64_t *)d_msg, n_words, params, world, rank, out);
    dev_free(ctx, d_msg, bytes, true);
    if (rc == BZ_OK) {
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            bz_commitment_free(*out);
            *out = nullptr;
            return set_err(ctx, BZ_ERR_CUDA, "shard commit", e);
        }
    }
    return rc;
}

int bz_commitment_leaf_cvs(bz_commitment *c, uint8_t *out, size_t n_leaves) {
    if (!c || !out) return BZ_ERR_ARG;
    bz_ctx *ctx = c->ctx;
    if (n_leaves != c->shape.n_leaves()) return set_msg(ctx, BZ_ERR_ARG, "leaf count");
    BZ_CUDA(ctx, cudaMemcpyAsync(out, c->d_tree, n_leaves * 32, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_merkle_from_shards(bz_ctx *ctx, const uint8_t *cvs, uint32_t world,
                          const bz_params *params, bz_commitment **out, uint8_t root[32]) {
    if (!ctx || !cvs || !out) return BZ_ERR_ARG;
    *out = nullptr;
    Shape shard;
    std::string why;
    int rc = shard_shape(params, world, 0, shard, why);
    if (rc) return set_msg(ctx, rc, why);
    Shape full;
    rc = shape_from_params(params, full, (size_t)1 << params->log_msg_len, why);
    if (rc) return set_msg(ctx, rc, why);
    const uint64_t n_leaves = full.n_leaves();
    bz_commitment *c = nullptr;
    rc = alloc_commitment(ctx, full, &c, /*with_codeword=*/false);
    if (rc) return rc;
    void *d_cvs = nullptr;
    const size_t bytes = (size_t)world * n_leaves * 32;
    rc = dev_alloc(ctx, bytes, &d_cvs, false);
    if (rc) {
        bz_commitment_free(c);
        return rc;
    }
    cudaError_t e = cudaMemcpyAsync(d_cvs, cvs, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        int n = launch_combine_shard_cvs((const uint8_t *)d_cvs, world, n_leaves, c->d_tree,
                                         ctx->stream);
        n += launch_merkle_levels(full, c->d_tree, ctx->stream, nullptr);
        ctx->launches += (uint64_t)n;
        e = cudaGetLastError();
    }
    dev_free(ctx, d_cvs, bytes, false);
    if (e != cudaSuccess) {
        bz_commitment_free(c);
        return set_err(ctx, BZ_ERR_CUDA, "shard tree", e);
    }
    rc = fetch_root(c);
    if (rc) {
        bz_commitment_free(c);
        return rc;
    }
    if (root) memcpy(root, c->root, 32);
    *out = c;
    return BZ_OK;
}

}  // extern "C"
