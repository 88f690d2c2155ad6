// Bit-matrix ingest for the binary PCS (BitZ src/ligerito.rs:19-33, 629-717;
// src/ligerito_flock.rs:198-245).
//
// A witness is a 2^row_vars x 2^col_vars matrix of bits (IntegerMatrixLayout,
// src/pcs.rs:14-41, cell (b, c) at flat index (b << col_vars) | c).  Three
// layouts of it:
//  * cells: one u128 per cell holding 0 or 1 (the reference's data tensor);
//  * rows: per column c, its 2^row_vars bits packed 64 per u64 word
//    (repack_leaf_bits), row c = words [c * W, (c + 1) * W), W = ceil(2^row_vars / 64);
//  * packed columns: per group g of 64 columns, 2^row_vars words whose bit k
//    is column 64g + k's bit i (pack_columns_from_rows /
//    rows_from_packed_cols, 64 x 64 bit transposes).
// The packed GF(2^128) message the commit takes is the rows buffer itself
// read as {lo, hi} word pairs (commit_rs_flock_from_rows pushes
// {row[2i], row[2i+1]} for every row in order), so it needs no kernel.
//
// The transposes run one warp per 64 x 64 block with __ballot_sync: ballot j
// collects bit j of the 32 lanes' words, i.e. 32 bits of one output word.
#include <cuda_runtime.h>

#include "bz_internal.h"

namespace bz {

namespace {

// rows[c * W + w] bit j = cell(64 w + j, c); cells holding anything but 0/1
// set *bad.
__global__ void repack_kernel(const uint4 *cells, int row_vars, int col_vars, uint64_t words,
                              uint64_t *rows, unsigned int *bad) {
    const uint64_t cols = (uint64_t)1 << col_vars, nrows = (uint64_t)1 << row_vars;
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= cols * words) return;
    const uint64_t c = idx & (cols - 1), w = idx >> col_vars;
    uint64_t word = 0;
    bool ok = true;
    for (int j = 0; j < 64; ++j) {
        const uint64_t b = 64 * w + (uint64_t)j;
        if (b >= nrows) break;
        const uint4 v = cells[(b << col_vars) | c];
        ok &= (v.y | v.z | v.w) == 0 && v.x <= 1;
        word |= (uint64_t)(v.x & 1) << j;
    }
    if (!ok) atomicOr(bad, 1u);
    rows[c * words + w] = word;
}

// packed[g * R + i] bit k = rows[(64 g + k) * W + i / 64] bit i % 64, one warp
// per (g, word index wi).
__global__ void pack_cols_kernel(const uint64_t *rows, uint64_t nrows, uint64_t cols,
                                 uint64_t words, uint64_t groups, uint64_t *packed) {
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= groups * words) return;
    const uint64_t g = warp / words, wi = warp % words;
    const uint64_t c0 = 64 * g + lane, c1 = c0 + 32;
    const uint64_t a = c0 < cols ? rows[c0 * words + wi] : 0;
    const uint64_t b = c1 < cols ? rows[c1 * words + wi] : 0;
    uint64_t keep0 = 0, keep1 = 0;  // output words t = lane and t = lane + 32
#pragma unroll 8
    for (int t = 0; t < 64; ++t) {
        const uint32_t lo = __ballot_sync(0xffffffffu, (a >> t) & 1);
        const uint32_t hi = __ballot_sync(0xffffffffu, (b >> t) & 1);
        const uint64_t v = (uint64_t)lo | ((uint64_t)hi << 32);
        if ((t & 31) == lane) {
            if (t < 32) keep0 = v;
            else keep1 = v;
        }
    }
    const uint64_t i0 = 64 * wi + lane, i1 = i0 + 32;
    if (i0 < nrows) packed[g * nrows + i0] = keep0;
    if (i1 < nrows) packed[g * nrows + i1] = keep1;
}

// rows[(64 g + k) * W + wi] bit t = packed[g * R + 64 wi + t] bit k.
__global__ void unpack_cols_kernel(const uint64_t *packed, uint64_t nrows, uint64_t cols,
                                   uint64_t words, uint64_t groups, uint64_t *rows) {
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= groups * words) return;
    const uint64_t g = warp / words, wi = warp % words;
    const uint64_t i0 = 64 * wi + lane, i1 = i0 + 32;
    const uint64_t a = i0 < nrows ? packed[g * nrows + i0] : 0;
    const uint64_t b = i1 < nrows ? packed[g * nrows + i1] : 0;
    uint64_t keep0 = 0, keep1 = 0;  // rows k = lane and k = lane + 32
#pragma unroll 8
    for (int k = 0; k < 64; ++k) {
        const uint32_t lo = __ballot_sync(0xffffffffu, (a >> k) & 1);
        const uint32_t hi = __ballot_sync(0xffffffffu, (b >> k) & 1);
        const uint64_t v = (uint64_t)lo | ((uint64_t)hi << 32);
        if ((k & 31) == lane) {
            if (k < 32) keep0 = v;
            else keep1 = v;
        }
    }
    const uint64_t c0 = 64 * g + lane, c1 = c0 + 32;
    if (c0 < cols) rows[c0 * words + wi] = keep0;
    if (c1 < cols) rows[c1 * words + wi] = keep1;
}

unsigned blocks_for(uint64_t threads) { return (unsigned)((threads + 255) / 256); }

}  // namespace

int launch_repack_leaf_bits(const uint4 *d_cells, int row_vars, int col_vars, uint64_t *d_rows,
                            unsigned int *d_bad, cudaStream_t st) {
    const uint64_t words = ((((uint64_t)1) << row_vars) + 63) / 64;
    const uint64_t n = (((uint64_t)1) << col_vars) * words;
    repack_kernel<<<blocks_for(n), 256, 0, st>>>(d_cells, row_vars, col_vars, words, d_rows, d_bad);
    return 1;
}

int launch_pack_columns(const uint64_t *d_rows, int row_vars, int col_vars, uint64_t *d_packed,
                        cudaStream_t st) {
    const uint64_t nrows = (uint64_t)1 << row_vars, cols = (uint64_t)1 << col_vars;
    const uint64_t words = (nrows + 63) / 64, groups = (cols + 63) / 64;
    pack_cols_kernel<<<blocks_for(32 * groups * words), 256, 0, st>>>(d_rows, nrows, cols, words,
                                                                      groups, d_packed);
    return 1;
}

int launch_unpack_columns(const uint64_t *d_packed, int row_vars, int col_vars, uint64_t *d_rows,
                          cudaStream_t st) {
    const uint64_t nrows = (uint64_t)1 << row_vars, cols = (uint64_t)1 << col_vars;
    const uint64_t words = (nrows + 63) / 64, groups = (cols + 63) / 64;
    unpack_cols_kernel<<<blocks_for(32 * groups * words), 256, 0, st>>>(d_packed, nrows, cols,
                                                                        words, groups, d_rows);
    return 1;
}

}  // namespace bz

// ---- C ABI -------------------------------------------------------------------
#include "runtime.h"

namespace {
bool shape_ok(uint32_t row_vars, uint32_t col_vars) {
    return row_vars <= 40 && col_vars <= 40 && row_vars + col_vars <= 44;
}
}  // namespace

extern "C" {

int bz_repack_leaf_bits(bz_ctx *ctx, const uint64_t *d_cells, uint32_t row_vars,
                        uint32_t col_vars, uint64_t *d_rows) {
    if (!ctx || !d_cells || !d_rows) return BZ_ERR_ARG;
    if (!shape_ok(row_vars, col_vars)) return bz::set_msg(ctx, BZ_ERR_SHAPE, "matrix too large");
    unsigned int *d_bad = (unsigned int *)((uint8_t *)ctx->d_small + 512);
    BZ_CUDA(ctx, cudaMemsetAsync(d_bad, 0, 4, ctx->stream));
    ctx->launches += bz::launch_repack_leaf_bits((const uint4 *)d_cells, (int)row_vars,
                                                 (int)col_vars, d_rows, d_bad, ctx->stream);
    BZ_CUDA(ctx, cudaGetLastError());
    unsigned int *h_bad = (unsigned int *)((uint8_t *)ctx->h_small + 512);
    BZ_CUDA(ctx, cudaMemcpyAsync(h_bad, d_bad, 4, cudaMemcpyDeviceToHost, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (*h_bad) return bz::set_msg(ctx, BZ_ERR_ARG, "binary matrix cell holds a value above 1");
    return BZ_OK;
}

int bz_pack_columns_from_rows(bz_ctx *ctx, const uint64_t *d_rows, uint32_t row_vars,
                              uint32_t col_vars, uint64_t *d_packed_cols) {
    if (!ctx || !d_rows || !d_packed_cols) return BZ_ERR_ARG;
    if (!shape_ok(row_vars, col_vars)) return bz::set_msg(ctx, BZ_ERR_SHAPE, "matrix too large");
    ctx->launches += bz::launch_pack_columns(d_rows, (int)row_vars, (int)col_vars, d_packed_cols,
                                             ctx->stream);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_rows_from_packed_cols(bz_ctx *ctx, const uint64_t *d_packed_cols, uint32_t row_vars,
                             uint32_t col_vars, uint64_t *d_rows) {
    if (!ctx || !d_rows || !d_packed_cols) return BZ_ERR_ARG;
    if (!shape_ok(row_vars, col_vars)) return bz::set_msg(ctx, BZ_ERR_SHAPE, "matrix too large");
    ctx->launches += bz::launch_unpack_columns(d_packed_cols, (int)row_vars, (int)col_vars, d_rows,
                                               ctx->stream);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_commit_rows(bz_ctx *ctx, const uint64_t *d_rows, uint32_t row_vars, uint32_t col_vars,
                   uint32_t log_inv_rate, uint32_t log_batch, uint32_t hash_kind,
                   bz_commitment **out, uint8_t root[32]) {
    if (!ctx || !d_rows || !out) return BZ_ERR_ARG;
    // commit_rs_flock_from_rows (src/ligerito_flock.rs:198-245): t >= 7 and
    // log_batch < m_p; the packed message is the rows buffer.
    if (row_vars < 7) return bz::set_msg(ctx, BZ_ERR_SHAPE, "packing needs row_vars >= 7");
    const uint32_t m_p = row_vars - 7 + col_vars;
    if (log_batch >= m_p)
        return bz::set_msg(ctx, BZ_ERR_SHAPE, "log_batch must leave a position variable");
    bz_params p;
    p.log_msg_len = m_p;
    p.log_inv_rate = log_inv_rate;
    p.log_batch_size = log_batch;
    p.hash_kind = hash_kind;
    return bz_commit_device(ctx, d_rows, (size_t)1 << m_p, &p, out, root);
}

}  // extern "C"
