// Device bodies of the Merkle leaf and level kernels (the tree layout and
// hashing rules are described at the top of merkle.cu).  merkle.cu wraps each
// body in a kernel of its own; the persistent batch kernel (persist.cu) calls
// the same bodies for its work items, with its own shared-memory layout.
#pragma once
#include <stdint.h>

#include "hash.cuh"

namespace bz {

// ---------------------------------------------------------------------------
// BLAKE3 leaves, C >= 1 chunks per leaf, C <= 256.
// Each thread computes one chunk CV; the CTA (T <= 256 threads = T chunks =
// T / C leaves, T a power of two >= C) reduces groups of C CVs to leaf CVs in
// shared memory.  Small trees launch smaller CTAs so the chunks spread over
// the SMs (a chunk's 16 compressions are sequential).
// ---------------------------------------------------------------------------
//
// Body: the CTA's blockDim.x chunks from chunk_base (a multiple of blockDim.x,
// blockDim.x a multiple of C); cvs holds blockDim.x padded rows of 9 words.
__device__ __forceinline__ void b3_leaves_chunked_body(const uint4 *cw, uint64_t n_chunks,
                                                       uint32_t *tree_leaves, int log_c,
                                                       uint64_t chunk0, uint64_t chunk_base,
                                                       uint32_t (*cvs)[9]) {
    const uint64_t chunk = chunk_base + threadIdx.x;
    const uint64_t c_in_leaf = chunk0 + (chunk & ((1u << log_c) - 1));
    uint32_t cv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) cv[i] = kIV[i];
    if (chunk < n_chunks) {
        const uint4 *p = cw + chunk * 64;  // 64 elements = 1024 bytes
#pragma unroll 1
        for (int blk = 0; blk < 16; ++blk) {
            uint32_t m[16];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 v = __ldcs(p + blk * 4 + q);
                m[4 * q] = v.x;
                m[4 * q + 1] = v.y;
                m[4 * q + 2] = v.z;
                m[4 * q + 3] = v.w;
            }
            const uint32_t flags = (blk == 0 ? B3_CHUNK_START : 0) | (blk == 15 ? B3_CHUNK_END : 0);
            b3_compress_cv(cv, m, c_in_leaf, 64, flags);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) cvs[threadIdx.x][i] = cv[i];
    __syncthreads();
    // In-leaf reduction: level s merges nodes (2j, 2j+1) within groups of C.
    for (int s = 0; s < log_c; ++s) {
        const int stride = 1 << s;
        const int t = threadIdx.x;
        if ((t & ((stride << 1) - 1)) == 0 && t + stride < (int)blockDim.x) {
            uint32_t out[8];
            b3_parent(cvs[t], cvs[t + stride], out);
#pragma unroll
            for (int i = 0; i < 8; ++i) cvs[t][i] = out[i];
        }
        __syncthreads();
    }
    if ((threadIdx.x & ((1 << log_c) - 1)) == 0 && chunk < n_chunks) {
        const uint64_t leaf = chunk >> log_c;
#pragma unroll
        for (int i = 0; i < 8; ++i) tree_leaves[leaf * 8 + i] = cvs[threadIdx.x][i];
    }
}

// BLAKE3 leaves of at most one chunk (leaf_bytes = 16 * 2^log_lanes <= 1024).
// Body: leaves first, first + step, .. below n_leaves.
__device__ __forceinline__ void b3_leaves_small_body(const uint4 *cw, int log_lanes,
                                                     uint64_t n_leaves, uint32_t *tree_leaves,
                                                     uint64_t first, uint64_t step) {
    for (uint64_t leaf = first; leaf < n_leaves; leaf += step) {
        const uint32_t elems = 1u << log_lanes;  // 16-byte elements
        const uint32_t bytes = elems * 16;
        const uint32_t nblk = (bytes + 63) / 64;
        const uint4 *p = cw + leaf * elems;
        uint32_t cv[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) cv[i] = kIV[i];
        for (uint32_t blk = 0; blk < nblk; ++blk) {
            uint32_t m[16];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t e = blk * 4 + q;
                const uint4 v = e < elems ? p[e] : make_uint4(0, 0, 0, 0);
                m[4 * q] = v.x;
                m[4 * q + 1] = v.y;
                m[4 * q + 2] = v.z;
                m[4 * q + 3] = v.w;
            }
            const uint32_t len = min(64u, bytes - blk * 64);
            const uint32_t flags =
                (blk == 0 ? B3_CHUNK_START : 0) | (blk == nblk - 1 ? B3_CHUNK_END : 0);
            b3_compress_cv(cv, m, 0, len, flags);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) tree_leaves[leaf * 8 + i] = cv[i];
    }
}

// ---------------------------------------------------------------------------
// Parent levels.  One CTA takes 2^k consecutive nodes of level `in` and
// writes every node of the k levels above them (each level into its own slot
// of the flat tree), so a 2^20-leaf tree needs 3 launches instead of 20.
// kind: 0 = SHA-256, 1 = BLAKE3.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sha256_pair(const uint32_t l[8], const uint32_t r[8],
                                            uint32_t out[8]) {
    uint32_t st[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                      0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
    uint32_t w[16];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        w[i] = bswap32(l[i]);
        w[8 + i] = bswap32(r[i]);
    }
    sha256_compress(st, w);
#pragma unroll
    for (int i = 0; i < 16; ++i) w[i] = 0;
    w[0] = 0x80000000u;
    w[15] = 512;
    sha256_compress(st, w);
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = bswap32(st[i]);
}

__device__ __forceinline__ void hash_pair(int kind, const uint32_t l[8], const uint32_t r[8],
                                          uint32_t out[8]) {
    if (kind == 1) b3_parent(l, r, out);
    else sha256_pair(l, r, out);
}

// in: n_in nodes (32 B each); outputs levels written at out_levels[0..k-1]
// with level j holding n_in >> (j+1) nodes.  blockDim = 256, each CTA covers
// 512 input nodes (or fewer at the top).
struct LevelsArgs {
    const uint32_t *in;
    uint32_t *out[10];
    uint64_t n_in;
    int k;  // levels to produce (<= 9)
    int kind;
};

// Body: unit u (512 input nodes) with threads 0..255; any further threads of
// the CTA only take part in its barriers.  nodes holds 256 padded rows.
__device__ __forceinline__ void merkle_levels_body(const LevelsArgs &a, uint64_t u,
                                                   uint32_t (*nodes)[9]) {
    const uint64_t base_in = u * 512;
    const int t = threadIdx.x;
    const bool lane_ok = t < 256;
    // level 0 of this CTA: parents of input pairs
    uint64_t n_lvl = a.n_in >> 1;  // nodes at the first output level
    {
        const uint64_t j = (u * 256) + t;
        uint32_t o[8];
        if (lane_ok && j < n_lvl) {
            uint32_t l[8], r[8];
            const uint4 *pl = reinterpret_cast<const uint4 *>(a.in + (base_in + 2 * t) * 8);
            const uint4 l0 = pl[0], l1 = pl[1], r0 = pl[2], r1 = pl[3];
            l[0] = l0.x; l[1] = l0.y; l[2] = l0.z; l[3] = l0.w;
            l[4] = l1.x; l[5] = l1.y; l[6] = l1.z; l[7] = l1.w;
            r[0] = r0.x; r[1] = r0.y; r[2] = r0.z; r[3] = r0.w;
            r[4] = r1.x; r[5] = r1.y; r[6] = r1.z; r[7] = r1.w;
            hash_pair(a.kind, l, r, o);
            uint4 *po = reinterpret_cast<uint4 *>(a.out[0] + j * 8);
            po[0] = make_uint4(o[0], o[1], o[2], o[3]);
            po[1] = make_uint4(o[4], o[5], o[6], o[7]);
#pragma unroll
            for (int i = 0; i < 8; ++i) nodes[t][i] = o[i];
        }
    }
    __syncthreads();
    uint64_t cta_nodes = n_lvl < 256 ? n_lvl : 256;  // nodes of this CTA at the current level
    for (int lv = 1; lv < a.k; ++lv) {
        const uint64_t half = cta_nodes >> 1;
        const bool active = (uint64_t)t < half;
        uint32_t o[8];
        if (active) {
            hash_pair(a.kind, nodes[2 * t], nodes[2 * t + 1], o);
            const uint64_t j = u * (256 >> lv) + t;
            uint4 *po = reinterpret_cast<uint4 *>(a.out[lv] + j * 8);
            po[0] = make_uint4(o[0], o[1], o[2], o[3]);
            po[1] = make_uint4(o[4], o[5], o[6], o[7]);
        }
        __syncthreads();  // every read of this level precedes the overwrite
        if (active) {
#pragma unroll
            for (int i = 0; i < 8; ++i) nodes[t][i] = o[i];
        }
        __syncthreads();
        cta_nodes = half;
    }
}

// SHA-256 leaves: one thread per leaf, sequential over the row.
// Body: leaves first, first + step, .. below n_leaves.
__device__ __forceinline__ void sha_leaves_body(const uint4 *cw, int log_lanes, uint64_t n_leaves,
                                                uint32_t *tree_leaves, uint64_t first,
                                                uint64_t step) {
    for (uint64_t leaf = first; leaf < n_leaves; leaf += step) {
        const uint64_t elems = (uint64_t)1 << log_lanes;
        const uint64_t bytes = elems * 16;
        const uint4 *p = cw + leaf * elems;
        uint32_t st[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                          0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
        const uint64_t full = bytes / 64;  // full 64-byte blocks
        for (uint64_t blk = 0; blk < full; ++blk) {
            uint32_t w[16];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 v = p[blk * 4 + q];
                w[4 * q] = bswap32(v.x);
                w[4 * q + 1] = bswap32(v.y);
                w[4 * q + 2] = bswap32(v.z);
                w[4 * q + 3] = bswap32(v.w);
            }
            sha256_compress(st, w);
        }
        // tail: remaining (bytes % 64) bytes, then 0x80, zeros, 64-bit length
        const uint32_t rem = (uint32_t)(bytes - full * 64);  // 0, 16, 32 or 48
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = 0;
        for (uint32_t e = 0; e < rem / 16; ++e) {
            const uint4 v = p[full * 4 + e];
            w[4 * e] = bswap32(v.x);
            w[4 * e + 1] = bswap32(v.y);
            w[4 * e + 2] = bswap32(v.z);
            w[4 * e + 3] = bswap32(v.w);
        }
        w[rem / 4] = 0x80000000u;
        const uint64_t bitlen = bytes * 8;
        if (rem + 9 > 64) {
            sha256_compress(st, w);
#pragma unroll
            for (int i = 0; i < 16; ++i) w[i] = 0;
        }
        w[14] = (uint32_t)(bitlen >> 32);
        w[15] = (uint32_t)bitlen;
        sha256_compress(st, w);
#pragma unroll
        for (int i = 0; i < 8; ++i) tree_leaves[leaf * 8 + i] = bswap32(st[i]);
    }
}

}  // namespace bz
