// Merkle tree over codeword rows (flock-core/src/merkle.rs:558-596,
// commit.rs:283-297): leaf i = the 16 * 2^log_lanes bytes of position i,
// flat layout [leaves .., level k-1 .., root].
//
// BLAKE3 leaves are non-root chaining values with BLAKE3's own chunk tree
// (merkle.rs:160-201).  For a leaf of C = L/64 >= 1 full 1 KiB chunks (C a
// power of two), the leaf CV is a perfect binary tree of PARENT merges over
// the C chunk CVs (chunk counter = chunk index inside the leaf), and the
// Merkle tree above the leaves is the same PARENT merge, so one CTA hashes
// 256 chunks (one per thread) and folds them in shared memory straight into
// leaf CVs.  Leaves shorter than 1 KiB are one partial chunk (counter 0).
// SHA-256 leaves are sha256(row) (merkle.rs:213) and parents sha256(l || r).
#include <cuda_runtime.h>

#include <algorithm>

#include "bz_internal.h"
#include "hash.cuh"
#include "merkle_kernels.cuh"

namespace bz {

// ---- kernels around the bodies of merkle_kernels.cuh -----------------------
__global__ void __launch_bounds__(256) b3_leaves_chunked(const uint4 *cw, uint64_t n_chunks,
                                                         uint32_t *tree_leaves, int log_c,
                                                         uint64_t chunk0) {
    __shared__ uint32_t cvs[256][9];  // padded rows
    b3_leaves_chunked_body(cw, n_chunks, tree_leaves, log_c, chunk0,
                           (uint64_t)blockIdx.x * blockDim.x, cvs);
}

__global__ void b3_leaves_small(const uint4 *cw, int log_lanes, uint64_t n_leaves,
                                uint32_t *tree_leaves) {
    b3_leaves_small_body(cw, log_lanes, n_leaves, tree_leaves,
                         (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                         (uint64_t)gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(256) merkle_levels(LevelsArgs a) {
    __shared__ uint32_t nodes[256][9];
    merkle_levels_body(a, blockIdx.x, nodes);
}

__global__ void sha_leaves(const uint4 *cw, int log_lanes, uint64_t n_leaves,
                           uint32_t *tree_leaves) {
    sha_leaves_body(cw, log_lanes, n_leaves, tree_leaves,
                    (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (uint64_t)gridDim.x * blockDim.x);
}

// A small BLAKE3 tree of short leaves (at most one chunk, log_lanes < 6) in
// one CTA: thread i hashes leaf i, then the CTA builds every level up to the
// root in shared memory, writing leaves and levels to the flat tree as
// merkle_levels does.  256 leaves of 512 B take 18.9 us against 28.7 us for
// b3_leaves_small + merkle_levels.  Full 1 KiB chunks are left to the
// multi-CTA kernels: there one SM's issue rate bounds a single CTA (256
// leaves of 1 KiB: 32.4 against 30.7 us).
constexpr int kTreeSmallMax = 1024;  // leaves (threads)
__global__ void __launch_bounds__(kTreeSmallMax) b3_tree_small(const uint4 *cw, int log_lanes,
                                                               uint32_t n_leaves,
                                                               uint32_t *tree) {
    __shared__ uint32_t nodes[kTreeSmallMax][9];  // padded rows
    const uint32_t t = threadIdx.x;
    uint32_t cv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) cv[i] = kIV[i];
    const uint32_t elems = 1u << log_lanes, bytes = elems * 16, nblk = (bytes + 63) / 64;
    const uint4 *p = cw + (uint64_t)t * elems;
#pragma unroll 1
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
    for (int i = 0; i < 8; ++i) {
        nodes[t][i] = cv[i];
        tree[(uint64_t)t * 8 + i] = cv[i];
    }
    __syncthreads();
    uint64_t off = n_leaves;
    for (uint32_t n = n_leaves; n > 1; n >>= 1) {
        const uint32_t half = n >> 1;
        uint32_t o[8];
        if (t < half) {
            b3_parent(nodes[2 * t], nodes[2 * t + 1], o);
#pragma unroll
            for (int i = 0; i < 8; ++i) tree[(off + t) * 8 + i] = o[i];
        }
        __syncthreads();  // every read of this level precedes the overwrite
        if (t < half) {
#pragma unroll
            for (int i = 0; i < 8; ++i) nodes[t][i] = o[i];
        }
        __syncthreads();
        off += half;
    }
}

// Generic BLAKE3 chunk CVs into scratch (leaves longer than 256 chunks).
__global__ void b3_chunk_cvs(const uint4 *cw, uint64_t n_chunks, int log_c, uint32_t *out,
                             uint64_t chunk0) {
    const uint64_t chunk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (chunk >= n_chunks) return;
    const uint64_t c_in_leaf = chunk0 + (chunk & ((1ull << log_c) - 1));
    uint32_t cv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) cv[i] = kIV[i];
    const uint4 *p = cw + chunk * 64;
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
#pragma unroll
    for (int i = 0; i < 8; ++i) out[chunk * 8 + i] = cv[i];
}

size_t merkle_scratch_bytes(const Shape &s) {
    if (s.hash_kind == 1 && s.log_lanes > 14) {
        const size_t chunks = s.cw_words() / 64;
        return chunks * 32 * 2;
    }
    return 0;
}

// Build all parent levels above `n_leaves` leaves stored at tree[0..).
static int launch_levels(uint32_t *tree, uint64_t n_leaves, int kind, cudaStream_t st,
                         LaunchLog *log);

// CTA size of b3_leaves_chunked: 256 threads, halved (down to 32 and to the
// chunks per leaf) while that leaves fewer than two CTAs per SM.
static unsigned leaf_threads(uint64_t n_chunks, int log_c, int num_sms) {
    unsigned t = 256;
    const unsigned floor = std::max(32u, 1u << log_c);
    while (t > floor && n_chunks / t < 2 * (uint64_t)num_sms) t >>= 1;
    return t;
}

bool leaves_range_supported(const Shape &s) { return !(s.hash_kind == 1 && s.log_lanes > 14); }

int launch_leaves_range(const Shape &s, const uint4 *d_cw, uint8_t *d_tree, uint64_t p0,
                        uint64_t p1, cudaStream_t st, int num_sms) {
    uint32_t *tree = reinterpret_cast<uint32_t *>(d_tree);
    const uint64_t n = p1 - p0;
    const uint4 *cw = d_cw + (p0 << s.log_lanes);
    uint32_t *leaves = tree + p0 * 8;
    if (s.hash_kind == 1) {
        if (s.log_lanes < 6) {
            b3_leaves_small<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cw, s.log_lanes, n,
                                                                      leaves);
        } else {
            const int log_c = s.log_lanes - 6;
            const uint64_t n_chunks = n << log_c;
            const unsigned t = leaf_threads(n_chunks, log_c, num_sms);
            b3_leaves_chunked<<<(unsigned)((n_chunks + t - 1) / t), t, 0, st>>>(
                cw, n_chunks, leaves, log_c, s.chunk0);
        }
    } else {
        sha_leaves<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(cw, s.log_lanes, n, leaves);
    }
    return 1;
}

int launch_merkle_levels(const Shape &s, uint8_t *d_tree, cudaStream_t st, LaunchLog *log) {
    return launch_levels(reinterpret_cast<uint32_t *>(d_tree), s.n_leaves(), s.hash_kind, st,
                         log);
}

static int launch_levels(uint32_t *tree, uint64_t n_leaves, int kind, cudaStream_t st,
                         LaunchLog *log) {
    int launches = 0;
    uint64_t in_off = 0, n_in = n_leaves;
    while (n_in > 1) {
        int k = 0;
        uint64_t n = n_in;
        while (n > 1 && k < 9) {
            n >>= 1;
            ++k;
        }
        LevelsArgs a;
        a.in = tree + in_off * 8;
        a.n_in = n_in;
        a.k = k;
        a.kind = kind;
        uint64_t off = in_off + n_in, cnt = n_in >> 1;
        for (int j = 0; j < k; ++j) {
            a.out[j] = tree + off * 8;
            off += cnt;
            cnt >>= 1;
        }
        const uint64_t ctas = (n_in + 511) / 512;
        merkle_levels<<<(unsigned)ctas, 256, 0, st>>>(a);
        if (log) log->mark("merkle_levels");
        ++launches;
        // advance: the last produced level becomes the next input
        uint64_t o = in_off + n_in, c = n_in >> 1;
        for (int j = 0; j < k - 1; ++j) {
            o += c;
            c >>= 1;
        }
        in_off = o;
        n_in = c;
    }
    return launches;
}

int launch_merkle(const Shape &s, const uint4 *d_cw, uint8_t *d_tree, uint8_t *d_scratch,
                  cudaStream_t st, int num_sms, LaunchLog *log) {
    auto mark = [&](const char *n) {
        if (log) log->mark(n);
    };
    const uint64_t n_leaves = s.n_leaves();
    uint32_t *tree = reinterpret_cast<uint32_t *>(d_tree);
    int launches = 0;
    if (s.hash_kind == 1) {
        if (s.log_lanes < 6 && n_leaves <= (uint64_t)kTreeSmallMax && n_leaves >= 2) {
            b3_tree_small<<<1, (unsigned)n_leaves, 0, st>>>(d_cw, s.log_lanes,
                                                            (uint32_t)n_leaves, tree);
            mark("b3_tree_small");
            return 1;
        }
        if (s.log_lanes < 6) {
            b3_leaves_small<<<(unsigned)((n_leaves + 255) / 256), 256, 0, st>>>(d_cw, s.log_lanes,
                                                                             n_leaves, tree);
            mark("b3_leaves_small");
            ++launches;
        } else if (s.log_lanes <= 14) {
            const int log_c = s.log_lanes - 6;
            const uint64_t n_chunks = n_leaves << log_c;
            const unsigned t = leaf_threads(n_chunks, log_c, num_sms);
            b3_leaves_chunked<<<(unsigned)((n_chunks + t - 1) / t), t, 0, st>>>(
                d_cw, n_chunks, tree, log_c, s.chunk0);
            mark("b3_leaves_chunked");
            ++launches;
        } else {
            const int log_c = s.log_lanes - 6;
            const uint64_t n_chunks = n_leaves << log_c;
            uint32_t *cvs = reinterpret_cast<uint32_t *>(d_scratch);
            b3_chunk_cvs<<<(unsigned)((n_chunks + 255) / 256), 256, 0, st>>>(d_cw, n_chunks,
                                                                           log_c, cvs, s.chunk0);
            mark("b3_chunk_cvs");
            ++launches;
            // reduce chunk CVs to leaf CVs: levels inside the scratch area,
            // the last one written straight into the tree leaves.
            uint32_t *bufs[2] = {cvs, cvs + n_chunks * 8};
            uint64_t n = n_chunks;
            int cur = 0;
            for (int lv = 0; lv < log_c; ++lv) {
                LevelsArgs a;
                a.in = bufs[cur];
                a.n_in = n;
                a.k = 1;
                a.kind = 1;
                a.out[0] = (lv == log_c - 1) ? tree : bufs[cur ^ 1];
                merkle_levels<<<(unsigned)((n + 511) / 512), 256, 0, st>>>(a);
                mark("merkle_levels");
                ++launches;
                n >>= 1;
                cur ^= 1;
            }
        }
    } else {
        sha_leaves<<<(unsigned)((n_leaves + 127) / 128), 128, 0, st>>>(d_cw, s.log_lanes,
                                                                       n_leaves, tree);
        mark("sha_leaves");
        ++launches;
    }
    launches += launch_levels(tree, n_leaves, s.hash_kind, st, log);
    return launches;
}

// ---------------------------------------------------------------------------
// Leaves of a lane-sharded BLAKE3 commit: one thread per position merges the
// world ranks' subtree CVs left to right with BLAKE3's CV stack (a subtree of
// 2^j ranks is merged with its left neighbour of the same size), which for a
// power-of-two world is the perfect binary tree of PARENT merges the leaf's
// own chunk tree has above those subtrees (merkle.rs:160-201).
// ---------------------------------------------------------------------------
constexpr int kMaxShardLevels = 11;  // world <= 1024
__global__ void b3_combine_shard_cvs(const uint32_t *cvs, uint32_t world, uint64_t n_leaves,
                                     uint32_t *leaves) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_leaves) return;
    uint32_t stack[kMaxShardLevels][8];
    int depth = 0;
    for (uint32_t r = 0; r < world; ++r) {
        uint32_t cv[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) cv[i] = cvs[((uint64_t)r * n_leaves + p) * 8 + i];
        // merge while the subtree just completed has a left sibling of equal
        // size: the number of trailing one bits of r
        for (uint32_t m = r; m & 1; m >>= 1) {
            uint32_t o[8];
            b3_parent(stack[--depth], cv, o);
#pragma unroll
            for (int i = 0; i < 8; ++i) cv[i] = o[i];
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) stack[depth][i] = cv[i];
        ++depth;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) leaves[p * 8 + i] = stack[0][i];
}

int launch_combine_shard_cvs(const uint8_t *d_cvs, uint32_t world, uint64_t n_leaves,
                             uint8_t *d_tree, cudaStream_t st) {
    if (world == 0 || (world & (world - 1)) || world > (1u << (kMaxShardLevels - 1))) return 0;
    b3_combine_shard_cvs<<<(unsigned)((n_leaves + 127) / 128), 128, 0, st>>>(
        reinterpret_cast<const uint32_t *>(d_cvs), world, n_leaves,
        reinterpret_cast<uint32_t *>(d_tree));
    return 1;
}

// ---------------------------------------------------------------------------
// Gathers for openings.
// ---------------------------------------------------------------------------
__global__ void gather_rows(const uint4 *cw, int log_lanes, const uint64_t *pos, size_t q,
                            uint4 *out) {
    const uint64_t L = (uint64_t)1 << log_lanes;
    const uint64_t total = q * L;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i >> log_lanes, ln = i & (L - 1);
        out[i] = cw[(pos[r] << log_lanes) | ln];
    }
}

__global__ void gather_nodes(const uint4 *tree, const uint64_t *idx, size_t n, uint4 *out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * n) return;
    out[i] = tree[idx[i >> 1] * 2 + (i & 1)];
}

int launch_gather_rows(const uint4 *d_cw, int log_lanes, const uint64_t *d_pos, size_t q,
                       uint4 *d_out, cudaStream_t st) {
    if (q == 0) return 0;
    const uint64_t total = (uint64_t)q << log_lanes;
    const unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, 4096);
    gather_rows<<<grid, 256, 0, st>>>(d_cw, log_lanes, d_pos, q, d_out);
    return 1;
}

int launch_gather_nodes(const uint8_t *d_tree, const uint64_t *d_idx, size_t n, uint8_t *d_out,
                        cudaStream_t st) {
    if (n == 0) return 0;
    gather_nodes<<<(unsigned)((2 * n + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const uint4 *>(d_tree), d_idx, n, reinterpret_cast<uint4 *>(d_out));
    return 1;
}

}  // namespace bz
