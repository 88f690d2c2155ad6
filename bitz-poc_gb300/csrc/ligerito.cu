// Device kernels of the recursive Ligerito prover beyond the lane folds
// (flock-core/src/pcs/ligerito.rs):
//
//  * induce: the basis polynomial a level's queries induce, through the
//    transposed forward NTT of the query weights scattered over the codeword
//    domain, keeping the low 2^log_msg_cols outputs
//    (induce_sumcheck_poly_via_ntt, :2124-2184; transpose_forward_ntt,
//    :2079-2122).
//  * glue: combined_basis[j] += beta * b_new[j] (SumcheckProver::glue,
//    :3125-3145).
//  * dot: sum_j f[j] * b[j], the claimed value of an out-of-domain
//    introduce (round_msg_and_eval_lsb, :2550-2587).
//  * the BitZ round-0 out-of-domain sample over the packed message: its
//    value MLE[P](point) and the eta * eq(point) term added to the opening
//    basis, both with eq(point) split into a 2^12-entry low table and a high
//    table (src/ligerito_flock.rs:1456-1486, 1590-1650).
//
// These arrays are the folded witness (2^(n - initial_k) elements and less),
// so the kernels are simple one-pass forms; sums are XORs of reduced
// products (field addition is order independent, so the result is
// bit-identical to the reference's sums).
#include <cuda_runtime.h>

#include "bz_internal.h"
#include "gf128.cuh"

namespace bz {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint4 warp_xor_u4(uint4 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x ^= __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y ^= __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z ^= __shfl_xor_sync(0xffffffffu, v.z, o);
        v.w ^= __shfl_xor_sync(0xffffffffu, v.w, o);
    }
    return v;
}

// XOR of v over the CTA (blockDim.x a multiple of 32, <= 1024); valid in
// thread 0.
__device__ uint4 cta_xor_u4(uint4 v) {
    __shared__ uint4 red[32];
    v = warp_xor_u4(v);
    const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
    if (ln == 0) red[w] = v;
    __syncthreads();
    uint4 acc = make_uint4(0, 0, 0, 0);
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) acc = gf_add(acc, red[k]);
    return acc;
}

__global__ void scatter_kernel(uint4 *data, const uint64_t *pos, const uint4 *w, int nq) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nq) data[pos[i]] = w[i];
}

// One layer of the transposed forward NTT over 2^log_d elements: blocks of
// 2^(log_d - layer) positions with twiddle t = twiddle(layer, block); each
// pair (a, b) = (top, bottom half) becomes (a + b, t * (a + b) + b).
__global__ void tntt_layer_kernel(uint4 *data, int log_d, int layer, const uint4 *tw) {
    const uint64_t pairs = (uint64_t)1 << (log_d - 1);
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pairs) return;
    const int half_log = log_d - layer - 1;
    const uint64_t block = p >> half_log;
    const uint64_t within = p & (((uint64_t)1 << half_log) - 1);
    const uint64_t ia = (block << (half_log + 1)) + within;
    const uint64_t ib = ia + ((uint64_t)1 << half_log);
    const uint4 t = tw[((uint64_t)1 << layer) + block];
    const uint4 a = data[ia], b = data[ib];
    const uint4 s = gf_add(a, b);
    data[ia] = s;
    data[ib] = gf_add(gf_mul(t, s), b);
}

// The deepest kTileLog layers of the transposed forward NTT (pair spans 1,
// 2, .., 2^(kTileLog-1)) stay inside aligned tiles of 2^kTileLog positions:
// one CTA loads its tile into shared memory, runs those layers from the
// deepest up with a barrier between layers, and stores it back.  Same
// butterfly and twiddles as tntt_layer_kernel.
constexpr int kTileLog = 9;
__global__ void __launch_bounds__(kThreads) tntt_tile_kernel(uint4 *data, int log_d,
                                                             const uint4 *tw) {
    __shared__ uint4 tile[1 << kTileLog];
    const uint64_t base = (uint64_t)blockIdx.x << kTileLog;
    for (int i = threadIdx.x; i < (1 << kTileLog); i += blockDim.x) tile[i] = data[base + i];
    __syncthreads();
    for (int half_log = 0; half_log < kTileLog; ++half_log) {
        const int layer = log_d - half_log - 1;
        for (int p = threadIdx.x; p < (1 << (kTileLog - 1)); p += blockDim.x) {
            const int within = p & ((1 << half_log) - 1);
            const int ia = ((p >> half_log) << (half_log + 1)) + within;
            const int ib = ia + (1 << half_log);
            const uint64_t block = (base + (uint64_t)ia) >> (half_log + 1);
            const uint4 t = tw[((uint64_t)1 << layer) + block];
            const uint4 a = tile[ia], b = tile[ib];
            const uint4 s = gf_add(a, b);
            tile[ia] = s;
            tile[ib] = gf_add(gf_mul(t, s), b);
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < (1 << kTileLog); i += blockDim.x) data[base + i] = tile[i];
}

// out[0] = XOR of in[0..n) (one CTA)
__global__ void __launch_bounds__(kThreads) xor_reduce_kernel(const uint4 *in, uint64_t n,
                                                              uint4 *out) {
    uint4 acc = make_uint4(0, 0, 0, 0);
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) acc = gf_add(acc, in[i]);
    acc = cta_xor_u4(acc);
    if (threadIdx.x == 0) out[0] = acc;
}

__global__ void glue_kernel(uint4 *b, const uint4 *nb, uint64_t n, uint4 beta) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = gf_add(b[i], gf_mul(beta, nb[i]));
}

// per-CTA partials of sum_j f[j] * b[j]
__global__ void __launch_bounds__(kThreads) dot_kernel(const uint4 *f, const uint4 *b, uint64_t n,
                                                       uint4 *partial) {
    uint4 acc = make_uint4(0, 0, 0, 0);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        acc = gf_add(acc, gf_mul(f[i], b[i]));
    acc = cta_xor_u4(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// The out-of-domain MLE split at 2^lo-element blocks (ood_eval,
// src/ligerito_flock.rs:1456-1486): CTA h computes
// head[h] * sum_j p[h * 2^lo + j] * tail[j] for its blocks h = blockIdx.x +
// k * gridDim.x and writes one partial.
__global__ void __launch_bounds__(kThreads) split_dot_kernel(const uint4 *p, const uint4 *tail,
                                                             int lo, const uint4 *head,
                                                             uint64_t n_blocks, uint4 *partial) {
    const uint64_t bl = (uint64_t)1 << lo;
    uint4 acc = make_uint4(0, 0, 0, 0);
    for (uint64_t h = blockIdx.x; h < n_blocks; h += gridDim.x) {
        uint4 inner = make_uint4(0, 0, 0, 0);
        for (uint64_t j = threadIdx.x; j < bl; j += blockDim.x)
            inner = gf_add(inner, gf_mul(p[h * bl + j], tail[j]));
        acc = gf_add(acc, gf_mul(inner, head[h]));
    }
    acc = cta_xor_u4(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// b[i] += (eta * head[i >> lo]) * tail[i & (2^lo - 1)]  (add_ood_basis,
// src/ligerito_flock.rs:1590-1650: eta * eq(point) added to the basis).  When
// a CTA's elements share one head entry (2^lo >= the CTA size), its thread 0
// forms eta * head once for all of them.
constexpr int kLogThreads = 8;
static_assert((1 << kLogThreads) == kThreads, "eq_axpy assumes 256-thread CTAs");
__global__ void __launch_bounds__(kThreads) eq_axpy_kernel(uint4 *b, const uint4 *tail, int lo,
                                                           const uint4 *head, uint4 eta,
                                                           uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint4 s;
    if (lo >= kLogThreads) {
        __shared__ uint4 s_cta;
        if (threadIdx.x == 0)
            s_cta = gf_mul(eta, head[((uint64_t)blockIdx.x * blockDim.x) >> lo]);
        __syncthreads();
        s = s_cta;
    } else {
        if (i >= n) return;
        s = gf_mul(eta, head[i >> lo]);
    }
    if (i >= n) return;
    b[i] = gf_add(b[i], gf_mul(s, tail[i & (((uint64_t)1 << lo) - 1)]));
}

unsigned grid_for(uint64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

size_t split_dot_partials(size_t n_blocks, int num_sms) {
    const size_t cap = (size_t)num_sms * 4;
    return n_blocks < cap ? (n_blocks ? n_blocks : 1) : cap;
}

int launch_split_dot(const uint4 *d_p, const uint4 *d_tail, int lo, const uint4 *d_head,
                     size_t n_blocks, uint4 *d_partial, uint4 *d_out, cudaStream_t st,
                     int num_sms) {
    const size_t ctas = split_dot_partials(n_blocks, num_sms);
    split_dot_kernel<<<(unsigned)ctas, kThreads, 0, st>>>(d_p, d_tail, lo, d_head, n_blocks,
                                                          d_partial);
    xor_reduce_kernel<<<1, kThreads, 0, st>>>(d_partial, ctas, d_out);
    return 2;
}

int launch_eq_axpy(uint4 *d_b, const uint4 *d_tail, int lo, const uint4 *d_head, uint4 eta,
                   size_t n, cudaStream_t st) {
    eq_axpy_kernel<<<grid_for(n), kThreads, 0, st>>>(d_b, d_tail, lo, d_head, eta, n);
    return 1;
}

int launch_induce_basis(uint4 *d_domain, int log_d, const uint64_t *d_pos, const uint4 *d_w,
                        int nq, const uint4 *d_tw, cudaStream_t st) {
    int launches = 0;
    cudaMemsetAsync(d_domain, 0, ((size_t)16) << log_d, st);
    if (nq) {
        scatter_kernel<<<grid_for(nq), kThreads, 0, st>>>(d_domain, d_pos, d_w, nq);
        ++launches;
    }
    int layer = log_d - 1;
    if (log_d >= kTileLog) {
        tntt_tile_kernel<<<(unsigned)((uint64_t)1 << (log_d - kTileLog)), kThreads, 0, st>>>(
            d_domain, log_d, d_tw);
        ++launches;
        layer = log_d - kTileLog - 1;
    }
    for (; layer >= 0; --layer) {
        tntt_layer_kernel<<<grid_for((uint64_t)1 << (log_d - 1)), kThreads, 0, st>>>(
            d_domain, log_d, layer, d_tw);
        ++launches;
    }
    return launches;
}

int launch_glue(uint4 *d_b, const uint4 *d_nb, size_t n, uint4 beta, cudaStream_t st) {
    glue_kernel<<<grid_for(n), kThreads, 0, st>>>(d_b, d_nb, n, beta);
    return 1;
}

size_t dot_partials_count(size_t n, int num_sms) {
    const size_t want = (n + kThreads - 1) / kThreads;
    const size_t cap = (size_t)num_sms * 4;
    return want < cap ? (want ? want : 1) : cap;
}

int launch_dot(const uint4 *d_f, const uint4 *d_b, size_t n, uint4 *d_partial, uint4 *d_out,
               cudaStream_t st, int num_sms) {
    const size_t ctas = dot_partials_count(n, num_sms);
    dot_kernel<<<(unsigned)ctas, kThreads, 0, st>>>(d_f, d_b, n, d_partial);
    xor_reduce_kernel<<<1, kThreads, 0, st>>>(d_partial, ctas, d_out);
    return 2;
}

}  // namespace bz
