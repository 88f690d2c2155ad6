// Opening-time kernels: sumcheck lane folds and messages
// (flock-core/src/pcs/ligerito.rs), the ring-switch passes (BitZ
// src/ligerito.rs), the eq table (src/poly/utils.rs) and the ChaCha20 input
// generator.
//
// Field sums are exact and order independent, so partial sums per CTA are
// XOR-reduced as unreduced 256-bit values and reduced once at the end, which
// is bit-identical to the reference's per-term sums (ligerito.rs:2646-2649).
#include <cuda_runtime.h>

#include <algorithm>

#include "bz_internal.h"
#include "gf128.cuh"
#include "t16.cuh"

namespace bz {

__device__ __forceinline__ void warp_xor_wide(gf_wide &a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) a.w[i] ^= __shfl_xor_sync(0xffffffffu, a.w[i], o);
    }
}

// Reduce two wide accumulators over the CTA and store 8 words at out.
__device__ void cta_store_pair(gf_wide u0, gf_wide u2, uint64_t *out) {
    __shared__ uint64_t red[32][8];
    warp_xor_wide(u0);
    warp_xor_wide(u2);
    const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
    if (ln == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            red[w][i] = u0.w[i];
            red[w][4 + i] = u2.w[i];
        }
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        uint64_t acc = 0;
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < nw; ++k) acc ^= red[k][threadIdx.x];
        out[threadIdx.x] = acc;
    }
}

// Dynamic shared memory of the kernels that multiply by one challenge r
// through byte tables: the 64 KB table of r and its 128 basis products
// (padded to kT16Bases).
constexpr size_t kRTableSmem = (size_t)kT16Entries * 16 + kT16Bases * 16;

// Build the byte tables of r in shared memory (all threads; syncs inside).
__device__ __forceinline__ const char *build_r_table(uint4 *smem, uint4 r) {
    __shared__ uint4 rs[1];
    if (threadIdx.x == 0) rs[0] = r;
    __syncthreads();
    t16_build(smem, smem + kT16Entries, rs, 1);
    return reinterpret_cast<const char *>(smem);
}

// XOR of the per-CTA partials (8 words each) of n CTAs and the single
// reduction: out = {u0, u2}.  256 threads: thread t XORs word t mod 8 of
// partials t / 8, t / 8 + 32, ...; lanes holding the same word then combine
// by shuffles and across warps.  Partials are read from L2 (other CTAs wrote
// them in this launch or the previous one).
constexpr int kFinishThreads = 256;

// out = {u0, u2}: the two unreduced sums acc[0..3], acc[4..7], reduced.
__device__ __forceinline__ void store_msg(const uint64_t *acc, uint64_t *out) {
    gf_wide w0, w2;
    for (int i = 0; i < 4; ++i) {
        w0.w[i] = acc[i];
        w2.w[i] = acc[4 + i];
    }
    const uint4 u0 = gf_reduce(w0), u2 = gf_reduce(w2);
    out[0] = lo64(u0);
    out[1] = hi64(u0);
    out[2] = lo64(u2);
    out[3] = hi64(u2);
}

__device__ __forceinline__ void st_release_sys(uint32_t *p, uint32_t v) {
    asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ void finish_msg_body(const uint64_t *partials, int n, uint64_t *out) {
    __shared__ uint64_t red[kFinishThreads / 32][8];
    __shared__ uint64_t acc[8];
    const int w = threadIdx.x & 7;
    uint64_t a = 0;
    for (int i = threadIdx.x >> 3; i < n; i += kFinishThreads / 8)
        a ^= __ldcg(partials + (uint64_t)i * 8 + w);
    a ^= __shfl_xor_sync(0xffffffffu, a, 8);
    a ^= __shfl_xor_sync(0xffffffffu, a, 16);
    if ((threadIdx.x & 31) < 8) red[threadIdx.x >> 5][w] = a;
    __syncthreads();
    if (threadIdx.x < 8) {
        uint64_t x = 0;
        for (int k = 0; k < kFinishThreads / 32; ++k) x ^= red[k][threadIdx.x];
        acc[threadIdx.x] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) store_msg(acc, out);
}

// The last CTA of a launch (the one whose ticket completes the count)
// reduces every CTA's partials and posts {u0, u2} to a mailbox in mapped host
// memory: the four words, then (a system-scope release store by the same
// thread) the sequence number the host waits for.  It resets the ticket for
// the next launch.  Without a mailbox (ticket null) the caller launches
// finish_msg_kernel.
struct MsgMailbox {
    unsigned int *ticket = nullptr;  // device counter, 0 between launches
    uint64_t *words = nullptr;       // mapped host memory: u0, u2
    uint32_t *seq = nullptr;         // mapped host memory
    uint32_t seq_val = 0;
};

__device__ void msg_epilogue(const uint64_t *partials, const MsgMailbox &mb) {
    if (!mb.ticket) return;
    __shared__ int last;
    __threadfence();  // this CTA's partial (written before the barrier below)
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(mb.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    finish_msg_body(partials, (int)gridDim.x, mb.words);
    if (threadIdx.x == 0) {
        st_release_sys(mb.seq, mb.seq_val);
        *mb.ticket = 0;
    }
}

// A single-CTA launch with a mailbox reduces its terms in shared memory and
// posts them itself (no partials, no ticket); otherwise every CTA stores its
// partial and the last one posts.
__device__ __forceinline__ void msg_finish(gf_wide u0, gf_wide u2, uint64_t *partials,
                                           const MsgMailbox &mb) {
    if (mb.ticket && gridDim.x == 1) {
        __shared__ uint64_t acc[8];
        cta_store_pair(u0, u2, acc);
        __syncthreads();
        if (threadIdx.x == 0) {
            store_msg(acc, mb.words);
            st_release_sys(mb.seq, mb.seq_val);
        }
        return;
    }
    cta_store_pair(u0, u2, partials + (uint64_t)blockIdx.x * 8);
    msg_epilogue(partials, mb);
}

// Out of line for the fold kernel: its loop runs at the 128-register cap, and
// an inlined epilogue adds spills to it.
__device__ __noinline__ void msg_finish_call(gf_wide u0, gf_wide u2, uint64_t *partials,
                                             const MsgMailbox &mb) {
    msg_finish(u0, u2, partials, mb);
}

__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Thread 0 of each CTA polls the gate word, sleeping between polls, until it
// reads the round's sequence number (open: r is read behind it), the number
// with bit 31 set (cancelled) or the time limit passes (bit 0 of *err is
// set).  Returns whether the gate opened; r is then the posted challenge.
__device__ bool gate_wait(const RGate &g, uint4 &r) {
    __shared__ uint4 rs;
    __shared__ int open;
    if (threadIdx.x == 0) {
        const uint64_t t0 = globaltimer_ns();
        int st = 0;
        for (;;) {
            const uint32_t v = ld_acquire_sys(g.go);
            if (v == g.seq) {
                st = 1;
                break;
            }
            if (v == (g.seq | kGateCancel)) break;
            if (globaltimer_ns() - t0 > g.limit_ns) {
                atomicOr(g.err, 1u);
                break;
            }
            __nanosleep(128);
        }
        if (st) {
            const volatile uint64_t *rp = g.r;
            const uint64_t lo = rp[0], hi = rp[1];
            rs = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi,
                            (uint32_t)(hi >> 32));
        }
        open = st;
    }
    __syncthreads();
    r = rs;
    return open != 0;
}

// nf[j] = f[2j] + (f[2j] + f[2j+1]) * r (same for b); thread k produces the
// folded pair (2k, 2k+1) and its message terms.  The four multiplies by the
// challenge r use r's byte tables; the two variable products of the message
// use the generic carry-less multiply.  Registers are capped at 128 so two
// CTAs share an SM (a few spilled words cost less than half the warps: the
// 2^24 first fold takes 0.30 ms instead of 0.35 ms).
// GATED: launched before r is known; r comes through the gate instead (a
// cancelled or timed-out CTA returns before touching the arrays or the
// mailbox ticket).
template <bool GATED>
__global__ void __launch_bounds__(256, 2) fold_and_msg_kernel(const uint4 *f, const uint4 *b,
                                                           uint64_t half, uint4 r, uint4 *nf,
                                                           uint4 *nb, uint64_t *partials,
                                                           MsgMailbox mb, RGate gate) {
    extern __shared__ uint4 smem[];
    if constexpr (GATED) {
        if (!gate_wait(gate, r)) return;
    }
    const char *T = build_r_table(smem, r);
    T16Lane8 lc;
    lc.init();
    gf_wide u0 = gf_wide_zero(), u2 = gf_wide_zero();
    const uint64_t pairs = half >> 1;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < pairs;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 *fp = f + 4 * k, *bp = b + 4 * k;
        const uint4 f0 = fp[0], f1 = fp[1], f2 = fp[2], f3 = fp[3];
        const uint4 b0 = bp[0], b1 = bp[1], b2 = bp[2], b3 = bp[3];
        const uint4 x0 = gf_add(f0, lc.mul(T, gf_add(f0, f1)));
        const uint4 x1 = gf_add(f2, lc.mul(T, gf_add(f2, f3)));
        const uint4 y0 = gf_add(b0, lc.mul(T, gf_add(b0, b1)));
        const uint4 y1 = gf_add(b2, lc.mul(T, gf_add(b2, b3)));
        nf[2 * k] = x0;
        nf[2 * k + 1] = x1;
        nb[2 * k] = y0;
        nb[2 * k + 1] = y1;
        gf_wide_xor(u0, gf_mul_wide(x0, y0));
        gf_wide_xor(u2, gf_mul_wide(gf_add(x0, x1), gf_add(y0, y1)));
    }
    if (half == 1 && blockIdx.x == 0 && threadIdx.x == 0) {
        nf[0] = gf_add(f[0], gf_mul(gf_add(f[0], f[1]), r));
        nb[0] = gf_add(b[0], gf_mul(gf_add(b[0], b[1]), r));
    }
    msg_finish_call(u0, u2, partials, mb);
}

__global__ void __launch_bounds__(256) round_msg_kernel(const uint4 *f, const uint4 *b,
                                                        uint64_t pairs, uint64_t *partials,
                                                        MsgMailbox mb) {
    gf_wide u0 = gf_wide_zero(), u2 = gf_wide_zero();
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < pairs;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 f0 = f[2 * j], f1 = f[2 * j + 1], b0 = b[2 * j], b1 = b[2 * j + 1];
        gf_wide_xor(u0, gf_mul_wide(f0, b0));
        gf_wide_xor(u2, gf_mul_wide(gf_add(f0, f1), gf_add(b0, b1)));
    }
    msg_finish(u0, u2, partials, mb);
}

// Final XOR of per-CTA partials and the single reduction: out = {u0, u2}.
__global__ void __launch_bounds__(kFinishThreads) finish_msg_kernel(const uint64_t *partials,
                                                                    int n, uint64_t *out) {
    finish_msg_body(partials, n, out);
}

static int msg_grid(uint64_t work, int num_sms) {
    const uint64_t g = (work + 255) / 256;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)num_sms * 4));
}

size_t fold_partials_bytes(size_t n) {
    (void)n;
    return (size_t)1024 * 8 * sizeof(uint64_t);  // up to 1024 CTAs
}

int fold_grid(size_t n, int num_sms) { return std::min(msg_grid(n / 4, num_sms), 1024); }

int launch_fold_and_msg(const uint4 *d_f, const uint4 *d_b, size_t n, uint4 r, uint4 *d_nf,
                        uint4 *d_nb, uint64_t *d_partials, uint64_t *d_msg_out, cudaStream_t st,
                        int num_sms, const MsgPost *post, const RGate *gate) {
    const uint64_t half = n / 2;
    const int grid = fold_grid(n, num_sms);
    MsgMailbox mb;
    if (post) mb = {post->ticket, post->words, post->seq, post->seq_val};
    if (gate)
        fold_and_msg_kernel<true><<<grid, 256, kRTableSmem, st>>>(d_f, d_b, half, r, d_nf, d_nb,
                                                                  d_partials, mb, *gate);
    else
        fold_and_msg_kernel<false><<<grid, 256, kRTableSmem, st>>>(d_f, d_b, half, r, d_nf, d_nb,
                                                                   d_partials, mb, RGate{});
    if (post) return 1;
    finish_msg_kernel<<<1, kFinishThreads, 0, st>>>(d_partials, grid, d_msg_out);
    return 2;
}

int launch_round_msg(const uint4 *d_f, const uint4 *d_b, size_t n, uint64_t *d_partials,
                     uint64_t *d_msg_out, cudaStream_t st, int num_sms, const MsgPost *post) {
    const uint64_t pairs = n / 2;
    const int grid = std::min(msg_grid(pairs, num_sms), 1024);
    MsgMailbox mb;
    if (post) mb = {post->ticket, post->words, post->seq, post->seq_val};
    round_msg_kernel<<<grid, 256, 0, st>>>(d_f, d_b, pairs, d_partials, mb);
    if (post) return 1;
    finish_msg_kernel<<<1, kFinishThreads, 0, st>>>(d_partials, grid, d_msg_out);
    return 2;
}

// One partial_eval_lsb round: out[i] = in[2i] + (in[2i] + in[2i+1]) * r
// (= in[2i]*(1+r) + in[2i+1]*r exactly, ligerito.rs:1686-1691).
__global__ void __launch_bounds__(256) partial_eval_round_kernel(const uint4 *in, uint64_t half,
                                                                 uint4 r, uint4 *out) {
    extern __shared__ uint4 smem[];
    const char *T = build_r_table(smem, r);
    T16Lane8 lc;
    lc.init();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < half;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 v0 = in[2 * i], v1 = in[2 * i + 1];
        out[i] = gf_add(v0, lc.mul(T, gf_add(v0, v1)));
    }
}

int launch_partial_eval_round(const uint4 *d_in, size_t n, uint4 r, uint4 *d_out,
                              cudaStream_t st) {
    const uint64_t half = n / 2;
    const unsigned grid = (unsigned)std::min<uint64_t>((half + 255) / 256, 152 * 3);
    partial_eval_round_kernel<<<std::max(grid, 1u), 256, kRTableSmem, st>>>(d_in, half, r, d_out);
    return 1;
}

// eq table rounds: entries [0, half) double into [0, 2 half).
__global__ void eq_round_kernel(uint4 *eq, uint64_t half, const uint4 *point, int i) {
    const uint4 r = point[i];
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < half;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 p = eq[j];
        const uint4 one = gf_mul(p, r);
        eq[half + j] = one;
        eq[j] = gf_add(p, one);
    }
}

// The first k rounds in one CTA (global writes of a round are visible to the
// CTA's threads after the barrier).
__global__ void __launch_bounds__(512) eq_small_kernel(uint4 *eq, const uint4 *point, int k) {
    if (threadIdx.x == 0) eq[0] = make_uint4(1, 0, 0, 0);
    __syncthreads();
    for (int i = 0; i < k; ++i) {
        const uint4 r = point[i];
        const uint32_t half = 1u << i;
        for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) {
            const uint4 p = eq[j];
            const uint4 one = gf_mul(p, r);
            eq[half + j] = one;
            eq[j] = gf_add(p, one);
        }
        __syncthreads();
    }
}

// eq over k variables in one launch, as the product of two half tables:
// eq[j] = lo[j mod 2^a] * hi[j >> a], lo over point[0..a) and hi over
// point[a..k).  Every factor of an entry is the same field element as in the
// doubling rounds (bit i of j picks r_i or 1 + r_i), so the entries are
// identical.  Each CTA builds both halves in shared memory (their rounds side
// by side), then writes its share of the products.
constexpr int kEqSplitMaxK = 22;
__global__ void __launch_bounds__(512) eq_split_kernel(uint4 *eq, const uint4 *point, int k,
                                                       int a) {
    extern __shared__ uint4 halves[];
    const int b = k - a;
    uint4 *lo = halves, *hi = halves + ((size_t)1 << a);
    if (threadIdx.x == 0) {
        lo[0] = make_uint4(1, 0, 0, 0);
        hi[0] = make_uint4(1, 0, 0, 0);
    }
    __syncthreads();
    for (int i = 0; i < (a > b ? a : b); ++i) {
        const uint32_t nlo = i < a ? 1u << i : 0u, nhi = i < b ? 1u << i : 0u;
        for (uint32_t j = threadIdx.x; j < nlo + nhi; j += blockDim.x) {
            const bool in_lo = j < nlo;
            uint4 *t = in_lo ? lo : hi;
            const uint32_t jj = in_lo ? j : j - nlo;
            const uint4 r = point[in_lo ? i : a + i];
            const uint4 p = t[jj];
            const uint4 one = gf_mul(p, r);
            t[(1u << i) + jj] = one;
            t[jj] = gf_add(p, one);
        }
        __syncthreads();
    }
    const uint64_t n = (uint64_t)1 << k;
    const uint64_t mask = ((uint64_t)1 << a) - 1;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += (uint64_t)gridDim.x * blockDim.x)
        eq[j] = gf_mul(lo[j & mask], hi[j >> a]);
}

constexpr size_t kEqSmallRounds = 12;

// Up to 6 variables: the doubling rounds in one CTA.  Up to 22: one split
// launch (2^12 entries: 3 to 4 us of products after 6 half-table rounds,
// against 12 rounds in one CTA; 2^20: one launch instead of nine).  Above:
// 12 rounds in one CTA, then one launch per further round.
int launch_build_eq(const uint4 *d_point, size_t k, uint4 *d_out, cudaStream_t st,
                    int num_sms) {
    if (k > 6 && k <= (size_t)kEqSplitMaxK) {
        const int a = (int)k / 2;
        const size_t smem = (((size_t)1 << a) + ((size_t)1 << (k - a))) * sizeof(uint4);
        const uint64_t n = (uint64_t)1 << k;
        const unsigned grid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>((n + 511) / 512, (uint64_t)2 * num_sms));
        eq_split_kernel<<<grid, 512, smem, st>>>(d_out, d_point, (int)k, a);
        return 1;
    }
    const size_t k0 = std::min(k, kEqSmallRounds);
    eq_small_kernel<<<1, 512, 0, st>>>(d_out, d_point, (int)k0);
    for (size_t i = k0; i < k; ++i) {
        const uint64_t half = (uint64_t)1 << i;
        const unsigned grid = (unsigned)std::min<uint64_t>((half + 255) / 256, 8192);
        eq_round_kernel<<<std::max(grid, 1u), 256, 0, st>>>(d_out, half, d_point, (int)i);
    }
    return (int)(k - k0) + 1;
}

// sv[j] = sum_y eq[y] * bit_j(P[y]) (src/ligerito.rs:317-375).  128 threads
// per CTA, one per output bit j.  For each tile of 256 y the CTA stages P in
// shared memory and, per group of 4 consecutive y, the 16 XORs of eq over
// every subset of the group.  Thread j gathers bit j of the group's 4 P words
// into a 4-bit index and adds that subset's sum: one lookup per 4 y instead
// of 4 masked additions.
constexpr int kSvTile = 256;
__global__ void __launch_bounds__(128) sv_fold_kernel(const uint4 *packed, const uint4 *eq,
                                                      uint64_t n, uint4 *partials) {
    __shared__ uint32_t sp[kSvTile][4];
    __shared__ uint4 sub[kSvTile / 4][16];
    const int j = threadIdx.x;
    const int wsel = j >> 5;
    const uint32_t bit = j & 31;
    uint4 acc = make_uint4(0, 0, 0, 0);
    for (uint64_t base = (uint64_t)blockIdx.x * kSvTile; base < n;
         base += (uint64_t)gridDim.x * kSvTile) {
        __syncthreads();
        for (int i = threadIdx.x; i < kSvTile; i += blockDim.x) {
            const uint64_t y = base + i;
            const uint4 v = y < n ? packed[y] : make_uint4(0, 0, 0, 0);
            sp[i][0] = v.x;
            sp[i][1] = v.y;
            sp[i][2] = v.z;
            sp[i][3] = v.w;
        }
        {
            // thread t builds subsets 8h .. 8h+7 of group g = t / 2 (h = t mod 2)
            const int g = threadIdx.x >> 1, h = threadIdx.x & 1;
            uint4 e[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint64_t y = base + 4 * g + k;
                e[k] = y < n ? eq[y] : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int m = 8 * h + q;
                uint4 t = make_uint4(0, 0, 0, 0);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if ((m >> k) & 1) t = gf_add(t, e[k]);
                sub[g][m] = t;
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int g = 0; g < kSvTile / 4; ++g) {
            uint32_t idx = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) idx |= ((sp[4 * g + k][wsel] >> bit) & 1u) << k;
            acc = gf_add(acc, sub[g][idx]);
        }
    }
    partials[(uint64_t)blockIdx.x * 128 + j] = acc;
}

// 1024 threads: thread (g, j) XORs output j of partials g, g + 8, ...; the 8
// groups then combine in shared memory.
constexpr int kSvFinishGroups = 8;
__global__ void __launch_bounds__(128 * kSvFinishGroups) sv_finish_kernel(const uint4 *partials,
                                                                          int n_ctas, uint4 *sv) {
    __shared__ uint4 red[kSvFinishGroups][128];
    const int j = threadIdx.x & 127, g = threadIdx.x >> 7;
    uint4 acc = make_uint4(0, 0, 0, 0);
    for (int c = g; c < n_ctas; c += kSvFinishGroups)
        acc = gf_add(acc, partials[(uint64_t)c * 128 + j]);
    red[g][j] = acc;
    __syncthreads();
    if (g == 0) {
        for (int k = 1; k < kSvFinishGroups; ++k) acc = gf_add(acc, red[k][j]);
        sv[j] = acc;
    }
}

size_t sv_partials_bytes(size_t n, int num_sms) {
    (void)n;
    return (size_t)num_sms * 4 * 128 * 16;
}

int launch_sv_fold(const uint4 *d_packed, const uint4 *d_eq, size_t n, uint64_t *d_partials,
                   uint4 *d_sv, cudaStream_t st, int num_sms) {
    const uint64_t tiles = (n + kSvTile - 1) / kSvTile;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)num_sms * 4));
    uint4 *parts = reinterpret_cast<uint4 *>(d_partials);
    sv_fold_kernel<<<grid, 128, 0, st>>>(d_packed, d_eq, n, parts);
    sv_finish_kernel<<<1, 128 * kSvFinishGroups, 0, st>>>(parts, grid, d_sv);
    return 2;
}

// phi_from_words with phi_byte_tables (src/ligerito.rs:384-427): phi(y) =
// sum over the set bits u of eq_hi[y] of eq_r2[u], a GF(2)-linear map of
// eq_hi[y] whose image of bit u is eq_r2[u].  So it is a byte-table multiply:
// the tables are expanded from those 128 images in the bank-conflict-free
// layout of the NTT's and the folds' tables, and each word is one 16-lookup
// table multiply.
__global__ void __launch_bounds__(256) phi_kernel(const uint4 *eq_hi, uint64_t n,
                                                  const uint4 *eq_r2, uint4 *out) {
    extern __shared__ uint4 smem[];
    uint4 *bases = smem + kT16Entries;
    for (int e = threadIdx.x; e < 128; e += blockDim.x)
        bases[(e >> 3) * 9 + (e & 7)] = eq_r2[e];
    __syncthreads();
    t16_expand(smem, bases, 1);
    const char *T = reinterpret_cast<const char *>(smem);
    T16Lane8 lc;
    lc.init();
    for (uint64_t y = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; y < n;
         y += (uint64_t)gridDim.x * blockDim.x)
        out[y] = lc.mul(T, eq_hi[y]);
}

void init_gkr_kernels();

void init_fold_kernels() {
    init_gkr_kernels();
    cudaFuncSetAttribute(phi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kRTableSmem);
    cudaFuncSetAttribute(eq_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)((2u << (kEqSplitMaxK / 2)) * sizeof(uint4)));
    cudaFuncSetAttribute(fold_and_msg_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kRTableSmem);
    cudaFuncSetAttribute(fold_and_msg_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kRTableSmem);
    cudaFuncSetAttribute(partial_eval_round_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kRTableSmem);
}

// Two CTAs per SM at most: every CTA builds the 64 KB of tables first, so a
// grid-stride loop over fewer CTAs builds them fewer times.
int launch_phi(const uint4 *d_eq_hi, size_t n, const uint4 *d_eq_r2, uint4 *d_out,
               cudaStream_t st, int num_sms) {
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((n + 255) / 256, (uint64_t)2 * num_sms));
    phi_kernel<<<grid, 256, kRTableSmem, st>>>(d_eq_hi, n, d_eq_r2, d_out);
    return 1;
}

// ---------------------------------------------------------------------------
// ChaCha20 (RFC 8439 section 2.3): one 64-byte block per thread = 4 words.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t rotl(uint32_t x, int n) { return __funnelshift_l(x, x, n); }
#define BZ_QR(a, b, c, d)                                 \
    do {                                                  \
        x[a] += x[b]; x[d] = rotl(x[d] ^ x[a], 16);       \
        x[c] += x[d]; x[b] = rotl(x[b] ^ x[c], 12);       \
        x[a] += x[b]; x[d] = rotl(x[d] ^ x[a], 8);        \
        x[c] += x[d]; x[b] = rotl(x[b] ^ x[c], 7);        \
    } while (0)

__global__ void chacha_kernel(uint32_t k0, uint32_t k1, uint64_t first_word, uint4 *out,
                              uint64_t n_words) {
    const uint64_t first_blk = first_word >> 2;
    const uint64_t last_blk = (first_word + n_words - 1) >> 2;
    for (uint64_t blk = first_blk + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
         blk <= last_blk; blk += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, k0, k1, 0, 0,
                           0, 0, 0, 0, (uint32_t)blk, 0, 0, 0};
        uint32_t x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = st[i];
#pragma unroll
        for (int i = 0; i < 10; ++i) {
            BZ_QR(0, 4, 8, 12); BZ_QR(1, 5, 9, 13); BZ_QR(2, 6, 10, 14); BZ_QR(3, 7, 11, 15);
            BZ_QR(0, 5, 10, 15); BZ_QR(1, 6, 11, 12); BZ_QR(2, 7, 8, 13); BZ_QR(3, 4, 9, 14);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] += st[i];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint64_t w = blk * 4 + q;
            if (w >= first_word && w < first_word + n_words)
                out[w - first_word] = make_uint4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
        }
    }
}

int launch_chacha(uint64_t seed, uint64_t first_word, uint4 *d_out, size_t n_words,
                  cudaStream_t st) {
    if (n_words == 0) return 0;
    const uint64_t blocks = ((first_word + n_words - 1) >> 2) - (first_word >> 2) + 1;
    const unsigned grid = (unsigned)std::min<uint64_t>((blocks + 255) / 256, 8192);
    chacha_kernel<<<grid, 256, 0, st>>>((uint32_t)seed, (uint32_t)(seed >> 32), first_word, d_out,
                                        n_words);
    return 1;
}

// ---------------------------------------------------------------------------
// Batched grand-product GKR (BitZ src/bitz/gkr.rs), the dense rounds.
// ---------------------------------------------------------------------------
// One product layer: out[i] = in[i] * in[half + i] (GrandProductCircuit::
// batched_eval, gkr.rs:93-108: the top index bit pairs the factors).
__global__ void __launch_bounds__(256) gkr_product_kernel(const uint4 *in, uint64_t half,
                                                          uint4 *out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < half;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = gf_mul(in[i], in[half + i]);
}

// One dense round over h slots (prove_dense_rounds, gkr.rs:188-282, with the
// column-free weights): the tables l and r (the layer's two halves) hold the
// round's lo entries at [0, h) and hi entries at [h, 2h).  With FOLD the
// previous round's challenge rho is applied first, in place: entries q0..q3
// at c, h + c, 2h + c, 3h + c become q0 + rho (q2 - q0) at c and
// q1 + rho (q3 - q1) at h + c (kernels.rs:146-186, 312-348).  Each CTA
// stores its partial sums of w_c l_end r_end and w_c (l_hi - l_lo)(r_hi -
// r_lo) (kernels.rs:248-262; l_end = l_hi when send_one), unreduced; the
// finish kernel reduces them.  With w_next, the next round's weights
// w_next[c] = w[c] + w[c + h/2] (eq over one coordinate fewer: the two
// values of the dropped coordinate's factor sum to 1) are written too.
template <bool FOLD>
__global__ void __launch_bounds__(256, 2) gkr_round_kernel(uint4 *l, uint4 *r, const uint4 *w,
                                                           uint64_t h, uint4 rho, int send_one,
                                                           uint64_t *partials, MsgMailbox mb,
                                                           uint4 *w_next) {
    extern __shared__ uint4 smem[];
    const char *T = nullptr;
    T16Lane8 lc;
    if constexpr (FOLD) {
        T = build_r_table(smem, rho);
        lc.init();
    }
    gf_wide e = gf_wide_zero(), f = gf_wide_zero();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < h; c += stride) {
        uint4 l0, l1, r0, r1;
        if constexpr (FOLD) {
            const uint4 a0 = l[c], a1 = l[h + c], a2 = l[2 * h + c], a3 = l[3 * h + c];
            const uint4 b0 = r[c], b1 = r[h + c], b2 = r[2 * h + c], b3 = r[3 * h + c];
            l0 = gf_add(a0, lc.mul(T, gf_add(a2, a0)));
            l1 = gf_add(a1, lc.mul(T, gf_add(a3, a1)));
            r0 = gf_add(b0, lc.mul(T, gf_add(b2, b0)));
            r1 = gf_add(b1, lc.mul(T, gf_add(b3, b1)));
            l[c] = l0;
            l[h + c] = l1;
            r[c] = r0;
            r[h + c] = r1;
        } else {
            l0 = l[c];
            l1 = l[h + c];
            r0 = r[c];
            r1 = r[h + c];
        }
        const uint4 wc = w[c];
        if (w_next && c < h / 2) w_next[c] = gf_add(wc, w[c + h / 2]);
        const uint4 le = send_one ? l1 : l0, re = send_one ? r1 : r0;
        gf_wide_xor(e, gf_mul_wide(gf_mul(wc, le), re));
        gf_wide_xor(f, gf_mul_wide(gf_mul(wc, gf_add(l1, l0)), gf_add(r1, r0)));
    }
    msg_finish_call(e, f, partials, mb);
}

// The leaf grid of the BitZ forest (src/bitz/forest_tests.rs:42-68): leaf
// row * 2^s + column is images[row] when bit (column mod 64) of
// packed[(column / 64) * 2^t + row] is set, else 1.
__global__ void __launch_bounds__(256) gkr_forest_leaves_kernel(const uint64_t *packed,
                                                                const uint4 *images, int t,
                                                                int s, uint4 *out) {
    const uint64_t n = (uint64_t)1 << (t + s), rows = (uint64_t)1 << t;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t row = i >> s, col = i & (((uint64_t)1 << s) - 1);
        const uint64_t bit = (packed[(col >> 6) * rows + row] >> (col & 63)) & 1;
        out[i] = bit ? images[row] : make_uint4(1, 0, 0, 0);
    }
}

int launch_gkr_product(const uint4 *d_in, size_t half, uint4 *d_out, cudaStream_t st,
                       int num_sms) {
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((half + 255) / 256, (uint64_t)num_sms * 8));
    gkr_product_kernel<<<grid, 256, 0, st>>>(d_in, half, d_out);
    return 1;
}

int gkr_round_grid(size_t h, int num_sms) { return std::min(msg_grid(h, num_sms), 1024); }

int launch_gkr_round(uint4 *d_l, uint4 *d_r, const uint4 *d_w, size_t h, bool fold, uint4 rho,
                     bool send_one, uint4 *d_w_next, uint64_t *d_partials, uint64_t *d_out,
                     cudaStream_t st, int num_sms, const MsgPost *post) {
    const int grid = gkr_round_grid(h, num_sms);
    MsgMailbox mb;
    if (post) mb = {post->ticket, post->words, post->seq, post->seq_val};
    if (fold)
        gkr_round_kernel<true><<<grid, 256, kRTableSmem, st>>>(d_l, d_r, d_w, h, rho, send_one,
                                                               d_partials, mb, d_w_next);
    else
        gkr_round_kernel<false><<<grid, 256, 0, st>>>(d_l, d_r, d_w, h, rho, send_one,
                                                      d_partials, mb, d_w_next);
    if (post) return 1;
    finish_msg_kernel<<<1, kFinishThreads, 0, st>>>(d_partials, grid, d_out);
    return 2;
}

void init_gkr_kernels() {
    cudaFuncSetAttribute(gkr_round_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kRTableSmem);
}

int launch_gkr_forest_leaves(const uint64_t *d_packed, const uint4 *d_images, int t, int s,
                             uint4 *d_out, cudaStream_t st, int num_sms) {
    const uint64_t n = (uint64_t)1 << (t + s);
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((n + 255) / 256, (uint64_t)num_sms * 8));
    gkr_forest_leaves_kernel<<<grid, 256, 0, st>>>(d_packed, d_images, t, s, d_out);
    return 1;
}

}  // namespace bz
