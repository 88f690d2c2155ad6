// Forward interleaved additive NTT over GF(2^128) (LCH novel basis) for the
// Reed-Solomon row encoding of the commit.
//
// Semantics follow flock-core/src/ntt/additive_ntt_f128.rs:
//   * twiddle(l, b) = span of the normalized subspace-polynomial row
//     evals[ell-l-1][1..] selected by the bits of b (:63-156);
//   * layer l: blocks of 2^(ell-l) positions, pairs (row, row + half), every
//     lane: u <- u + t*v ; v <- v + u (:243-274);
//   * the first r layers of [msg, 0, ..] are copies, so the transform starts
//     at layer r from 2^r replicas of the message (commit.rs:223-258).
// Data layout: cw[pos * L + lane], 16 bytes per element, L = 2^log_lanes.
//
// GB300 mapping (integer pipes; no tensor cores -- nothing here is a dense
// floating-point contraction):
//   * "table" passes fuse two layers (radix-4) or one (radix-2) over the
//     wide-twiddle layers.  Every thread owns one (block, row, lane) quad, so
//     global loads/stores are 16-byte vectors coalesced across lanes.  A
//     multiply by the block twiddle t is 16 lookups into a 64 KB shared-memory
//     table T_k[x] = x * X^(8k) * t (one per byte k of the operand).  Tables
//     are laid out so byte position k lives in bank group k mod 8 and each
//     thread walks the byte positions in an order rotated by (lane mod 8):
//     the 8 threads of a quarter-warp always hit 8 different bank groups, so
//     the 128-bit lookups are bank-conflict free.  The first table pass reads
//     the message and writes all 2^r replicas (the replicate fill is fused).
//   * the deepest radix-4 passes (schedule bit SCHED_NARROW) exploit that
//     their twiddles are narrow (at depth i the twiddle has at most about
//     2^i * ell bits): a byte times such a twiddle is an unreduced product of
//     at most 64 bits, so one compact 256-entry table of one or two words
//     replaces the sixteen 16-byte tables (ntt_table_pass2_pf with WO or
//     WAB below 4).
//   * the "deep" pass runs the last D layers (D <= 4) on 2^D consecutive
//     positions held in registers, the multiply being a shift-and-XOR over
//     the narrow twiddle's set bits, with the twiddle warp-uniform.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "bz_internal.h"
#include "gf128.cuh"
#include "t16.cuh"
#include "t8.cuh"
#include "ntt_kernels.cuh"

namespace bz {

// ===========================================================================
// Host: normalized subspace-polynomial rows and the twiddle heap.
// ===========================================================================
// evals[i][k], i < ell, k < ell - i (additive_ntt_f128.rs:66-100) for the
// basis {1, x, .., x^(ell-1)} (:136-140), element (i, k) at words
// 2 * (i * ell + k) and + 1.
static std::vector<uint64_t> normalized_evals(int ell) {
    std::vector<uint64_t> ev(2 * (size_t)ell * ell, 0);
    auto at = [&](int i, int k) { return &ev[2 * ((size_t)i * ell + k)]; };
    for (int k = 0; k < ell; ++k) {
        at(0, k)[0] = k < 64 ? (1ull << k) : 0;
        at(0, k)[1] = k >= 64 ? (1ull << (k - 64)) : 0;
    }
    for (int i = 1; i < ell; ++i) {
        for (int k = 1; k < ell - (i - 1); ++k) {
            const uint64_t *p = at(i - 1, k), *p0 = at(i - 1, 0);
            uint64_t s[2] = {p[0] ^ p0[0], p[1] ^ p0[1]};
            hgf_mul(p, s, at(i, k - 1));
        }
    }
    for (int i = 0; i < ell; ++i) {
        uint64_t inv[2];
        hgf_inv(at(i, 0), inv);
        for (int k = 0; k < ell - i; ++k) {
            uint64_t t[2];
            hgf_mul(at(i, k), inv, t);
            at(i, k)[0] = t[0];
            at(i, k)[1] = t[1];
        }
    }
    return ev;
}

std::vector<uint64_t> twiddle_heap(int ell) {
    std::vector<uint64_t> ev = normalized_evals(ell);
    auto at = [&](int i, int k) { return &ev[2 * ((size_t)i * ell + k)]; };
    std::vector<uint64_t> heap(2 * ((size_t)1 << ell) + 2, 0);
    for (int l = 0; l < ell; ++l) {
        const size_t base = (size_t)1 << l;
        const int row = ell - l - 1;
        heap[2 * base] = 0;
        heap[2 * base + 1] = 0;
        for (size_t b = 1; b < base; ++b) {
            const int j = __builtin_ctzll(b);
            const uint64_t *prev = &heap[2 * (base + (b & (b - 1)))];
            const uint64_t *e = at(row, 1 + j);
            heap[2 * (base + b)] = prev[0] ^ e[0];
            heap[2 * (base + b) + 1] = prev[1] ^ e[1];
        }
    }
    return heap;
}

// Bit length of the widest twiddle of `layer`: twiddle(layer, b) is the XOR
// of evals[ell - layer - 1][1 + j] over the set bits j < layer of b, so it
// is no wider than its widest generator.  Deep layers have narrow twiddles
// (about ell, 2 ell - 3, 4 ell - 11 bits at depths 0, 1, 2).
int twiddle_bits(int ell, int layer) {
    static std::mutex mu;
    static std::map<int, std::vector<int>> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(ell);
    if (it == cache.end()) {
        const std::vector<uint64_t> ev = normalized_evals(ell);
        std::vector<int> bits(ell, 0);
        for (int l = 0; l < ell; ++l) {
            const int row = ell - l - 1;
            for (int k = 1; k <= l; ++k) {
                const uint64_t lo = ev[2 * ((size_t)row * ell + k)];
                const uint64_t hi = ev[2 * ((size_t)row * ell + k) + 1];
                const int b = hi ? 128 - __builtin_clzll(hi) : (lo ? 64 - __builtin_clzll(lo) : 0);
                bits[l] = std::max(bits[l], b);
            }
        }
        it = cache.emplace(ell, std::move(bits)).first;
    }
    return it->second[layer];
}

// Schedule of a shape the autotuner has not timed.  With at least 512 lanes
// every layer fits the table passes (each 512-thread chunk stays inside one
// block); radix-8 passes (three layers per sweep) measured faster than the
// prefetching radix-4 passes at 2^20, 2^24 and 2^28 (3.33 against 3.49 ms at
// 2^24); narrower shapes run their last three layers in the
// register-resident deep pass.
uint32_t default_schedule(const Shape &s) {
    if (s.log_lanes >= 9 && s.k_code() - s.log_inv_rate >= 3) return SCHED_RADIX8;
    if (s.log_lanes >= 9) return SCHED_PREFETCH | SCHED_NARROW;
    const int layers = s.log_dim();
    const int deep = std::min(layers, 3);
    return (uint32_t)deep;
}

// CTAs per SM a table pass is cut into: 1 (one long CTA per SM) or, under
// SCHED_SHORT_CTAS, 16 shorter ones, so a kernel of a higher-priority stream
// waits for one of those instead of the whole pass to get an SM.  Served
// commits take it: against 8, the small requests' slowdown p99 fell from
// 10-14 to 6-13 at light load with the same saturated throughput; 32 cost
// throughput.
static int cta_waves(uint32_t schedule) { return (schedule & SCHED_SHORT_CTAS) ? 16 : 1; }

// ---- kernels: one CTA per contiguous range of task chunks ------------------
// Chunks [c_beg, c_end) of this CTA when n_tasks is cut into blockDim.x-task
// chunks spread evenly over the grid.
__device__ __forceinline__ void cta_chunks(uint64_t n_tasks, uint64_t &c_beg, uint64_t &c_end) {
    const uint64_t chunks = n_tasks / blockDim.x;
    c_beg = chunks * blockIdx.x / gridDim.x;
    c_end = chunks * (blockIdx.x + 1) / gridDim.x;
}

template <int LAYERS, int THREADS>
__global__ void __launch_bounds__(THREADS, 1) ntt_table_pass(TablePassArgs a) {
    extern __shared__ uint4 smem[];
    __shared__ uint4 tw_buf[kTwWindow * (LAYERS == 2 ? 3 : 1)];
    __shared__ uint64_t win[2];
    __shared__ int tz[3];
    uint64_t c_beg, c_end;
    cta_chunks(a.n_tasks, c_beg, c_end);
    table_pass_body<LAYERS>(a, c_beg, c_end, smem, tw_buf, win, tz);
}

template <int THREADS, int MINB, int WO, int WAB>
__global__ void __launch_bounds__(THREADS, MINB) ntt_table_pass2_pf(TablePassArgs a) {
    extern __shared__ uint4 smem[];
    __shared__ uint4 tw_buf[kTwWindow * 3];
    __shared__ uint64_t win[2];
    uint64_t c_beg, c_end;
    cta_chunks(a.n_tasks, c_beg, c_end);
    table_pass2_pf_body<WO, WAB>(a, c_beg, c_end, smem, tw_buf, win);
}

template <int W0, int W1, int W2>
__global__ void __launch_bounds__(512, 1) ntt_pass8(TablePassArgs a) {
    extern __shared__ uint4 smem[];
    __shared__ uint4 tw_buf[kTw8Window * 7];
    __shared__ uint64_t win[2];
    uint64_t c_beg, c_end;
    cta_chunks(a.n_tasks, c_beg, c_end);
    pass8_body<W0, W1, W2>(a, c_beg, c_end, reinterpret_cast<char *>(smem), tw_buf, win);
}

template <int D, int MODE>
__global__ void __launch_bounds__(256) ntt_deep_pass(DeepArgs a) {
    deep_pass_body<D, MODE>(a, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, a.n_tasks,
                            (uint64_t)gridDim.x * blockDim.x);
}

__global__ void ntt_generic_layer(const uint4 *src, uint4 *dst, const uint4 *tw, int ell,
                                  int layer, int log_lanes, int src_pos_bits, uint64_t n_tasks) {
    generic_layer_body(src, dst, tw, ell, layer, log_lanes, src_pos_bits,
                       (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, n_tasks,
                       (uint64_t)gridDim.x * blockDim.x);
}


// Fused tail: the last DT table layers and the DN narrow layers on one group
// of 2^(DT+DN) consecutive positions per thread (one lane), so the
// shared-memory lookups of the table layers and the ALU work of the narrow
// layers overlap inside one pass over the codeword.  Needs >= 512 lanes so
// every CTA chunk shares the group G (and therefore the tables).
template <int DT, int DN, int MODE>
__global__ void __launch_bounds__(512, 1) ntt_tail_pass(DeepArgs a) {
    extern __shared__ uint4 smem[];
    constexpr int NT = DT == 2 ? 3 : 1;
    constexpr int P = 1 << (DT + DN);
    uint4 *tbl = smem;
    uint4 *bases = smem + NT * kT16Entries;
    __shared__ uint4 ts[3];
    __shared__ int tz[3];
    T16Lane lane_ctx;
    lane_ctx.init();
    const int l0 = a.ell - DT - DN;
    const uint64_t lanes_mask = ((uint64_t)1 << a.log_lanes) - 1;
    const uint64_t src_mask = ((uint64_t)1 << a.src_pos_bits) - 1;
    const uint64_t chunks = a.n_tasks / blockDim.x;
    const uint64_t c_beg = chunks * blockIdx.x / gridDim.x;
    const uint64_t c_end = chunks * (blockIdx.x + 1) / gridDim.x;
    int64_t cur_g = -1;
    for (uint64_t c = c_beg; c < c_end; ++c) {
        const uint64_t task = a.task_base + c * blockDim.x + threadIdx.x;
        const uint64_t G = task >> a.log_lanes;  // uniform across the CTA
        const uint64_t ln = task & lanes_mask;
        if ((int64_t)G != cur_g) {
            __syncthreads();
            if (threadIdx.x == 0) {
                ts[0] = a.tw[((uint64_t)1 << l0) + G];
                if (DT == 2) {
                    ts[1] = a.tw[((uint64_t)1 << (l0 + 1)) + 2 * G];
                    ts[2] = a.tw[((uint64_t)1 << (l0 + 1)) + 2 * G + 1];
                }
                for (int i = 0; i < NT; ++i) tz[i] = gf_is_zero(ts[i]);
            }
            __syncthreads();
            t16_build(tbl, bases, ts, NT);
            cur_g = (int64_t)G;
        }
        uint4 v[P];
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const uint64_t pos = (G << (DT + DN)) + i;
            v[i] = __ldcs(a.src + (((pos & src_mask) << a.log_lanes) | ln));
        }
        const char *T0 = reinterpret_cast<const char *>(tbl);
        // table layer l0: pairs (i, i + P/2)
#pragma unroll
        for (int i = 0; i < P / 2; ++i) {
            if (!tz[0]) v[i] = gf_add(v[i], lane_ctx.mul(T0, v[i + P / 2]));
            v[i + P / 2] = gf_add(v[i + P / 2], v[i]);
        }
        if (DT == 2) {
            // table layer l0+1: blocks 2G (first half) and 2G+1 (second half)
#pragma unroll
            for (int hb = 0; hb < 2; ++hb) {
                const char *Tb = T0 + (size_t)(1 + hb) * kT16Entries * 16;
                const bool z = tz[1 + hb];
#pragma unroll
                for (int i = 0; i < P / 4; ++i) {
                    uint4 &u = v[hb * (P / 2) + i];
                    uint4 &w = v[hb * (P / 2) + i + P / 4];
                    if (!z) u = gf_add(u, lane_ctx.mul(Tb, w));
                    w = gf_add(w, u);
                }
            }
        }
        // narrow layers: groups of 2^DN positions, group index G * 2^DT + g
        narrow_layers<DN, P, MODE>(v, a.tw, a.ell, G);
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const uint64_t pos = (G << (DT + DN)) + i;
            __stcs(a.dst + ((pos << a.log_lanes) | ln), v[i]);
        }
    }
}


// The whole transform of a small shape in one launch: one CTA per lane holds
// the lane's 2^ell codeword positions in shared memory (the replicated
// message, read through the position mask as the first table pass does), and
// each thread does one butterfly per layer with the generic multiply.  The
// layers, blocks and twiddles are those of ntt_generic_layer.
__global__ void __launch_bounds__(512) ntt_small_kernel(const uint4 *msg, uint4 *cw,
                                                        const uint4 *tw, int ell, int r,
                                                        int log_lanes, int msg_pos_bits) {
    extern __shared__ uint4 col[];
    const uint32_t P = 1u << ell;
    const uint64_t lane = blockIdx.x;
    const uint32_t msg_mask = (1u << msg_pos_bits) - 1;
    for (uint32_t p = threadIdx.x; p < P; p += blockDim.x)
        col[p] = msg[((uint64_t)(p & msg_mask) << log_lanes) | lane];
    for (int layer = r; layer < ell; ++layer) {
        __syncthreads();
        const int log_h = ell - layer - 1;
        for (uint32_t pair = threadIdx.x; pair < P / 2; pair += blockDim.x) {
            const uint32_t B = pair >> log_h, rr = pair & ((1u << log_h) - 1);
            const uint32_t p0 = (B << (log_h + 1)) + rr, p1 = p0 + (1u << log_h);
            const uint4 t = tw[(1u << layer) + B];
            uint4 u = col[p0], w = col[p1];
            u = gf_add(u, gf_mul(w, t));
            w = gf_add(w, u);
            col[p0] = u;
            col[p1] = w;
        }
    }
    __syncthreads();
    for (uint32_t p = threadIdx.x; p < P; p += blockDim.x)
        cw[((uint64_t)p << log_lanes) | lane] = col[p];
}

// Shapes small enough for ntt_small_kernel to beat the table passes (the
// recursive levels' commits and small requests).  Measured on GB300: 2^12
// elements as 64 lanes of 2^8 positions 11.9 us against 30.4 us for the pass
// sequence, 2^14 as 128 lanes of 2^9 positions 15.7 against 33.3 us; at 256
// lanes of 2^10 positions (2^16 elements) the passes win, 31 against 42 us.
bool small_ntt_ok(const Shape &s) {
    return s.log_dim() >= 1 && s.k_code() <= 9 && s.log_lanes <= 8;
}

// cw[rep * N + i] = msg[i] for every replica (commit.rs:239-258).
__global__ void replicate_fill(const uint4 *msg, uint4 *cw, uint64_t msg_words, int reps) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < msg_words;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 v = __ldcs(msg + i);
        for (int r = 0; r < reps; ++r) __stcs(cw + (uint64_t)r * msg_words + i, v);
    }
}

static inline unsigned grid_for(uint64_t n, int threads, int num_sms, int per_sm) {
    uint64_t g = (n + threads - 1) / threads;
    const uint64_t cap = (uint64_t)num_sms * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (unsigned)g;
}

#define BZ_TAIL_ATTR(DT, DN, M)                                                           \
    cudaFuncSetAttribute(ntt_tail_pass<DT, DN, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                         (int)table_smem(DT))
#define BZ_TAIL_ATTR_M(DT, DN) BZ_TAIL_ATTR(DT, DN, 0); BZ_TAIL_ATTR(DT, DN, 1); BZ_TAIL_ATTR(DT, DN, 2)

void init_ntt_kernels() {
    cudaFuncSetAttribute(ntt_table_pass<2, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)table_smem(2));
    cudaFuncSetAttribute(ntt_table_pass<1, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)table_smem(1));
    cudaFuncSetAttribute(ntt_table_pass<2, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)table_smem(2));
    cudaFuncSetAttribute(ntt_table_pass<1, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)table_smem(1));
#define BZ_PF_ATTR(T, M, WO, WAB)                                                          \
    cudaFuncSetAttribute(ntt_table_pass2_pf<T, M, WO, WAB>,                                  \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pf_smem(WO, WAB))
    BZ_PF_ATTR(512, 1, 4, 4);
    BZ_PF_ATTR(256, 1, 4, 4);
    BZ_PF_ATTR(256, 2, 4, 4);
    BZ_PF_ATTR(512, 1, 1, 1);
    BZ_PF_ATTR(512, 1, 2, 1);
    BZ_PF_ATTR(512, 1, 4, 1);
    BZ_PF_ATTR(512, 1, 2, 2);
    BZ_PF_ATTR(512, 1, 4, 2);
#undef BZ_PF_ATTR
    BZ_TAIL_ATTR_M(1, 1); BZ_TAIL_ATTR_M(1, 2); BZ_TAIL_ATTR_M(1, 3);
    BZ_TAIL_ATTR_M(2, 1); BZ_TAIL_ATTR_M(2, 2);
#define BZ_P8_ATTR(A, B, C)                                                                  \
    cudaFuncSetAttribute(ntt_pass8<A, B, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                         kPass8Smem)
    BZ_P8_ATTR(4, 4, 4); BZ_P8_ATTR(4, 4, 2); BZ_P8_ATTR(4, 4, 1); BZ_P8_ATTR(4, 2, 2);
    BZ_P8_ATTR(4, 2, 1); BZ_P8_ATTR(4, 1, 1); BZ_P8_ATTR(2, 2, 2); BZ_P8_ATTR(2, 2, 1);
    BZ_P8_ATTR(2, 1, 1); BZ_P8_ATTR(1, 1, 1);
#undef BZ_P8_ATTR
}

// One radix-8 pass over layers layer .. layer+2 of every position.  The table
// width of each layer follows its widest twiddle; a shallower layer never
// takes a narrower table than a deeper one of the same pass.
// Returns whether any of its layers multiplies through compact tables.
static bool launch_pass8(const Shape &s, int layer, const uint4 *src, int src_bits, uint4 *dst,
                         const uint4 *tw, cudaStream_t st, int num_sms, int waves = 1) {
    const int ell = s.k_code(), L = s.log_lanes;
    TablePassArgs a;
    a.src = src;
    a.dst = dst;
    a.tw = tw;
    a.ell = ell;
    a.layer = layer;
    a.log_lanes = L;
    a.src_pos_bits = src_bits;
    a.task_base = 0;
    a.n_tasks = (((uint64_t)1 << ell) >> 3) << L;
    int w2 = narrow_class(twiddle_bits(ell, layer + 2));
    int w1 = std::max(narrow_class(twiddle_bits(ell, layer + 1)), w2);
    int w0 = std::max(narrow_class(twiddle_bits(ell, layer)), w1);
    const unsigned grid =
        (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)num_sms * waves,
                                                           a.n_tasks / 512));
    const int key = w0 * 100 + w1 * 10 + w2;
#define BZ_P8_CASE(A, B, C) \
    case A * 100 + B * 10 + C: ntt_pass8<A, B, C><<<grid, 512, kPass8Smem, st>>>(a); break
    switch (key) {
        BZ_P8_CASE(4, 4, 2); BZ_P8_CASE(4, 4, 1); BZ_P8_CASE(4, 2, 2); BZ_P8_CASE(4, 2, 1);
        BZ_P8_CASE(4, 1, 1); BZ_P8_CASE(2, 2, 2); BZ_P8_CASE(2, 2, 1); BZ_P8_CASE(2, 1, 1);
        BZ_P8_CASE(1, 1, 1);
        default: ntt_pass8<4, 4, 4><<<grid, 512, kPass8Smem, st>>>(a); break;
    }
#undef BZ_P8_CASE
    return w2 < 4;
}

template <int D>
static void launch_deep(const DeepArgs &a, int mode, unsigned grid, cudaStream_t st) {
    if (mode == 1) ntt_deep_pass<D, 1><<<grid, 256, 0, st>>>(a);
    else if (mode == 2) ntt_deep_pass<D, 2><<<grid, 256, 0, st>>>(a);
    else ntt_deep_pass<D, 0><<<grid, 256, 0, st>>>(a);
}

template <int DT, int DN>
static void launch_tail(const DeepArgs &a, int mode, unsigned grid, cudaStream_t st) {
    const size_t sm = table_smem(DT);
    if (mode == 1) ntt_tail_pass<DT, DN, 1><<<grid, 512, sm, st>>>(a);
    else if (mode == 2) ntt_tail_pass<DT, DN, 2><<<grid, 512, sm, st>>>(a);
    else ntt_tail_pass<DT, DN, 0><<<grid, 512, sm, st>>>(a);
}

// Whether a table pass runs with compact tables (ntt_table_pass2_pf with
// WAB < 4): those of the narrow twiddles of its second layer, and of its
// first when narrow too.
bool narrow_table_pass(const Shape &s, uint32_t schedule, int layer, int layers, int threads) {
    return (schedule & SCHED_NARROW) && layers == 2 && threads == 512 &&
           narrow_class(twiddle_bits(s.k_code(), layer + 1)) <= 2;
}

int launch_table_pass(const Shape &s, int layer, int layers, const uint4 *src, int src_bits,
                      uint4 *dst, const uint4 *tw, uint64_t p0, uint64_t p1, int threads,
                      cudaStream_t st, int num_sms, uint32_t schedule) {
    const bool prefetch = (schedule & SCHED_PREFETCH) != 0, lean = (schedule & SCHED_LEAN) != 0;
    const int ell = s.k_code(), L = s.log_lanes;
    const int log_q = ell - layer - layers;  // quad / pair stride (positions)
    TablePassArgs a;
    a.src = src;
    a.dst = dst;
    a.tw = tw;
    a.ell = ell;
    a.layer = layer;
    a.log_lanes = L;
    a.src_pos_bits = src_bits;
    // tasks are (B, rr, lane) with B the block index at `layer`
    const uint64_t b0 = p0 >> (ell - layer), b1 = p1 >> (ell - layer);
    a.task_base = (b0 << log_q) << L;
    a.n_tasks = ((b1 - b0) << log_q) << L;
    const unsigned grid =
        (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)num_sms * cta_waves(schedule),
                                                           a.n_tasks / threads));
    if (narrow_table_pass(s, schedule, layer, layers, threads)) {
        const int wo = narrow_class(twiddle_bits(ell, layer));
        const int wab = narrow_class(twiddle_bits(ell, layer + 1));
        const size_t sm = pf_smem(wo, wab);
        if (wab == 1 && wo == 1) ntt_table_pass2_pf<512, 1, 1, 1><<<grid, 512, sm, st>>>(a);
        else if (wab == 1 && wo == 2) ntt_table_pass2_pf<512, 1, 2, 1><<<grid, 512, sm, st>>>(a);
        else if (wab == 1) ntt_table_pass2_pf<512, 1, 4, 1><<<grid, 512, sm, st>>>(a);
        else if (wo == 2) ntt_table_pass2_pf<512, 1, 2, 2><<<grid, 512, sm, st>>>(a);
        else ntt_table_pass2_pf<512, 1, 4, 2><<<grid, 512, sm, st>>>(a);
    } else if (prefetch && layers == 2) {
        const size_t sm = pf_smem(4, 4);
        if (threads == 256 && lean)
            ntt_table_pass2_pf<256, 2, 4, 4><<<grid, 256, sm, st>>>(a);
        else if (threads == 256)
            ntt_table_pass2_pf<256, 1, 4, 4><<<grid, 256, sm, st>>>(a);
        else
            ntt_table_pass2_pf<512, 1, 4, 4><<<grid, 512, sm, st>>>(a);
    } else if (threads == 256) {
        if (layers == 2) ntt_table_pass<2, 256><<<grid, 256, table_smem(2), st>>>(a);
        else ntt_table_pass<1, 256><<<grid, 256, table_smem(1), st>>>(a);
    } else {
        if (layers == 2) ntt_table_pass<2, 512><<<grid, 512, table_smem(2), st>>>(a);
        else ntt_table_pass<1, 512><<<grid, 512, table_smem(1), st>>>(a);
    }
    return 1;
}

int launch_deep_range(const Shape &s, int deep, int mode, const uint4 *src, int src_bits,
                      uint4 *dst, const uint4 *tw, uint64_t p0, uint64_t p1, cudaStream_t st,
                      int num_sms) {
    DeepArgs a;
    a.src = src;
    a.dst = dst;
    a.tw = tw;
    a.ell = s.k_code();
    a.log_lanes = s.log_lanes;
    a.src_pos_bits = src_bits;
    a.task_base = (p0 >> deep) << s.log_lanes;
    a.n_tasks = ((p1 - p0) >> deep) << s.log_lanes;
    const unsigned grid = grid_for(a.n_tasks, 256, num_sms, 8);
    switch (deep) {
        case 1: launch_deep<1>(a, mode, grid, st); break;
        case 2: launch_deep<2>(a, mode, grid, st); break;
        case 3: launch_deep<3>(a, mode, grid, st); break;
        default: launch_deep<4>(a, mode, grid, st); break;
    }
    return 1;
}

int launch_ntt(const Shape &s, uint32_t schedule, const uint4 *d_msg, uint4 *d_cw,
               const uint4 *d_tw, cudaStream_t st, int num_sms, LaunchLog *log) {
    auto mark = [&](const char *n) {
        if (log) log->mark(n);
    };
    const int ell = s.k_code(), r = s.log_inv_rate, L = s.log_lanes, b = s.log_dim();
    const uint64_t P = (uint64_t)1 << ell;
    int launches = 0;
    const uint4 *src = d_msg;
    int src_bits = b;  // message positions are the low b bits of a codeword position
    if (b == 0) {
        replicate_fill<<<grid_for(s.msg_words(), 256, num_sms, 8), 256, 0, st>>>(
            d_msg, d_cw, s.msg_words(), 1 << r);
        mark("replicate_fill");
        return 1;
    }
    const bool generic = (schedule & SCHED_GENERIC) != 0;
    if (!generic && small_ntt_ok(s)) {
        const unsigned threads = (unsigned)std::min<uint64_t>(P / 2, 512);
        ntt_small_kernel<<<1u << L, threads, P * sizeof(uint4), st>>>(d_msg, d_cw, d_tw, ell, r,
                                                                      L, b);
        mark("ntt_small");
        return 1;
    }
    if (generic) {
        for (int layer = r; layer < ell; ++layer) {
            const uint64_t n_tasks = ((uint64_t)1 << (ell - 1)) << L;
            ntt_generic_layer<<<grid_for(n_tasks, 256, num_sms, 8), 256, 0, st>>>(
                src, d_cw, d_tw, ell, layer, L, src_bits, n_tasks);
            mark("ntt_generic_layer");
            ++launches;
            src = d_cw;
            src_bits = 62;
        }
        return launches;
    }
    if ((schedule & SCHED_RADIX8) && L >= 9 && ell - r >= 3) {
        // radix-8 passes; the 1-2 layers left over run as one radix-4 or
        // radix-2 table pass, last (deepest, narrowest twiddles) or first
        const int total = ell - r, rest = total % 3;
        const bool head = (schedule & SCHED_R8_HEAD) != 0;
        const uint32_t pass_sched = SCHED_PREFETCH | SCHED_NARROW | (schedule & SCHED_SHORT_CTAS);
        int layer = r;
        auto small_pass = [&](int layers) {
            launches += launch_table_pass(s, layer, layers, src, src_bits, d_cw, d_tw, 0, P, 512,
                                          st, num_sms, pass_sched);
            if (log) {
                std::string n = layers == 2 ? "ntt_table_pass2" : "ntt_table_pass1";
                if (src == d_msg) n += "_first";
                if (narrow_table_pass(s, pass_sched, layer, layers, 512)) n += "_nw";
                log->mark((n + "@" + std::to_string(layer)).c_str());
            }
            src = d_cw;
            src_bits = 62;
            layer += layers;
        };
        if (head && rest) small_pass(rest);
        while (ell - layer >= 3) {
            const bool nw = launch_pass8(s, layer, src, src_bits, d_cw, d_tw, st, num_sms,
                                         cta_waves(schedule));
            ++launches;
            if (log) {
                // "<kernel>@<first layer>": the profile's reader counts the
                // multiplies of each launch from its layer
                std::string n = src == d_msg ? "ntt_pass8_first" : "ntt_pass8";
                if (nw) n += "_nw";
                log->mark((n + "@" + std::to_string(layer)).c_str());
            }
            src = d_cw;
            src_bits = 62;
            layer += 3;
        }
        if (layer < ell) small_pass(ell - layer);
        return launches;
    }
    int deep = (int)(schedule & SCHED_DEEP_MASK);
    if (deep > b) deep = b;
    if (deep > 4) deep = 4;
    const bool radix2 = (schedule & SCHED_RADIX2) != 0;
    const int mode = (int)((schedule >> SCHED_MODE_SHIFT) & 3);
    const int threads = (schedule & SCHED_SMALL_CTA) ? 256 : 512;
    const int log_threads = threads == 256 ? 8 : 9;
    int table_end = ell - deep;
    // fused tail: the last 1-2 table layers run with the narrow layers
    int tail_dt = 0;
    if ((schedule & SCHED_FUSED_TAIL) && deep >= 1 && L >= 9 && table_end > r) {
        tail_dt = (!radix2 && table_end - r >= 2 && deep <= 2) ? 2 : 1;
        if (tail_dt + deep > 4) tail_dt = 0;
        else table_end -= tail_dt;
    }
    int layer = r;
    while (layer < table_end) {
        const int layers = (!radix2 && layer + 1 < table_end) ? 2 : 1;
        if (!table_pass_ok(ell, layer, layers, L, log_threads)) {
            // too few tasks per block for table passes: generic single layers
            const uint64_t n_tasks = ((uint64_t)1 << (ell - 1)) << L;
            ntt_generic_layer<<<grid_for(n_tasks, 256, num_sms, 8), 256, 0, st>>>(
                src, d_cw, d_tw, ell, layer, L, src_bits, n_tasks);
            mark("ntt_generic_layer");
            ++launches;
            src = d_cw;
            src_bits = 62;
            layer += 1;
            continue;
        }
        launches += launch_table_pass(s, layer, layers, src, src_bits, d_cw, d_tw, 0, P, threads,
                                      st, num_sms, schedule);
        if (log) {
            // "<kernel>@<first layer>": the profile's reader counts the
            // multiplies of each launch from its layer
            std::string n = layers == 2 ? "ntt_table_pass2" : "ntt_table_pass1";
            if (src == d_msg) n += "_first";
            if (narrow_table_pass(s, schedule, layer, layers, threads)) n += "_nw";
            log->mark((n + "@" + std::to_string(layer)).c_str());
        }
        src = d_cw;
        src_bits = 62;
        layer += layers;
    }
    if (deep > 0) {
        if (tail_dt) {
            DeepArgs a;
            a.src = src;
            a.dst = d_cw;
            a.tw = d_tw;
            a.ell = ell;
            a.log_lanes = L;
            a.src_pos_bits = src_bits;
            a.task_base = 0;
            a.n_tasks = ((uint64_t)1 << (ell - deep - tail_dt)) << L;
            const unsigned grid = (unsigned)std::min<uint64_t>(num_sms, a.n_tasks / 512);
            if (tail_dt == 2) {
                if (deep == 1) launch_tail<2, 1>(a, mode, grid, st);
                else launch_tail<2, 2>(a, mode, grid, st);
            } else {
                if (deep == 1) launch_tail<1, 1>(a, mode, grid, st);
                else if (deep == 2) launch_tail<1, 2>(a, mode, grid, st);
                else launch_tail<1, 3>(a, mode, grid, st);
            }
            mark("ntt_tail_pass");
        } else {
            launch_deep_range(s, deep, mode, src, src_bits, d_cw, d_tw, 0, P, st, num_sms);
            mark("ntt_deep_pass");
        }
        ++launches;
    }
    return launches;
}

}  // namespace bz
