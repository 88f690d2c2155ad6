// Device bodies of the NTT passes over GF(2^128) (the semantics and the
// GB300 mapping are described at the top of ntt.cu).  ntt.cu wraps each body
// in a kernel of its own; the persistent batch kernel (persist.cu) calls the
// same bodies for its work items.  A body takes its CTA's range of task
// chunks (or of tasks) explicitly and its shared-memory scratch as pointers,
// so both callers lay out shared memory as they need.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include "gf128.cuh"
#include "t16.cuh"
#include "t8.cuh"

namespace bz {

struct TablePassArgs {
    const uint4 *src;   // message (first pass) or codeword
    uint4 *dst;         // codeword
    const uint4 *tw;    // twiddle heap
    int ell;            // k_code
    int layer;          // first layer of this pass
    int log_lanes;
    int src_pos_bits;   // positions are masked to this many bits when reading src
    uint64_t n_tasks;
    uint64_t task_base; // first task (restricts the pass to a range of positions)
};

// Twiddles of the blocks a CTA visits, staged in shared memory kTwWindow
// blocks at a time by all threads, so a table rebuild at a block boundary
// reads them from shared memory instead of waiting on one thread's global
// loads.  win[0], win[1] = first staged block and count (set by thread 0 after
// a barrier); NT = 3 stages (t_o, t_a, t_b) per block, NT = 1 stages t.
constexpr int kTwWindow = 64;
template <int NT>
__device__ __forceinline__ const uint4 *tw_window(const uint4 *tw, int layer, uint64_t B,
                                                  uint64_t b_last, uint4 *buf, uint64_t *win) {
    uint64_t b0 = win[0];
    const uint64_t n0 = win[1];
    if (B >= b0 + n0) {  // uniform: every thread read the same win[] after a barrier
        const uint64_t n = min((uint64_t)kTwWindow, b_last + 1 - B);
        for (uint64_t j = threadIdx.x; j < n * NT; j += blockDim.x) {
            const uint64_t b = B + j / NT;
            const int w = (int)(j % NT);
            buf[j] = w == 0 ? tw[((uint64_t)1 << layer) + b]
                            : tw[((uint64_t)1 << (layer + 1)) + 2 * b + (uint64_t)(w - 1)];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            win[0] = B;
            win[1] = n;
        }
        b0 = B;
    }
    return buf + (B - b0) * NT;
}

// LAYERS = 2: radix-4 quad (a, b, c, d) at positions B*4Q + g*Q + rr:
//   layer l   : (a,c), (b,d) with t_o = twiddle(l, B)
//   layer l+1 : (a,b) with t_a = twiddle(l+1, 2B), (c,d) with t_b = twiddle(l+1, 2B+1)
// (the fused 2-layer row op of additive_ntt_f128.rs:829-857, equal to the two
// single layers applied in order).
// LAYERS = 1: pair (p, p+H) at layer l with t = twiddle(l, B).
//
// Body: task chunks [c_beg, c_end) of blockDim.x tasks each; smem holds the
// byte tables and their bases (table_smem bytes), tw_buf kTwWindow * NT
// twiddles, win two words and tz three.
template <int LAYERS>
__device__ __forceinline__ void table_pass_body(const TablePassArgs &a, uint64_t c_beg,
                                                uint64_t c_end, uint4 *smem, uint4 *tw_buf,
                                                uint64_t *win, int *tz) {
    constexpr int NT = LAYERS == 2 ? 3 : 1;
    uint4 *tbl = smem;
    uint4 *bases = smem + NT * kT16Entries;
    if (threadIdx.x == 0) win[0] = win[1] = 0;

    T16Lane lane_ctx;
    lane_ctx.init();

    const int log_q = a.ell - a.layer - LAYERS;  // log2 of the pair/quad stride
    const int log_task_per_b = log_q + a.log_lanes;
    const uint64_t lanes_mask = ((uint64_t)1 << a.log_lanes) - 1;
    const uint64_t q_mask = ((uint64_t)1 << log_q) - 1;
    const uint64_t src_mask = ((uint64_t)1 << a.src_pos_bits) - 1;

    const uint64_t b_last = (a.task_base + c_end * blockDim.x - 1) >> log_task_per_b;
    int64_t cur_b = -1;

    for (uint64_t c = c_beg; c < c_end; ++c) {
        const uint64_t task = a.task_base + c * blockDim.x + threadIdx.x;
        const uint64_t B = task >> log_task_per_b;  // uniform across the CTA
        if ((int64_t)B != cur_b) {
            __syncthreads();
            const uint4 *ts = tw_window<NT>(a.tw, a.layer, B, b_last, tw_buf, win);
            if (threadIdx.x < NT) tz[threadIdx.x] = gf_is_zero(ts[threadIdx.x]);
            t16_build(tbl, bases, ts, NT);  // its barriers publish tz
            cur_b = (int64_t)B;
        }
        const uint64_t rr = (task >> a.log_lanes) & q_mask;
        const uint64_t ln = task & lanes_mask;
        const char *T0 = reinterpret_cast<const char *>(tbl);
        if (LAYERS == 2) {
            uint64_t p[4];
#pragma unroll
            for (int g = 0; g < 4; ++g)
                p[g] = (B << (log_q + 2)) + ((uint64_t)g << log_q) + rr;
            uint4 v[4];
#pragma unroll
            for (int g = 0; g < 4; ++g)
                v[g] = __ldcs(a.src + (((p[g] & src_mask) << a.log_lanes) | ln));
            const char *T1 = T0 + kT16Entries * 16, *T2 = T1 + kT16Entries * 16;
            if (!tz[0]) {
                v[0] = gf_add(v[0], lane_ctx.mul(T0, v[2]));
                v[1] = gf_add(v[1], lane_ctx.mul(T0, v[3]));
            }
            v[2] = gf_add(v[2], v[0]);
            v[3] = gf_add(v[3], v[1]);
            if (!tz[1]) v[0] = gf_add(v[0], lane_ctx.mul(T1, v[1]));
            v[1] = gf_add(v[1], v[0]);
            if (!tz[2]) v[2] = gf_add(v[2], lane_ctx.mul(T2, v[3]));
            v[3] = gf_add(v[3], v[2]);
#pragma unroll
            for (int g = 0; g < 4; ++g) __stcs(a.dst + ((p[g] << a.log_lanes) | ln), v[g]);
        } else {
            const uint64_t p0 = (B << (log_q + 1)) + rr, p1 = p0 + ((uint64_t)1 << log_q);
            uint4 u = __ldcs(a.src + (((p0 & src_mask) << a.log_lanes) | ln));
            uint4 w = __ldcs(a.src + (((p1 & src_mask) << a.log_lanes) | ln));
            if (!tz[0]) u = gf_add(u, lane_ctx.mul(T0, w));
            w = gf_add(w, u);
            __stcs(a.dst + ((p0 << a.log_lanes) | ln), u);
            __stcs(a.dst + ((p1 << a.log_lanes) | ln), w);
        }
    }
}

// ---- Compact tables for narrow twiddles ------------------------------------
// The deepest layers have narrow twiddles (about ell, 2 ell - 3, 4 ell - 11
// bits at depths 0, 1, 2).  For a twiddle t of w bits, a byte x multiplies
// into u[x] = x (x) t, an unreduced carry-less product of w + 7 bits, so one
// 256-entry table of W words (W = 1 for w <= 25, W = 2 for w <= 57) serves
// all 16 byte positions: t * v = reduce(XOR_k u[v_k] << 8k), each shift fixed
// per k.  The table is stored in bank copies (W = 1: 32 copies of 4 B, word
// x * 32 + c; W = 2: 16 copies of 8 B, slot x * 16 + c) and a thread reads
// the copy of its lane, so the lookups of a warp (W = 1) or half-warp (W = 2)
// always hit distinct banks: one wavefront per 32 lookups for W = 1, two for
// W = 2, against four for the 16-byte entries of a byte table; the shifts
// cost a few more ALU operations.  Every compact table is 32 KB.
constexpr int kNwBytes = 32768;

constexpr int narrow_class(int bits) { return bits + 7 <= 32 ? 1 : (bits + 7 <= 64 ? 2 : 4); }

// Build the compact table of t (W words wide) into tb; all threads.  Thread
// pair (x, h) writes half of x's copies, rotated by x, so that every store
// instruction of a warp covers the banks once.
template <int W>
__device__ __forceinline__ void nw_build_item(char *tb, uint64_t t, int u) {
    constexpr int copies = W == 1 ? 32 : 16, half = copies / 2;
    const uint32_t x = (uint32_t)u >> 1, h = (uint32_t)u & 1;
    uint64_t p = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if ((x >> i) & 1) p ^= t << i;
#pragma unroll
    for (int i = 0; i < half; ++i) {
        const uint32_t c = h * half + ((i + x) & (half - 1));
        if (W == 1)
            reinterpret_cast<uint32_t *>(tb)[x * 32 + c] = (uint32_t)p;
        else
            reinterpret_cast<uint2 *>(tb)[x * 16 + c] =
                make_uint2((uint32_t)p, (uint32_t)(p >> 32));
    }
}

template <int W>
__device__ __forceinline__ void nw_build(char *tb, uint64_t t) {
    for (int u = threadIdx.x; u < 512; u += blockDim.x) nw_build_item<W>(tb, t, u);
}

// t * v through the compact table tb of width W.
//
// The lookups of byte position r of the four operand words are gathered
// unshifted into one multi-word value S_r = XOR_q u[byte r of word q] << 32q
// (for W = 1 every word of S_r is a single lookup, for W = 2 neighbouring
// entries overlap by one word), and t * v = reduce(XOR_r S_r << 8r): one
// funnel shift per word and byte position instead of two shifts and two
// xors per lookup, which keeps this ALU-bound multiply off the ALU pipe.
template <int W>
__device__ __forceinline__ uint4 nw_mul(const char *tb, uint4 v) {
    const uint32_t lane_off = W == 1 ? (threadIdx.x & 31) << 2 : (threadIdx.x & 15) << 3;
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    constexpr int NS = W == 1 ? 4 : 5;  // words of S_r
    uint32_t S[4][NS];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            // byte r of word q, times 128 (the row pitch of both layouts)
            const uint32_t x7 = (r == 0 ? (w[q] << 7) : (w[q] >> (8 * r - 7))) & 0x7F80u;
            if constexpr (W == 1) {
                S[r][q] = *reinterpret_cast<const uint32_t *>(tb + (x7 | lane_off));
            } else {
                const uint2 u = *reinterpret_cast<const uint2 *>(tb + (x7 | lane_off));
                if (q == 0) S[r][0] = u.x;
                else S[r][q] ^= u.x;
                S[r][q + 1] = u.y;
            }
        }
    }
    // acc = XOR_r S_r << 8r (NS + 1 words)
    uint32_t acc[6];
#pragma unroll
    for (int k = 0; k <= NS; ++k) {
        uint32_t x = k < NS ? S[0][k] : 0u;
#pragma unroll
        for (int r = 1; r < 4; ++r) {
            const uint32_t hi = k < NS ? S[r][k] : 0u, lo = k > 0 ? S[r][k - 1] : 0u;
            x ^= __funnelshift_l(lo, hi, 8 * r);
        }
        acc[k] = x;
    }
    // bits 128 and up: X^128 = X^7 + X^2 + X + 1.  W = 1: the products have
    // at most 32 bits, so bits 128+ are below 2^24 and the fold stays in one
    // word; W = 2: at most 64-bit products, h < 2^56 and f stays below 2^63,
    // so neither needs a second fold.
    if constexpr (W == 1) {
        const uint32_t h = acc[4];
        const uint32_t f = h ^ (h << 1) ^ (h << 2) ^ (h << 7);
        return make_uint4(acc[0] ^ f, acc[1], acc[2], acc[3]);
    } else {
        const uint64_t h = (uint64_t)acc[4] | ((uint64_t)acc[5] << 32);
        const uint64_t f = h ^ (h << 1) ^ (h << 2) ^ (h << 7);
        return make_uint4(acc[0] ^ (uint32_t)f, acc[1] ^ (uint32_t)(f >> 32), acc[2], acc[3]);
    }
}

// Radix-4 table pass with the next task's four loads issued before the
// current task's multiplies (register double buffering), so global-memory
// latency overlaps the shared-memory lookups.  Each of the three twiddles
// multiplies through its 64 KB byte table (width 4) or, when it is narrow,
// through a compact table of WO (t_o) or WAB (t_a, t_b) words; t_a and t_b
// are one layer deeper than t_o, so WAB <= WO.  Shared memory holds the byte
// tables first (those of t_o, then t_a and t_b when WAB == 4), then their
// basis scratch, then the compact tables.
//
// Body: task chunks [c_beg, c_end) of blockDim.x tasks; smem holds the tables
// (pf_smem bytes), tw_buf 3 * kTwWindow twiddles and win two words.
template <int WO, int WAB>
__device__ __forceinline__ void table_pass2_pf_body(const TablePassArgs &a, uint64_t c_beg,
                                                    uint64_t c_end, uint4 *smem, uint4 *tw_buf,
                                                    uint64_t *win) {
    static_assert(WAB <= WO, "t_a and t_b are never wider than t_o");
    constexpr int NFULL = (WO == 4) + 2 * (WAB == 4);   // byte tables, in order o, a, b
    constexpr int NCOMPACT = 3 - NFULL;
    uint4 *tbl = smem;
    uint4 *bases = smem + NFULL * kT16Entries;
    char *cw = reinterpret_cast<char *>(bases + NFULL * kT16Bases);
    // compact tables in order (o when WO < 4), a, b
    char *cw_o = cw;
    char *cw_a = cw + (WO == 4 ? 0 : kNwBytes);
    char *cw_b = cw_a + kNwBytes;
    const char *T0 = reinterpret_cast<const char *>(tbl);
    const char *T1 = T0 + kT16Entries * 16, *T2 = T1 + kT16Entries * 16;
    if (threadIdx.x == 0) win[0] = win[1] = 0;
    bool z0 = false, z1 = false, z2 = false;  // zero twiddles of the current block
    T16Lane8 lane_ctx;
    if (NFULL) lane_ctx.init();
    const int log_q = a.ell - a.layer - 2;
    const int log_task_per_b = log_q + a.log_lanes;
    const uint64_t lanes_mask = ((uint64_t)1 << a.log_lanes) - 1;
    const uint64_t q_mask = ((uint64_t)1 << log_q) - 1;
    const uint64_t src_mask = ((uint64_t)1 << a.src_pos_bits) - 1;
    const uint64_t b_last = (a.task_base + c_end * blockDim.x - 1) >> log_task_per_b;
    int64_t cur_b = -1;
    auto src_index = [&](uint64_t task, int g) -> uint64_t {
        const uint64_t B = task >> log_task_per_b;
        const uint64_t rr = (task >> a.log_lanes) & q_mask;
        const uint64_t p = (B << (log_q + 2)) + ((uint64_t)g << log_q) + rr;
        return ((p & src_mask) << a.log_lanes) | (task & lanes_mask);
    };
    auto lo64 = [](uint4 t) { return (uint64_t)t.x | ((uint64_t)t.y << 32); };
    uint4 nxt[4];
    if (c_beg < c_end) {
        const uint64_t t0 = a.task_base + c_beg * blockDim.x + threadIdx.x;
#pragma unroll
        for (int g = 0; g < 4; ++g) nxt[g] = __ldcs(a.src + src_index(t0, g));
    }
    for (uint64_t c = c_beg; c < c_end; ++c) {
        const uint64_t task = a.task_base + c * blockDim.x + threadIdx.x;
        const uint64_t B = task >> log_task_per_b;  // uniform across the CTA
        uint4 v[4];
#pragma unroll
        for (int g = 0; g < 4; ++g) v[g] = nxt[g];
        if (c + 1 < c_end) {
            const uint64_t tn = task + blockDim.x;
#pragma unroll
            for (int g = 0; g < 4; ++g) nxt[g] = __ldcs(a.src + src_index(tn, g));
        }
        if ((int64_t)B != cur_b) {
            __syncthreads();
            const uint4 *ts = tw_window<3>(a.tw, a.layer, B, b_last, tw_buf, win);
            z0 = gf_is_zero(ts[0]);
            z1 = gf_is_zero(ts[1]);
            z2 = gf_is_zero(ts[2]);
            if constexpr (NFULL > 0) t16_build(tbl, bases, ts, NFULL);  // syncs inside
            if constexpr (WO < 4) nw_build<WO>(cw_o, lo64(ts[0]));
            if constexpr (WAB < 4) {
                nw_build<WAB>(cw_a, lo64(ts[1]));
                nw_build<WAB>(cw_b, lo64(ts[2]));
            }
            if constexpr (NCOMPACT > 0) __syncthreads();
            cur_b = (int64_t)B;
        }
        if (!z0) {
            if constexpr (WO == 4) {
                v[0] = gf_add(v[0], lane_ctx.mul(T0, v[2]));
                v[1] = gf_add(v[1], lane_ctx.mul(T0, v[3]));
            } else {
                v[0] = gf_add(v[0], nw_mul<WO>(cw_o, v[2]));
                v[1] = gf_add(v[1], nw_mul<WO>(cw_o, v[3]));
            }
        }
        v[2] = gf_add(v[2], v[0]);
        v[3] = gf_add(v[3], v[1]);
        if constexpr (WAB == 4) {
            if (!z1) v[0] = gf_add(v[0], lane_ctx.mul(T1, v[1]));
            v[1] = gf_add(v[1], v[0]);
            if (!z2) v[2] = gf_add(v[2], lane_ctx.mul(T2, v[3]));
        } else {
            if (!z1) v[0] = gf_add(v[0], nw_mul<WAB>(cw_a, v[1]));
            v[1] = gf_add(v[1], v[0]);
            if (!z2) v[2] = gf_add(v[2], nw_mul<WAB>(cw_b, v[3]));
        }
        v[3] = gf_add(v[3], v[2]);
        const uint64_t rr = (task >> a.log_lanes) & q_mask;
        const uint64_t ln = task & lanes_mask;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const uint64_t p = (B << (log_q + 2)) + ((uint64_t)g << log_q) + rr;
            __stcs(a.dst + ((p << a.log_lanes) | ln), v[g]);
        }
    }
}

// ---- Radix-8 passes ---------------------------------------------------------
// Layers l, l+1, l+2 on octets at positions B*8Q + g*Q + rr (g = 0..7),
// Q = 2^(ell - l - 3):
//   layer l  : pairs (g, g+4), g < 4, with twiddle(l, B)
//   layer l+1: (0,2), (1,3) with twiddle(l+1, 2B); (4,6), (5,7) with
//              twiddle(l+1, 2B+1)
//   layer l+2: (2j, 2j+1) with twiddle(l+2, 4B+j), j < 4
// i.e. the three single layers of additive_ntt_f128.rs:243-274 applied in
// order (u <- u + t*v; v <- v + u), twelve multiplies per octet.  The seven
// twiddles of a block B multiply through 32 KB tables each (224 KB): eight
// byte tables of 16-byte entries (t8.cuh, width 4) or, for a narrow twiddle,
// the compact one- or two-word table (width 1 or 2).  One sweep over the
// codeword does three layers where the 64 KB radix-4 tables allow two.
constexpr int kTw8Window = 8;
constexpr int kPass8Smem = 7 * kT8Bytes;

__device__ __forceinline__ uint4 tw8_at(const uint4 *tw, int layer, uint64_t B, int j) {
    if (j == 0) return tw[((uint64_t)1 << layer) + B];
    if (j < 3) return tw[((uint64_t)1 << (layer + 1)) + 2 * B + (uint64_t)(j - 1)];
    return tw[((uint64_t)1 << (layer + 2)) + 4 * B + (uint64_t)(j - 3)];
}

// Table-build work items per twiddle: 128 for the byte tables (t8_build_item),
// 512 for a compact table (nw_build_item).
template <int W>
constexpr int build_items() { return W == 4 ? 128 : 512; }

template <int W>
__device__ __forceinline__ void build_item(char *tb, uint4 t, int u) {
    if constexpr (W == 4) t8_build_item(tb, t, u);
    else nw_build_item<W>(tb, (uint64_t)t.x | ((uint64_t)t.y << 32), u);
}

template <int W>
__device__ __forceinline__ uint4 pass_mul(const T8Lane &lc, const char *tb, uint4 v) {
    if constexpr (W == 4) return lc.mul(tb, v);
    else return nw_mul<W>(tb, v);
}

//
// Body: task chunks [c_beg, c_end) of blockDim.x tasks; tbl holds the seven
// tables (kPass8Smem bytes), tw_buf kTw8Window * 7 twiddles, win two words.
template <int W0, int W1, int W2>
__device__ __forceinline__ void pass8_body(const TablePassArgs &a, uint64_t c_beg, uint64_t c_end,
                                           char *tbl, uint4 *tw_buf, uint64_t *win) {
    if (threadIdx.x == 0) win[0] = win[1] = 0;
    T8Lane lc;
    lc.init();
    const int log_q = a.ell - a.layer - 3;
    const int log_task_per_b = log_q + a.log_lanes;
    const uint64_t lanes_mask = ((uint64_t)1 << a.log_lanes) - 1;
    const uint64_t q_mask = ((uint64_t)1 << log_q) - 1;
    const uint64_t src_mask = ((uint64_t)1 << a.src_pos_bits) - 1;
    const uint64_t b_last = (a.task_base + c_end * blockDim.x - 1) >> log_task_per_b;
    int64_t cur_b = -1;
    uint32_t zmask = 0;  // zero twiddles of the current block
    constexpr int n0 = build_items<W0>(), n1 = build_items<W1>(), n2 = build_items<W2>();
    constexpr int n_items = n0 + 2 * n1 + 4 * n2;
    for (uint64_t c = c_beg; c < c_end; ++c) {
        const uint64_t task = a.task_base + c * blockDim.x + threadIdx.x;
        const uint64_t B = task >> log_task_per_b;  // uniform across the CTA
        if ((int64_t)B != cur_b) {
            __syncthreads();  // every lookup into the previous block's tables is done
            uint64_t b0 = win[0];
            if (B >= b0 + win[1]) {  // uniform: all threads read win[] after a barrier
                const uint64_t n = min((uint64_t)kTw8Window, b_last + 1 - B);
                for (uint64_t j = threadIdx.x; j < n * 7; j += blockDim.x)
                    tw_buf[j] = tw8_at(a.tw, a.layer, B + j / 7, (int)(j % 7));
                __syncthreads();
                if (threadIdx.x == 0) {
                    win[0] = B;
                    win[1] = n;
                }
                b0 = B;
            }
            const uint4 *ts = tw_buf + (B - b0) * 7;
            zmask = 0;
#pragma unroll
            for (int j = 0; j < 7; ++j) zmask |= gf_is_zero(ts[j]) ? (1u << j) : 0u;
            for (int u = threadIdx.x; u < n_items; u += blockDim.x) {
                if (u < n0) {
                    build_item<W0>(tbl, ts[0], u);
                } else if (u < n0 + 2 * n1) {
                    const int k = (u - n0) / n1;
                    build_item<W1>(tbl + (1 + k) * kT8Bytes, ts[1 + k], (u - n0) - k * n1);
                } else {
                    const int k = (u - n0 - 2 * n1) / n2;
                    build_item<W2>(tbl + (3 + k) * kT8Bytes, ts[3 + k], (u - n0 - 2 * n1) - k * n2);
                }
            }
            __syncthreads();
            cur_b = (int64_t)B;
        }
        const uint64_t rr = (task >> a.log_lanes) & q_mask;
        const uint64_t ln = task & lanes_mask;
        const uint64_t pbase = (B << (log_q + 3)) + rr;
        uint4 v[8];
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const uint64_t p = pbase + ((uint64_t)g << log_q);
            v[g] = __ldcs(a.src + (((p & src_mask) << a.log_lanes) | ln));
        }
        if (!(zmask & 1)) {
#pragma unroll
            for (int g = 0; g < 4; ++g) v[g] = gf_add(v[g], pass_mul<W0>(lc, tbl, v[g + 4]));
        }
#pragma unroll
        for (int g = 0; g < 4; ++g) v[g + 4] = gf_add(v[g + 4], v[g]);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const char *tb = tbl + (1 + h) * kT8Bytes;
            uint4 &x0 = v[4 * h], &x1 = v[4 * h + 1], &x2 = v[4 * h + 2], &x3 = v[4 * h + 3];
            if (!(zmask & (2u << h))) {
                x0 = gf_add(x0, pass_mul<W1>(lc, tb, x2));
                x1 = gf_add(x1, pass_mul<W1>(lc, tb, x3));
            }
            x2 = gf_add(x2, x0);
            x3 = gf_add(x3, x1);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const char *tb = tbl + (3 + j) * kT8Bytes;
            if (!(zmask & (8u << j))) v[2 * j] = gf_add(v[2 * j], pass_mul<W2>(lc, tb, v[2 * j + 1]));
            v[2 * j + 1] = gf_add(v[2 * j + 1], v[2 * j]);
        }
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const uint64_t p = pbase + ((uint64_t)g << log_q);
            __stcs(a.dst + ((p << a.log_lanes) | ln), v[g]);
        }
    }
}

struct DeepArgs {
    const uint4 *src;
    uint4 *dst;
    const uint4 *tw;
    int ell;
    int log_lanes;
    int src_pos_bits;
    uint64_t n_tasks;  // 2^(ell - D) * L
    uint64_t task_base;
};

// The narrow layers (depth < D) of one group of 2^D consecutive positions
// held in registers: layer ell-D+j has 2^j sub-blocks with block index
// (G << j) | sb (twiddles warp-uniform when the warp shares G).
template <int D, int P, int MODE>
__device__ __forceinline__ void narrow_layers(uint4 (&v)[P], const uint4 *tw, int ell,
                                              uint64_t G) {
    constexpr int PS = P >> D;  // groups of 2^D inside v (1 for the deep pass)
#pragma unroll
    for (int j = 0; j < D; ++j) {
        const int l = ell - D + j;
        const int half = (1 << D) >> (j + 1);
#pragma unroll
        for (int g = 0; g < PS; ++g) {
#pragma unroll
            for (int sb = 0; sb < (1 << j); ++sb) {
                const uint64_t B = (((G * PS + g)) << j) | (uint64_t)sb;
                const uint4 t = tw[((uint64_t)1 << l) + B];
                const bool tz = gf_is_zero(t);
#pragma unroll
                for (int i = 0; i < half; ++i) {
                    uint4 &u = v[g * (1 << D) + sb * 2 * half + i];
                    uint4 &w = v[g * (1 << D) + sb * 2 * half + i + half];
                    if (!tz) u = gf_add(u, gf_mul_narrow_m<MODE>(w, t));
                    w = gf_add(w, u);
                }
            }
        }
    }
}

// Last D layers on 2^D consecutive positions per thread (one lane).
// Body: tasks it = first, first + step, .. below end (a thread's own first).
template <int D, int MODE>
__device__ __forceinline__ void deep_pass_body(const DeepArgs &a, uint64_t first, uint64_t end,
                                               uint64_t step) {
    constexpr int P = 1 << D;
    const uint64_t lanes_mask = ((uint64_t)1 << a.log_lanes) - 1;
    const uint64_t src_mask = ((uint64_t)1 << a.src_pos_bits) - 1;
    for (uint64_t it = first; it < end; it += step) {
        const uint64_t task = a.task_base + it;
        const uint64_t G = task >> a.log_lanes;
        const uint64_t ln = task & lanes_mask;
        uint4 v[P];
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const uint64_t pos = (G << D) + i;
            v[i] = __ldcs(a.src + (((pos & src_mask) << a.log_lanes) | ln));
        }
        narrow_layers<D, P, MODE>(v, a.tw, a.ell, G);
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const uint64_t pos = (G << D) + i;
            __stcs(a.dst + ((pos << a.log_lanes) | ln), v[i]);
        }
    }
}

// One layer, generic multiply: the reference path and the fallback for
// shapes too small for the table passes.
// Body: tasks first, first + step, .. below end.
__device__ __forceinline__ void generic_layer_body(const uint4 *src, uint4 *dst, const uint4 *tw,
                                                   int ell, int layer, int log_lanes,
                                                   int src_pos_bits, uint64_t first,
                                                   uint64_t end, uint64_t step) {
    const int log_h = ell - layer - 1;
    const uint64_t lanes_mask = ((uint64_t)1 << log_lanes) - 1;
    const uint64_t src_mask = ((uint64_t)1 << src_pos_bits) - 1;
    for (uint64_t task = first; task < end; task += step) {
        const uint64_t ln = task & lanes_mask;
        const uint64_t pair = task >> log_lanes;
        const uint64_t B = pair >> log_h, rr = pair & (((uint64_t)1 << log_h) - 1);
        const uint64_t p0 = (B << (log_h + 1)) + rr, p1 = p0 + ((uint64_t)1 << log_h);
        const uint4 t = tw[((uint64_t)1 << layer) + B];
        uint4 u = src[((p0 & src_mask) << log_lanes) | ln];
        uint4 w = src[((p1 & src_mask) << log_lanes) | ln];
        u = gf_add(u, gf_mul(w, t));
        w = gf_add(w, u);
        dst[(p0 << log_lanes) | ln] = u;
        dst[(p1 << log_lanes) | ln] = w;
    }
}

// ---- host-side sizes and limits of the bodies above -------------------------
// Every CTA chunk (512 tasks) of a table pass must lie inside one block B.
constexpr bool table_pass_ok(int ell, int layer, int layers, int log_lanes, int log_threads = 9) {
    const int log_task_per_b = ell - layer - layers + log_lanes;
    return log_task_per_b >= log_threads;
}

// Dynamic shared memory of table_pass_body<LAYERS> (tables and bases).
constexpr size_t table_smem(int layers) {
    const int nt = layers == 2 ? 3 : 1;
    return (size_t)nt * kT16Entries * 16 + (size_t)nt * kT16Bases * 16;
}

// Dynamic shared memory of table_pass2_pf_body<WO, WAB>.
constexpr size_t pf_smem(int wo, int wab) {
    const int nfull = (wo == 4) + 2 * (wab == 4);
    return (size_t)nfull * (kT16Entries + kT16Bases) * 16 + (size_t)(3 - nfull) * kNwBytes;
}

}  // namespace bz
