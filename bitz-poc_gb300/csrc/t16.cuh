// Multiply by a block-constant GF(2^128) element through byte tables in
// shared memory (used by the NTT table passes and the sumcheck folds).
//
// For a constant t, table k (byte position k = 0..15 of the operand) holds
// T_k[x] = x * X^(8k) * t for every byte value x, so t * v = XOR_k T_k[v_k]:
// 16 lookups of 16 bytes.  The 16 tables (64 KB) are laid out so byte
// position k lives in bank group k mod 8, and each thread walks the byte
// positions in an order rotated by (thread index mod 8): the 8 threads of a
// quarter-warp always read 8 different bank groups, so the 128-bit lookups
// are bank-conflict free.
#pragma once
#include <stdint.h>

#include "gf128.cuh"

namespace bz {

constexpr int kT16Entries = 4096;  // 16 byte positions x 256 values
// Scratch per twiddle for the 128 basis products t * X^e: groups of 8 (one
// byte position) padded to 9 entries, so threads that read the same basis of
// different byte positions hit different bank groups.
constexpr int kT16Bases = 16 * 9;

// Byte offset of entry (k, x) inside one table.
__device__ __forceinline__ uint32_t t16_off(uint32_t k, uint32_t x) {
    return ((k >> 3) << 15) + (x << 7) + ((k & 7) << 4);
}

// Expand 128 basis images per table (bases[i * kT16Bases + (e >> 3) * 9 +
// (e & 7)] = image of bit e) into the byte tables tbl[i * 4096 ..]: T_k[x] =
// XOR of the images of the set bits of x at byte position k.  Called by all
// threads; syncs at the end.  Thread u builds the 16 entries (k, hi * 16 + lo)
// of byte position k = u mod 16: the 8 threads of a quarter-warp take 8
// different byte positions, so both their basis reads and their table writes
// fall in 8 different bank groups.
static __device__ __noinline__ void t16_expand(uint4 *tbl, const uint4 *bases, int n_tw) {
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int u = tid; u < 256 * n_tw; u += nthr) {
        const int i = u >> 8, k = u & 15, hi = (u >> 4) & 15;
        const uint4 *b = bases + i * kT16Bases + 9 * k;
        uint4 H = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if ((hi >> q) & 1) H = gf_add(H, b[4 + q]);
        uint4 L[16];
        L[0] = make_uint4(0, 0, 0, 0);
        const uint4 b0 = b[0], b1 = b[1], b2 = b[2], b3 = b[3];
#pragma unroll
        for (int x = 1; x < 16; ++x) {
            const int low = x & -x;
            const uint4 bb = low == 1 ? b0 : low == 2 ? b1 : low == 4 ? b2 : b3;
            L[x] = gf_add(L[x & (x - 1)], bb);
        }
        char *tb = reinterpret_cast<char *>(tbl + (size_t)i * kT16Entries);
#pragma unroll
        for (int lo = 0; lo < 16; ++lo)
            *reinterpret_cast<uint4 *>(tb + t16_off(k, (hi << 4) | lo)) = gf_add(H, L[lo]);
    }
    __syncthreads();
}

// Tables of multiplication by each twiddle ts[i] (the image of bit e is
// ts[i] * X^e).  `bases` is kT16Bases * n_tw uint4 of scratch.  Called by all
// threads; syncs inside.
static __device__ __noinline__ void t16_build(uint4 *tbl, uint4 *bases, const uint4 *ts, int n_tw) {
    for (int j = threadIdx.x; j < 128 * n_tw; j += blockDim.x) {
        const int i = j >> 7, e = j & 127;
        bases[i * kT16Bases + (e >> 3) * 9 + (e & 7)] = gf_mul_xpow(ts[i], (uint32_t)e);
    }
    __syncthreads();
    t16_expand(tbl, bases, n_tw);
}

// Per-thread lookup offsets: step m reads byte position (m + s) mod 16.
struct T16Lane {
    uint32_t off[16];
    uint32_t s;
    __device__ __forceinline__ void init() {
        s = threadIdx.x & 7;
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            const uint32_t k = (m + s) & 15;
            off[m] = ((k >> 3) << 15) + ((k & 7) << 4);
        }
    }
    // v rotated right by 8*s bits: byte m of the result is byte (m+s)&15 of v.
    __device__ __forceinline__ uint4 rot(uint4 v) const {
        uint4 r = (s & 4) ? make_uint4(v.y, v.z, v.w, v.x) : v;
        const uint32_t sh = (s & 3) << 3;
        return make_uint4(__funnelshift_r(r.x, r.y, sh), __funnelshift_r(r.y, r.z, sh),
                          __funnelshift_r(r.z, r.w, sh), __funnelshift_r(r.w, r.x, sh));
    }
    __device__ __forceinline__ uint4 mul(const char *tb, uint4 v) const {
        const uint4 vr = rot(v);
        uint4 acc = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            const uint32_t w = (m < 4) ? vr.x : (m < 8) ? vr.y : (m < 12) ? vr.z : vr.w;
            const uint32_t x = __byte_perm(w, 0u, 0x4440u | (uint32_t)(m & 3));
            const uint4 e = *reinterpret_cast<const uint4 *>(tb + (x << 7) + off[m]);
            acc = gf_add(acc, e);
        }
        return acc;
    }
};

// Same lookups with 8 offset registers: byte positions m and m + 8 differ only
// in the table half, so off[m + 8] = off[m] ^ (1 << 15).
struct T16Lane8 {
    uint32_t off[8];
    uint32_t s;
    __device__ __forceinline__ void init() {
        s = threadIdx.x & 7;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const uint32_t k = (m + s) & 15;
            off[m] = ((k >> 3) << 15) + ((k & 7) << 4);
        }
    }
    __device__ __forceinline__ uint4 rot(uint4 v) const {
        uint4 r = (s & 4) ? make_uint4(v.y, v.z, v.w, v.x) : v;
        const uint32_t sh = (s & 3) << 3;
        return make_uint4(__funnelshift_r(r.x, r.y, sh), __funnelshift_r(r.y, r.z, sh),
                          __funnelshift_r(r.z, r.w, sh), __funnelshift_r(r.w, r.x, sh));
    }
    __device__ __forceinline__ uint4 mul(const char *tb, uint4 v) const {
        const uint4 vr = rot(v);
        uint4 acc = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int m = 0; m < 16; ++m) {
            const uint32_t w = (m < 4) ? vr.x : (m < 8) ? vr.y : (m < 12) ? vr.z : vr.w;
            const uint32_t x = __byte_perm(w, 0u, 0x4440u | (uint32_t)(m & 3));
            const uint32_t o = m < 8 ? off[m] : (off[m - 8] ^ 0x8000u);
            const uint4 e = *reinterpret_cast<const uint4 *>(tb + (x << 7) + o);
            acc = gf_add(acc, e);
        }
        return acc;
    }
};

}  // namespace bz
