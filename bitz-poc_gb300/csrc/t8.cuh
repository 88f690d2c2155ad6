// Multiply by a block-constant GF(2^128) element through eight byte tables in
// shared memory (32 KB per constant), used by the radix-8 NTT passes.
//
// For a constant t, table s (s = 0..7) holds T_s[x] = x * X^(8s) * t for every
// byte value x, so a 64-bit operand w times t is XOR_s T_s[byte s of w]: 8
// lookups of 16 bytes.  A 128-bit operand v = lo + X^64 hi takes 16 lookups,
// S_lo = lo * t and S_hi = hi * t through the same eight tables, and
// t * v = S_lo + X^64 S_hi, where the high word h1 of S_hi folds down once by
// X^128 = X^7 + X^2 + X + 1.  Half the memory of one table per byte position
// of the operand (64 KB) for the same lookups, so the seven twiddles of a
// radix-8 pass fit in shared memory.
//
// Layout: row x (128 bytes) holds T_0[x] .. T_7[x], so table s lives in bank
// group s.  Each thread walks the byte positions in an order rotated by
// (thread index mod 8): the 8 threads of a quarter-warp read 8 different
// bank groups at every step, so the 128-bit lookups are conflict free.
#pragma once
#include <stdint.h>

#include "gf128.cuh"

namespace bz {

constexpr int kT8Bytes = 32768;  // 256 rows x 8 entries x 16 bytes

// t * X for t in GF(2^128).
BZ_HD uint4 gf_mul_x(uint4 t) {
    const uint32_t c = t.w >> 31;
    uint4 r = make_uint4(t.x << 1, __funnelshift_l(t.x, t.y, 1), __funnelshift_l(t.y, t.z, 1),
                         __funnelshift_l(t.z, t.w, 1));
    r.x ^= c * 0x87u;
    return r;
}

// Work item u (0 .. 127) of the table of t: byte position s = u mod 8 and the
// high nibble hi = u / 8 of the byte value; writes the 16 entries
// (hi * 16 + lo, s).  The 8 threads of a quarter-warp take 8 different byte
// positions, so their stores fall in 8 different bank groups.
__device__ __forceinline__ void t8_build_item(char *tb, uint4 t, int u) {
    const int s = u & 7, hi = (u >> 3) & 15;
    uint4 b[8];
    b[0] = gf_mul_xpow(t, (uint32_t)(8 * s));
#pragma unroll
    for (int e = 1; e < 8; ++e) b[e] = gf_mul_x(b[e - 1]);
    uint4 H = make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if ((hi >> q) & 1) H = gf_add(H, b[4 + q]);
    uint4 L[16];
    L[0] = make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int x = 1; x < 16; ++x) {
        const int low = x & -x;
        const uint4 bb = low == 1 ? b[0] : low == 2 ? b[1] : low == 4 ? b[2] : b[3];
        L[x] = gf_add(L[x & (x - 1)], bb);
    }
#pragma unroll
    for (int lo = 0; lo < 16; ++lo)
        *reinterpret_cast<uint4 *>(tb + ((hi << 4) | lo) * 128 + s * 16) = gf_add(H, L[lo]);
}

// Per-thread lookup order: step m reads byte position (m + r) mod 8, r =
// thread index mod 8.
struct T8Lane {
    uint32_t off[8];
    uint32_t r;
    __device__ __forceinline__ void init() {
        r = threadIdx.x & 7;
#pragma unroll
        for (int m = 0; m < 8; ++m) off[m] = ((m + r) & 7) << 4;
    }
    // (a, b) as a 64-bit value rotated right by 8r bits: byte m of the result
    // is byte (m + r) mod 8 of the input.
    __device__ __forceinline__ void rot(uint32_t &a, uint32_t &b) const {
        uint32_t x = (r & 4) ? b : a, y = (r & 4) ? a : b;
        const uint32_t sh = (r & 3) << 3;
        a = __funnelshift_r(x, y, sh);
        b = __funnelshift_r(y, x, sh);
    }
    __device__ __forceinline__ uint4 mul(const char *tb, uint4 v) const {
        uint32_t l0 = v.x, l1 = v.y, h0 = v.z, h1 = v.w;
        rot(l0, l1);
        rot(h0, h1);
        uint4 A = make_uint4(0, 0, 0, 0), B = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const uint32_t wl = m < 4 ? l0 : l1, wh = m < 4 ? h0 : h1;
            const uint32_t sel = 0x4440u | (uint32_t)(m & 3);
            const uint32_t xl = __byte_perm(wl, 0u, sel), xh = __byte_perm(wh, 0u, sel);
            A = gf_add(A, *reinterpret_cast<const uint4 *>(tb + (xl << 7) + off[m]));
            B = gf_add(B, *reinterpret_cast<const uint4 *>(tb + (xh << 7) + off[m]));
        }
        // A + X^64 B: B's low word moves up, its high word g1 folds by X^128 = g
        const uint64_t g1 = (uint64_t)B.z | ((uint64_t)B.w << 32);
        const uint64_t f_lo = g1 ^ (g1 << 1) ^ (g1 << 2) ^ (g1 << 7);
        const uint64_t f_hi = (g1 >> 63) ^ (g1 >> 62) ^ (g1 >> 57);
        return make_uint4(A.x ^ (uint32_t)f_lo, A.y ^ (uint32_t)(f_lo >> 32),
                          A.z ^ B.x ^ (uint32_t)f_hi, A.w ^ B.y);
    }
};

}  // namespace bz
