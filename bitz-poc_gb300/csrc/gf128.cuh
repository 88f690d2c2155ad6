// Device arithmetic in GF(2^128) with X^128 = X^7 + X^2 + X + 1
// (vendor/field/src/gf128.rs:80-96).  An element is a uint4 holding the four
// little-endian 32-bit words of the reference's {lo: u64, hi: u64}.
//
// GB300 has no carry-less multiply instruction, so three multiply forms exist:
//  * gf_mul: variable x variable.  Karatsuba down to 32x32 carry-less products,
//    each computed on the integer multiplier with four interleaved residue
//    classes (bits i = c mod 4), which keeps every partial count below 16 so
//    no carry crosses a 4-bit lane; XOR of the class products keeps parity.
//  * mul_narrow: variable x warp-uniform constant of few bits (the deep NTT
//    layers' twiddles): shift-and-XOR over the constant's set bits.
//  * byte tables (ntt.cu / fold.cu): variable x block-constant, 16 lookups of a
//    per-constant 64 KB shared-memory table.
#pragma once
#include <stdint.h>

#define BZ_HD __device__ __forceinline__

BZ_HD uint4 gf_add(uint4 a, uint4 b) {
    return make_uint4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w);
}
BZ_HD bool gf_is_zero(uint4 a) { return (a.x | a.y | a.z | a.w) == 0; }

// 32x32 -> 64 carry-less product on the integer multiplier.  Class k of the
// result collects the products a_i * b_j with i + j = k (mod 4).  One product
// of classes (i, j) puts at most 8 partial bits on a result bit.  Two products
// whose i + j differ by 4 put at most 15 there (8 + 7, checked over every
// position), so such a pair is summed by the multiply-add itself: one XOR
// fewer per pair.
BZ_HD uint64_t clmul32(uint32_t a, uint32_t b) {
    const uint32_t M = 0x11111111u;
    const uint32_t a0 = a & M, a1 = a & (M << 1), a2 = a & (M << 2), a3 = a & (M << 3);
    const uint32_t b0 = b & M, b1 = b & (M << 1), b2 = b & (M << 2), b3 = b & (M << 3);
    auto p = [](uint32_t x, uint32_t y) -> uint64_t { return (uint64_t)x * (uint64_t)y; };
    const uint64_t z0 = (p(a0, b0) + p(a1, b3)) ^ p(a2, b2) ^ p(a3, b1);
    const uint64_t z1 = (p(a0, b1) + p(a2, b3)) ^ (p(a1, b0) + p(a3, b2));
    const uint64_t z2 = (p(a0, b2) + p(a3, b3)) ^ p(a1, b1) ^ p(a2, b0);
    const uint64_t z3 = p(a0, b3) ^ p(a1, b2) ^ p(a2, b1) ^ p(a3, b0);
    const uint64_t W = 0x1111111111111111ull;
    return (z0 & W) | (z1 & (W << 1)) | (z2 & (W << 2)) | (z3 & (W << 3));
}

// 64x64 -> 128 (Karatsuba over 32-bit halves), result as (lo, hi).
BZ_HD void clmul64(uint64_t a, uint64_t b, uint64_t &lo, uint64_t &hi) {
    const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32);
    const uint32_t b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
    const uint64_t l = clmul32(a0, b0);
    const uint64_t h = clmul32(a1, b1);
    const uint64_t m = clmul32(a0 ^ a1, b0 ^ b1) ^ l ^ h;
    lo = l ^ (m << 32);
    hi = h ^ (m >> 32);
}

// Unreduced 256-bit product, words little-endian.
struct gf_wide {
    uint64_t w[4];
};
BZ_HD gf_wide gf_wide_zero() {
    gf_wide r;
    r.w[0] = r.w[1] = r.w[2] = r.w[3] = 0;
    return r;
}
BZ_HD void gf_wide_xor(gf_wide &acc, const gf_wide &x) {
    acc.w[0] ^= x.w[0];
    acc.w[1] ^= x.w[1];
    acc.w[2] ^= x.w[2];
    acc.w[3] ^= x.w[3];
}

BZ_HD uint64_t lo64(uint4 a) { return (uint64_t)a.x | ((uint64_t)a.y << 32); }
BZ_HD uint64_t hi64(uint4 a) { return (uint64_t)a.z | ((uint64_t)a.w << 32); }
BZ_HD uint4 mk(uint64_t lo, uint64_t hi) {
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// 128x128 -> 256 (Karatsuba over 64-bit halves).
BZ_HD gf_wide gf_mul_wide(uint4 a, uint4 b) {
    const uint64_t a0 = lo64(a), a1 = hi64(a), b0 = lo64(b), b1 = hi64(b);
    uint64_t l0, l1, h0, h1, m0, m1;
    clmul64(a0, b0, l0, l1);
    clmul64(a1, b1, h0, h1);
    clmul64(a0 ^ a1, b0 ^ b1, m0, m1);
    m0 ^= l0 ^ h0;
    m1 ^= l1 ^ h1;
    gf_wide r;
    r.w[0] = l0;
    r.w[1] = l1 ^ m0;
    r.w[2] = h0 ^ m1;
    r.w[3] = h1;
    return r;
}

// Reduce modulo X^128 + X^7 + X^2 + X + 1: the high 128 bits H fold down as
// H*g, and the <= 7 bits of H*g above X^128 fold once more.
BZ_HD uint4 gf_reduce(const gf_wide &r) {
    const uint64_t h0 = r.w[2], h1 = r.w[3];
    const uint64_t f0 = h0 ^ (h0 << 1) ^ (h0 << 2) ^ (h0 << 7);
    const uint64_t f1 = h1 ^ (h1 << 1) ^ (h1 << 2) ^ (h1 << 7) ^ (h0 >> 63) ^ (h0 >> 62) ^
                        (h0 >> 57);
    const uint64_t spill = (h1 >> 63) ^ (h1 >> 62) ^ (h1 >> 57);
    const uint64_t lo = r.w[0] ^ f0 ^ spill ^ (spill << 1) ^ (spill << 2) ^ (spill << 7);
    const uint64_t hi = r.w[1] ^ f1;
    return mk(lo, hi);
}

BZ_HD uint4 gf_mul(uint4 a, uint4 b) { return gf_reduce(gf_mul_wide(a, b)); }

// t * X^e for 0 <= e < 128: t shifted left by e bits into 256 bits, reduced.
BZ_HD uint4 gf_mul_xpow(uint4 t, uint32_t e) {
    const uint64_t lo = lo64(t), hi = hi64(t);
    const uint32_t s = e & 63;
    const uint64_t a0 = lo << s;
    const uint64_t a1 = s ? (hi << s) | (lo >> (64 - s)) : hi;
    const uint64_t a2 = s ? hi >> (64 - s) : 0;
    gf_wide w;
    const bool up = e >= 64;
    w.w[0] = up ? 0 : a0;
    w.w[1] = up ? a0 : a1;
    w.w[2] = up ? a1 : a2;
    w.w[3] = up ? a2 : 0;
    return gf_reduce(w);
}

// ---------------------------------------------------------------------------
// Variable x constant with few set bits: XOR of v << s over the set bits s of
// the constant t (t = {t0 bits 0..63, t1 bits 64..127}).  The loop trip count
// is data dependent but warp-uniform when every lane shares t.
// Accumulates into a 6-word (192-bit) window per 64-bit constant word, then
// reduces.
// ---------------------------------------------------------------------------
BZ_HD void shl_xor_into(uint32_t acc[8], uint4 v, uint32_t s, int word_off) {
    // acc[word_off .. word_off+4] ^= (v << s) for 0 <= s < 32
    const uint32_t o0 = v.x << s;
    const uint32_t o1 = __funnelshift_l(v.x, v.y, s);
    const uint32_t o2 = __funnelshift_l(v.y, v.z, s);
    const uint32_t o3 = __funnelshift_l(v.z, v.w, s);
    const uint32_t o4 = __funnelshift_l(v.w, 0u, s);
    acc[word_off + 0] ^= o0;
    acc[word_off + 1] ^= o1;
    acc[word_off + 2] ^= o2;
    acc[word_off + 3] ^= o3;
    acc[word_off + 4] ^= o4;
}

BZ_HD uint4 gf_reduce32(const uint32_t acc[8]) {
    gf_wide w;
    w.w[0] = (uint64_t)acc[0] | ((uint64_t)acc[1] << 32);
    w.w[1] = (uint64_t)acc[2] | ((uint64_t)acc[3] << 32);
    w.w[2] = (uint64_t)acc[4] | ((uint64_t)acc[5] << 32);
    w.w[3] = (uint64_t)acc[6] | ((uint64_t)acc[7] << 32);
    return gf_reduce(w);
}

// v * t where t is given as 4 little-endian 32-bit words; words that are zero
// cost one test.  Meant for twiddles of at most ~64 bits.
BZ_HD uint4 gf_mul_narrow(uint4 v, uint4 t) {
    uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t tw[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        uint32_t bits = tw[w];
        while (bits) {
            const uint32_t s = __ffs(bits) - 1;
            bits &= bits - 1;
            if (w == 0) shl_xor_into(acc, v, s, 0);
            else if (w == 1) shl_xor_into(acc, v, s, 1);
            else if (w == 2) shl_xor_into(acc, v, s, 2);
            else shl_xor_into(acc, v, s, 3);
        }
    }
    return gf_reduce32(acc);
}

// Same product with the shifts done on the integer multiplier (FMA pipe):
// v_k * 2^s gives both halves of the funnel shift in one wide multiply, so a
// set bit costs 4 wide multiplies + 5 XORs instead of 5 shifts + 5 XORs on
// the ALU pipe.  MODE 1 uses the multiplier for every set bit, MODE 2 for
// every other set bit (balancing the two pipes).
BZ_HD void mul_xor_into(uint32_t acc[8], uint4 v, uint32_t m, int o) {
    const uint64_t p0 = (uint64_t)v.x * m, p1 = (uint64_t)v.y * m;
    const uint64_t p2 = (uint64_t)v.z * m, p3 = (uint64_t)v.w * m;
    acc[o + 0] ^= (uint32_t)p0;
    acc[o + 1] ^= (uint32_t)(p0 >> 32) ^ (uint32_t)p1;
    acc[o + 2] ^= (uint32_t)(p1 >> 32) ^ (uint32_t)p2;
    acc[o + 3] ^= (uint32_t)(p2 >> 32) ^ (uint32_t)p3;
    acc[o + 4] ^= (uint32_t)(p3 >> 32);
}

template <int MODE>
BZ_HD uint4 gf_mul_narrow_m(uint4 v, uint4 t) {
    if (MODE == 0) return gf_mul_narrow(v, t);
    uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t tw[4] = {t.x, t.y, t.z, t.w};
    bool use_mul = true;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        uint32_t bits = tw[w];
        while (bits) {
            const uint32_t m = bits & (0u - bits);  // lowest set bit
            bits ^= m;
            if (MODE == 1 || use_mul) {
                mul_xor_into(acc, v, m, w);
            } else {
                shl_xor_into(acc, v, __ffs(m) - 1, w);
            }
            if (MODE == 2) use_mul = !use_mul;
        }
    }
    return gf_reduce32(acc);
}

BZ_HD uint4 ld_u4(const uint4 *p) { return *p; }
BZ_HD void st_u4(uint4 *p, uint4 v) { *p = v; }
