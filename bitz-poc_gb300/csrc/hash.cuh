// Device BLAKE3 and SHA-256 compression functions for the Merkle tree.
// BLAKE3 follows the BLAKE3 specification (the `blake3` crate 1.8.7 used by
// flock-core/src/merkle.rs:160-201); SHA-256 follows FIPS 180-4 (the `sha2`
// crate used by merkle.rs:203-232).
#pragma once
#include <stdint.h>

namespace bz {

__device__ __constant__ uint32_t kIV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                           0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
__device__ __constant__ uint32_t kOne = 1;
constexpr uint32_t B3_CHUNK_START = 1, B3_CHUNK_END = 2, B3_PARENT = 4, B3_ROOT = 8;

__device__ __forceinline__ uint32_t rotr(uint32_t x, int n) { return __funnelshift_r(x, x, n); }

// The two c += d additions are written as multiply-adds by a runtime 1
// (`one`, read from constant memory so the compiler cannot fold it): they
// then issue on the FMA pipe instead of the ALU pipe, which BLAKE3's xors and
// rotates otherwise saturate.  BZ_B3_FMA_ADDS (0, 1 or 2) moves that many of
// the two a += b + m additions to the FMA pipe as well (two multiply-adds
// each instead of one three-input add); with both moved the leaf hashing of
// a 2^24-element commit takes 0.57 ms instead of 0.67 ms on GB300.
#ifndef BZ_B3_FMA_ADDS
#define BZ_B3_FMA_ADDS 2
#endif
#if BZ_B3_FMA_ADDS >= 1
#define BZ_B3ADD1(a, b, x) (s##a = (x) * one + (s##b * one + s##a))
#else
#define BZ_B3ADD1(a, b, x) (s##a = s##a + s##b + (x))
#endif
#if BZ_B3_FMA_ADDS >= 2
#define BZ_B3ADD2(a, b, x) (s##a = (x) * one + (s##b * one + s##a))
#else
#define BZ_B3ADD2(a, b, x) (s##a = s##a + s##b + (x))
#endif
#define BZ_B3G(a, b, c, d, x, y)          \
    do {                                  \
        BZ_B3ADD1(a, b, x);               \
        s##d = rotr(s##d ^ s##a, 16);     \
        s##c = s##d * one + s##c;         \
        s##b = rotr(s##b ^ s##c, 12);     \
        BZ_B3ADD2(a, b, y);               \
        s##d = rotr(s##d ^ s##a, 8);      \
        s##c = s##d * one + s##c;         \
        s##b = rotr(s##b ^ s##c, 7);      \
    } while (0)

// One BLAKE3 round on message words in the given order.
#define BZ_B3ROUND(m0, m1, m2, m3, m4, m5, m6, m7, m8, m9, m10, m11, m12, m13, m14, m15) \
    do {                                                                                  \
        BZ_B3G(0, 4, 8, 12, m0, m1);                                                      \
        BZ_B3G(1, 5, 9, 13, m2, m3);                                                      \
        BZ_B3G(2, 6, 10, 14, m4, m5);                                                     \
        BZ_B3G(3, 7, 11, 15, m6, m7);                                                     \
        BZ_B3G(0, 5, 10, 15, m8, m9);                                                     \
        BZ_B3G(1, 6, 11, 12, m10, m11);                                                   \
        BZ_B3G(2, 7, 8, 13, m12, m13);                                                    \
        BZ_B3G(3, 4, 9, 14, m14, m15);                                                    \
    } while (0)

// Chaining-value compression: cv <- first 8 words of compress(cv, m, ...).
// The message permutation of the specification is applied by listing each
// round's word order explicitly (rounds 1..7).
__device__ __forceinline__ void b3_compress_cv(uint32_t cv[8], const uint32_t m[16],
                                               uint64_t counter, uint32_t block_len,
                                               uint32_t flags) {
    const uint32_t one = kOne;
    uint32_t s0 = cv[0], s1 = cv[1], s2 = cv[2], s3 = cv[3], s4 = cv[4], s5 = cv[5], s6 = cv[6],
             s7 = cv[7];
    uint32_t s8 = kIV[0], s9 = kIV[1], s10 = kIV[2], s11 = kIV[3];
    uint32_t s12 = (uint32_t)counter, s13 = (uint32_t)(counter >> 32), s14 = block_len,
             s15 = flags;
    BZ_B3ROUND(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12],
               m[13], m[14], m[15]);
    BZ_B3ROUND(m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13], m[1], m[11], m[12], m[5], m[9],
               m[14], m[15], m[8]);
    BZ_B3ROUND(m[3], m[4], m[10], m[12], m[13], m[2], m[7], m[14], m[6], m[5], m[9], m[0], m[11],
               m[15], m[8], m[1]);
    BZ_B3ROUND(m[10], m[7], m[12], m[9], m[14], m[3], m[13], m[15], m[4], m[0], m[11], m[2],
               m[5], m[8], m[1], m[6]);
    BZ_B3ROUND(m[12], m[13], m[9], m[11], m[15], m[10], m[14], m[8], m[7], m[2], m[5], m[3],
               m[0], m[1], m[6], m[4]);
    BZ_B3ROUND(m[9], m[14], m[11], m[5], m[8], m[12], m[15], m[1], m[13], m[3], m[0], m[10],
               m[2], m[6], m[4], m[7]);
    BZ_B3ROUND(m[11], m[15], m[5], m[0], m[1], m[9], m[8], m[6], m[14], m[10], m[2], m[12],
               m[3], m[4], m[7], m[13]);
    cv[0] = s0 ^ s8;
    cv[1] = s1 ^ s9;
    cv[2] = s2 ^ s10;
    cv[3] = s3 ^ s11;
    cv[4] = s4 ^ s12;
    cv[5] = s5 ^ s13;
    cv[6] = s6 ^ s14;
    cv[7] = s7 ^ s15;
}

// Non-root parent CV of two child CVs (merge_subtrees_non_root, Mode::Hash).
__device__ __forceinline__ void b3_parent(const uint32_t l[8], const uint32_t r[8],
                                          uint32_t out[8]) {
    uint32_t m[16];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        m[i] = l[i];
        m[8 + i] = r[i];
    }
    uint32_t cv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) cv[i] = kIV[i];
    b3_compress_cv(cv, m, 0, 64, B3_PARENT);
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = cv[i];
}

// ---------------------------------------------------------------------------
// SHA-256
// ---------------------------------------------------------------------------
__device__ __constant__ uint32_t kSHA[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

// w: 16 big-endian message words (already byte-swapped).
__device__ __forceinline__ void sha256_compress(uint32_t st[8], const uint32_t w_in[16]) {
    uint32_t w[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) w[i] = w_in[i];
    uint32_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6],
             h = st[7];
#pragma unroll
    for (int i = 0; i < 64; ++i) {
        uint32_t wi;
        if (i < 16) {
            wi = w[i];
        } else {
            const uint32_t x = w[(i - 15) & 15], y = w[(i - 2) & 15];
            const uint32_t s0 = rotr(x, 7) ^ rotr(x, 18) ^ (x >> 3);
            const uint32_t s1 = rotr(y, 17) ^ rotr(y, 19) ^ (y >> 10);
            wi = w[i & 15] + s0 + w[(i - 7) & 15] + s1;
            w[i & 15] = wi;
        }
        const uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
        const uint32_t ch = (e & f) ^ (~e & g);
        const uint32_t t1 = h + S1 + ch + kSHA[i] + wi;
        const uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
        const uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
        h = g;
        g = f;
        f = e;
        e = d + t1;
        d = c;
        c = b;
        b = a;
        a = t1 + S0 + mj;
    }
    st[0] += a;
    st[1] += b;
    st[2] += c;
    st[3] += d;
    st[4] += e;
    st[5] += f;
    st[6] += g;
    st[7] += h;
}

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

}  // namespace bz
