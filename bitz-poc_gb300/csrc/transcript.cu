// Fiat-Shamir transcript of the opening, on the host.
//
// The state is an incremental BLAKE3 hasher (the `blake3` crate's Hasher that
// BitZ's Blake3Transcript wraps, src/transcript/mod.rs:18-96); squeezes read
// its extended output (finalize_xof) without consuming the state.  Everything
// absorbed here is a few bytes per protocol message, so the hasher is plain
// portable C++; the bulk hashing of the commitment stays on the GPU.
//
// The incremental hasher keeps the chunk being filled and a stack of the
// chaining values of completed subtrees (one per set bit of the number of
// completed chunks): completing chunk c pushes its CV and merges the top of
// the stack once for every trailing zero bit of c + 1, which builds exactly
// the left-complete binary tree of the BLAKE3 specification.  A completed
// chunk is only pushed when more input arrives, so the last chunk (and with
// it the root node) is always still open at finalisation.
#include <string.h>

#include <new>

#include "../../include/bitz_gpu.h"
#include "transcript.h"

namespace bzh {

namespace {

constexpr uint32_t kIV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                             0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
// Message word order of round i+1 is the order of round i taken through this
// permutation (BLAKE3 specification, section 2.2).
constexpr uint8_t kPerm[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
constexpr uint32_t CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8;

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

// Message word order of every round: kSigma[0] is the identity and
// kSigma[r + 1][i] = kSigma[r][kPerm[i]].
struct Sigma {
    uint8_t o[7][16];
    constexpr Sigma() : o() {
        for (int i = 0; i < 16; ++i) o[0][i] = (uint8_t)i;
        for (int r = 1; r < 7; ++r)
            for (int i = 0; i < 16; ++i) o[r][i] = o[r - 1][kPerm[i]];
    }
};
constexpr Sigma kSigma;

#define BZH_G(a, b, c, d, x, y)      \
    do {                             \
        a = a + b + (x);             \
        d = rotr(d ^ a, 16);         \
        c = c + d;                   \
        b = rotr(b ^ c, 12);         \
        a = a + b + (y);             \
        d = rotr(d ^ a, 8);          \
        c = c + d;                   \
        b = rotr(b ^ c, 7);          \
    } while (0)

// Full 16-word compression output: out[i] = s[i] ^ s[i+8] and
// out[i+8] = s[i+8] ^ cv[i].  The state lives in locals and every round
// reads the message through its fixed word order, so the compiler keeps the
// whole state in registers.
void compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
              uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t s0 = cv[0], s1 = cv[1], s2 = cv[2], s3 = cv[3], s4 = cv[4], s5 = cv[5],
             s6 = cv[6], s7 = cv[7];
    uint32_t s8 = kIV[0], s9 = kIV[1], s10 = kIV[2], s11 = kIV[3];
    uint32_t s12 = (uint32_t)counter, s13 = (uint32_t)(counter >> 32), s14 = block_len,
             s15 = flags;
    const uint32_t *m = block;
#pragma GCC unroll 7
    for (int r = 0; r < 7; ++r) {
        const uint8_t *o = kSigma.o[r];
        BZH_G(s0, s4, s8, s12, m[o[0]], m[o[1]]);
        BZH_G(s1, s5, s9, s13, m[o[2]], m[o[3]]);
        BZH_G(s2, s6, s10, s14, m[o[4]], m[o[5]]);
        BZH_G(s3, s7, s11, s15, m[o[6]], m[o[7]]);
        BZH_G(s0, s5, s10, s15, m[o[8]], m[o[9]]);
        BZH_G(s1, s6, s11, s12, m[o[10]], m[o[11]]);
        BZH_G(s2, s7, s8, s13, m[o[12]], m[o[13]]);
        BZH_G(s3, s4, s9, s14, m[o[14]], m[o[15]]);
    }
    out[0] = s0 ^ s8;
    out[1] = s1 ^ s9;
    out[2] = s2 ^ s10;
    out[3] = s3 ^ s11;
    out[4] = s4 ^ s12;
    out[5] = s5 ^ s13;
    out[6] = s6 ^ s14;
    out[7] = s7 ^ s15;
    out[8] = s8 ^ cv[0];
    out[9] = s9 ^ cv[1];
    out[10] = s10 ^ cv[2];
    out[11] = s11 ^ cv[3];
    out[12] = s12 ^ cv[4];
    out[13] = s13 ^ cv[5];
    out[14] = s14 ^ cv[6];
    out[15] = s15 ^ cv[7];
}

void load_words(const uint8_t *p, size_t len, uint32_t w[16]) {
    uint8_t b[64] = {0};
    memcpy(b, p, len);
    for (int i = 0; i < 16; ++i)
        w[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) |
               ((uint32_t)b[4 * i + 2] << 16) | ((uint32_t)b[4 * i + 3] << 24);
}

}  // namespace

void Node::chaining_value(uint32_t out[8]) const {
    uint32_t o[16];
    compress(cv, block, counter, block_len, flags, o);
    memcpy(out, o, 32);
}

void Node::root_output(uint8_t *out, size_t n) const {
    for (uint64_t t = 0; 64 * t < n; ++t) {
        uint32_t o[16];
        compress(cv, block, t, block_len, flags | ROOT, o);
        for (size_t i = 0; i < 64 && 64 * t + i < n; ++i)
            out[64 * t + i] = (uint8_t)(o[i / 4] >> (8 * (i % 4)));
    }
}

Hasher::Hasher() { reset_chunk(0); }

void Hasher::reset_chunk(uint64_t index) {
    memcpy(chunk_cv_, kIV, sizeof chunk_cv_);
    chunk_index_ = index;
    buf_len_ = 0;
    blocks_done_ = 0;
}

void Hasher::push_chunk_cv(const uint32_t cv[8], uint64_t completed) {
    uint32_t cur[8];
    memcpy(cur, cv, sizeof cur);
    for (; (completed & 1) == 0; completed >>= 1) {
        Node p;
        memcpy(p.cv, kIV, sizeof p.cv);
        memcpy(p.block, stack_[--depth_], 32);
        memcpy(p.block + 8, cur, 32);
        p.counter = 0;
        p.block_len = 64;
        p.flags = PARENT;
        p.chaining_value(cur);
    }
    memcpy(stack_[depth_++], cur, 32);
}

void Hasher::update(const uint8_t *p, size_t n) {
    while (n) {
        if (buf_len_ == 64) {
            // a full block with more input behind it is never the chunk's last
            if (blocks_done_ == 15) {
                Node last = chunk_node();
                uint32_t cv[8];
                last.chaining_value(cv);
                push_chunk_cv(cv, chunk_index_ + 1);
                reset_chunk(chunk_index_ + 1);
            } else {
                uint32_t w[16], o[16];
                load_words(buf_, 64, w);
                compress(chunk_cv_, w, chunk_index_, 64, blocks_done_ == 0 ? CHUNK_START : 0, o);
                memcpy(chunk_cv_, o, 32);
                ++blocks_done_;
                buf_len_ = 0;
            }
        }
        size_t take = 64 - buf_len_;
        if (take > n) take = n;
        memcpy(buf_ + buf_len_, p, take);
        buf_len_ += (uint32_t)take;
        p += take;
        n -= take;
    }
}

Node Hasher::chunk_node() const {
    Node c;
    memcpy(c.cv, chunk_cv_, sizeof c.cv);
    load_words(buf_, buf_len_, c.block);
    c.counter = chunk_index_;
    c.block_len = buf_len_;
    c.flags = (blocks_done_ == 0 ? CHUNK_START : 0) | CHUNK_END;
    return c;
}

Node Hasher::root_node() const {
    Node n = chunk_node();
    for (int i = depth_ - 1; i >= 0; --i) {
        uint32_t right[8];
        n.chaining_value(right);
        Node p;
        memcpy(p.cv, kIV, sizeof p.cv);
        memcpy(p.block, stack_[i], 32);
        memcpy(p.block + 8, right, 32);
        p.counter = 0;
        p.block_len = 64;
        p.flags = PARENT;
        n = p;
    }
    return n;
}

void Hasher::xof(uint8_t *out, size_t n) const { root_node().root_output(out, n); }

// ---- Blake3Transcript (src/transcript/mod.rs:18-96, traits.rs:371-376) ----

void Transcript::absorb_slice(const uint8_t *p, size_t n) {
    uint8_t hdr[9];
    hdr[0] = 0x06;
    for (int i = 0; i < 8; ++i) hdr[1 + i] = (uint8_t)((uint64_t)n >> (8 * i));
    h.update(hdr, 9);
    h.update(p, n);
    const uint8_t tail = 0x07;
    h.update(&tail, 1);
}

void Transcript::challenge(uint8_t *out, size_t n) {
    h.xof(out, n);
    const uint8_t open = 0x12, close = 0x34;
    h.update(&open, 1);
    h.update(out, n);
    h.update(&close, 1);
}

void Transcript::sample_f128(uint64_t out[2]) {
    uint8_t b[16];
    challenge(b, 16);
    out[0] = out[1] = 0;
    for (int i = 0; i < 8; ++i) {
        out[0] |= (uint64_t)b[i] << (8 * i);
        out[1] |= (uint64_t)b[8 + i] << (8 * i);
    }
}

void Transcript::observe_f128(const uint64_t v[2]) {
    uint8_t b[16];
    for (int i = 0; i < 8; ++i) {
        b[i] = (uint8_t)(v[0] >> (8 * i));
        b[8 + i] = (uint8_t)(v[1] >> (8 * i));
    }
    absorb_slice(b, 16);
}

void Transcript::fill_sampling_bytes(uint8_t *out, size_t n) {
    static const char kTag[] = "bitz/sampling-read/v1";
    h.xof(out, n);
    h.update((const uint8_t *)kTag, sizeof kTag - 1);
    uint8_t len[8];
    for (int i = 0; i < 8; ++i) len[i] = (uint8_t)((uint64_t)n >> (8 * i));
    h.update(len, 8);
    h.update(out, n);
}

}  // namespace bzh

struct bz_transcript {
    bzh::Transcript t;
};

extern "C" {

int bz_transcript_create(bz_transcript **out) {
    if (!out) return BZ_ERR_ARG;
    *out = new (std::nothrow) bz_transcript();
    return *out ? BZ_OK : BZ_ERR_NOMEM;
}

int bz_transcript_clone(const bz_transcript *t, bz_transcript **out) {
    if (!t || !out) return BZ_ERR_ARG;
    *out = new (std::nothrow) bz_transcript(*t);
    return *out ? BZ_OK : BZ_ERR_NOMEM;
}

int bz_transcript_destroy(bz_transcript *t) {
    delete t;
    return BZ_OK;
}

int bz_transcript_absorb(bz_transcript *t, const uint8_t *data, size_t len) {
    if (!t || (len && !data)) return BZ_ERR_ARG;
    t->t.h.update(data, len);
    return BZ_OK;
}

int bz_transcript_absorb_slice(bz_transcript *t, const uint8_t *data, size_t len) {
    if (!t || (len && !data)) return BZ_ERR_ARG;
    t->t.absorb_slice(data, len);
    return BZ_OK;
}

int bz_transcript_challenge(bz_transcript *t, uint8_t *out, size_t len) {
    if (!t || (len && !out)) return BZ_ERR_ARG;
    t->t.challenge(out, len);
    return BZ_OK;
}

int bz_transcript_sample_f128(bz_transcript *t, uint64_t out[2]) {
    if (!t || !out) return BZ_ERR_ARG;
    t->t.sample_f128(out);
    return BZ_OK;
}

int bz_transcript_observe_f128(bz_transcript *t, const uint64_t v[2]) {
    if (!t || !v) return BZ_ERR_ARG;
    t->t.observe_f128(v);
    return BZ_OK;
}

int bz_transcript_fill_sampling_bytes(bz_transcript *t, uint8_t *out, size_t len) {
    if (!t || (len && !out)) return BZ_ERR_ARG;
    t->t.fill_sampling_bytes(out, len);
    return BZ_OK;
}

int bz_transcript_state_digest(const bz_transcript *t, uint8_t out[32]) {
    if (!t || !out) return BZ_ERR_ARG;
    t->t.h.xof(out, 32);
    return BZ_OK;
}

int bz_blake3_xof(const uint8_t *data, size_t len, uint8_t *out, size_t out_len) {
    if ((len && !data) || (out_len && !out)) return BZ_ERR_ARG;
    bzh::Hasher h;
    h.update(data, len);
    h.xof(out, out_len);
    return BZ_OK;
}

}  // extern "C"

bzh::Transcript *bz_transcript_inner(bz_transcript *t) { return t ? &t->t : nullptr; }
