// Proof-of-work nonce search on the GPU, and the challenger's grind/verify on
// top of the host transcript.
//
// The reference grinds with first_pow_nonce / smallest_pow_nonce
// (src/utils/blake3x4.rs:42-120): the smallest nonce such that
// blake3(prefix || nonce as u64 LE) has at least `bits` leading zero bits,
// counted from the most significant bit of digest byte 0.  The prefix and
// nonce fit one 64-byte block, so every candidate is one BLAKE3 compression
// with CHUNK_START | CHUNK_END | ROOT.
//
// Search: persistent blocks take chunks of consecutive nonces in increasing
// order from a global counter and record hits with atomicMin.  A block stops
// when the counter passes the window or when its next chunk starts above the
// best hit so far.  Because chunks are handed out in order and a chunk that
// was started is always finished, every chunk that starts below the final
// minimum was scanned completely: the result is the serial scan's nonce,
// independent of scheduling.  No block waits on another; the host sizes each
// launch to a bounded window and continues with the next window only when
// the current one had no hit.
#include <cuda_runtime.h>
#include <math.h>

#include "../../include/bitz_gpu.h"
#include "hash.cuh"
#include "runtime.h"
#include "transcript.h"

namespace {

constexpr int kPowThreads = 256;
constexpr int kPowPerThread = 4;                    // nonces per thread per chunk above 20 bits
constexpr uint64_t kPowWindow = (uint64_t)1 << 34;  // nonces per launch (< 1 s)
// Device state at this byte offset of the context's small buffer: the chunk
// counter, the best hit and the blocks' exit ticket.  The launch's last block
// posts the best hit to the mapped mailbox (kPowBestOffset, then the sequence
// number at kPowSeqOffset) and restores the state for the next launch.
constexpr size_t kPowCtlOffset = 256;
constexpr size_t kPowBestOffset = 256, kPowSeqOffset = 320;  // mapped mailbox bytes

struct PowPost {
    unsigned int *ticket;
    unsigned long long *best;  // device view of mapped host memory
    uint32_t *seq;             // device view of mapped host memory
    uint32_t seq_val;
};

struct PowBlock {
    uint32_t w[16];  // prefix words, zero where the nonce goes
};

// `bits` leading zero bits of the digest read as a big-endian bit string.
__device__ __forceinline__ bool pow_pass(const uint32_t h[8], uint32_t bits) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (bits == 0) return true;
        const uint32_t be = __byte_perm(h[i], 0, 0x0123);
        if (bits < 32) return (be >> (32 - bits)) == 0;
        if (be) return false;
        bits -= 32;
    }
    return bits == 0;
}

__global__ void __launch_bounds__(kPowThreads) pow_scan_kernel(PowBlock blk, uint32_t block_len,
                                                               uint32_t nonce_off, uint32_t bits,
                                                               uint64_t start, uint64_t span,
                                                               uint32_t per,
                                                               unsigned long long *ctl,
                                                               PowPost post) {
    __shared__ unsigned long long s_base;
    __shared__ int s_stop;
    const uint32_t wi = nonce_off >> 2, sh = (nonce_off & 3) * 8;
    const unsigned long long chunk = (unsigned long long)kPowThreads * per;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long base = atomicAdd(&ctl[0], chunk);
            const unsigned long long best = *(volatile unsigned long long *)&ctl[1];
            s_base = base;
            s_stop = base >= span || start + base > best;
        }
        __syncthreads();
        const uint64_t base = s_base;
        const int stop = s_stop;
        __syncthreads();
        if (stop) break;
#pragma unroll 1
        for (uint32_t i = 0; i < per; ++i) {
            const uint64_t rel = base + (uint64_t)i * kPowThreads + threadIdx.x;
            if (rel >= span) break;
            const uint64_t nonce = start + rel;
            const uint32_t lo = (uint32_t)nonce, hi = (uint32_t)(nonce >> 32);
            // the 8 nonce bytes start at byte nonce_off: up to three words
            const uint32_t a = lo << sh;
            const uint32_t b = sh ? (lo >> (32 - sh)) | (hi << sh) : hi;
            const uint32_t c = sh ? hi >> (32 - sh) : 0u;
            uint32_t m[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
                m[j] = blk.w[j] | ((uint32_t)j == wi ? a : 0u) | ((uint32_t)j == wi + 1 ? b : 0u) |
                       ((uint32_t)j == wi + 2 ? c : 0u);
            uint32_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) h[j] = bz::kIV[j];
            bz::b3_compress_cv(h, m, 0, block_len,
                               bz::B3_CHUNK_START | bz::B3_CHUNK_END | bz::B3_ROOT);
            if (pow_pass(h, bits)) atomicMin(&ctl[1], (unsigned long long)nonce);
        }
    }
    // every hit of this block was recorded before the barrier that preceded
    // the stop; the last block to leave posts the minimum and resets
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(post.ticket, 1u) == gridDim.x - 1) {
            __threadfence();
            *(volatile unsigned long long *)post.best = *(volatile unsigned long long *)&ctl[1];
            asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(post.seq), "r"(post.seq_val)
                         : "memory");
            ctl[0] = 0;
            ctl[1] = ~0ull;
            *post.ticket = 0;
        }
    }
}

}  // namespace

extern "C" {

int bz_pow_first_nonce(bz_ctx *ctx, const uint8_t *prefix, size_t prefix_len, uint32_t bits,
                       uint64_t start, uint64_t end, uint64_t *nonce) {
    if (!ctx || !nonce || (prefix_len && !prefix)) return BZ_ERR_ARG;
    if (prefix_len + 8 > 64) return bz::set_msg(ctx, BZ_ERR_ARG, "prefix + nonce exceed one block");
    if (bits > 256) return bz::set_msg(ctx, BZ_ERR_ARG, "bits > 256");
    if (start >= end) return bz::set_msg(ctx, BZ_ERR_NOTFOUND, "empty nonce range");
    if (bits == 0) {
        *nonce = start;
        return BZ_OK;
    }
    PowBlock blk;
    uint8_t bytes[64] = {0};
    for (size_t i = 0; i < prefix_len; ++i) bytes[i] = prefix[i];
    for (int i = 0; i < 16; ++i)
        blk.w[i] = (uint32_t)bytes[4 * i] | ((uint32_t)bytes[4 * i + 1] << 8) |
                   ((uint32_t)bytes[4 * i + 2] << 16) | ((uint32_t)bytes[4 * i + 3] << 24);
    unsigned long long *ctl =
        (unsigned long long *)((uint8_t *)ctx->d_small + kPowCtlOffset);
    unsigned int *ticket = (unsigned int *)(ctl + 2);
    if (!ctx->pow_ready) {
        BZ_CUDA(ctx, cudaMemsetAsync(ctl, 0, 8, ctx->stream));
        BZ_CUDA(ctx, cudaMemsetAsync(ctl + 1, 0xFF, 8, ctx->stream));
        BZ_CUDA(ctx, cudaMemsetAsync(ticket, 0, 4, ctx->stream));
        ctx->pow_ready = true;
    }
    // one nonce per thread per chunk for short searches (the first chunks end
    // sooner), four above 20 bits; enough blocks for ~4 expected hits' worth
    // of nonces, at most 8 per SM
    const uint32_t per = bits <= 20 ? 1u : (uint32_t)kPowPerThread;
    const double chunk = (double)kPowThreads * per;
    const double want = ldexp(4.0, bits < 60 ? (int)bits : 60) / chunk;
    const int max_blocks = ctx->num_sms * 8;
    const int blocks = want >= max_blocks ? max_blocks : (want < 1.0 ? 1 : (int)want);
    PowPost post;
    post.ticket = ticket;
    post.best = (unsigned long long *)((uint8_t *)ctx->d_mbox + kPowBestOffset);
    post.seq = (uint32_t *)((uint8_t *)ctx->d_mbox + kPowSeqOffset);
    for (uint64_t s = start; s < end;) {
        const uint64_t span = end - s < kPowWindow ? end - s : kPowWindow;
        if (++ctx->pow_seq == 0) ++ctx->pow_seq;
        post.seq_val = ctx->pow_seq;
        pow_scan_kernel<<<blocks, kPowThreads, 0, ctx->stream>>>(
            blk, (uint32_t)(prefix_len + 8), (uint32_t)prefix_len, bits, s, span, per, ctl, post);
        ctx->launches += 1;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            ctx->pow_ready = false;
            return bz::set_err(ctx, BZ_ERR_CUDA, "pow_scan_kernel launch", e);
        }
        const int rc = bz::mapped_wait(ctx, kPowSeqOffset, post.seq_val, "proof-of-work search");
        if (rc) {
            ctx->pow_ready = false;
            return rc;
        }
        const unsigned long long best =
            *(const volatile unsigned long long *)((uint8_t *)ctx->h_mbox + kPowBestOffset);
        if (best != ~0ull) {
            *nonce = best;
            return BZ_OK;
        }
        s += span;
    }
    return bz::set_msg(ctx, BZ_ERR_NOTFOUND, "no nonce in range passes");
}

int bz_transcript_grind_pow(bz_ctx *ctx, bz_transcript *t, uint32_t bits, uint64_t *nonce) {
    bzh::Transcript *tr = bz_transcript_inner(t);
    if (!ctx || !tr || !nonce) return BZ_ERR_ARG;
    // ZincChallenger::grind_pow / pow_seed (src/ligerito_flock.rs:70-99,115-122)
    uint64_t seed_w[2];
    tr->sample_f128(seed_w);
    uint8_t seed[16];
    for (int i = 0; i < 8; ++i) {
        seed[i] = (uint8_t)(seed_w[0] >> (8 * i));
        seed[8 + i] = (uint8_t)(seed_w[1] >> (8 * i));
    }
    uint64_t n = 0;
    if (bits) {
        int rc = bz_pow_first_nonce(ctx, seed, 16, bits, 0, ~0ull, &n);
        if (rc) return rc;
    }
    uint8_t le[8];
    for (int i = 0; i < 8; ++i) le[i] = (uint8_t)(n >> (8 * i));
    tr->absorb_slice(le, 8);
    *nonce = n;
    return BZ_OK;
}

int bz_transcript_verify_pow(bz_transcript *t, uint64_t nonce, uint32_t bits, int *ok) {
    bzh::Transcript *tr = bz_transcript_inner(t);
    if (!tr || !ok) return BZ_ERR_ARG;
    // ZincChallenger::verify_pow (src/ligerito_flock.rs:101-113)
    uint64_t seed_w[2];
    tr->sample_f128(seed_w);
    uint8_t msg[24];
    for (int i = 0; i < 8; ++i) {
        msg[i] = (uint8_t)(seed_w[0] >> (8 * i));
        msg[8 + i] = (uint8_t)(seed_w[1] >> (8 * i));
        msg[16 + i] = (uint8_t)(nonce >> (8 * i));
    }
    int pass;
    if (bits == 0) {
        pass = nonce == 0;
    } else {
        bzh::Hasher h;
        h.update(msg, 24);
        uint8_t d[32];
        h.xof(d, 32);
        uint32_t lz = 0;
        for (int i = 0; i < 32; ++i) {
            if (d[i] == 0) {
                lz += 8;
                continue;
            }
            for (uint8_t b = d[i]; !(b & 0x80); b = (uint8_t)(b << 1)) ++lz;
            break;
        }
        pass = lz >= bits;
    }
    tr->absorb_slice(msg + 16, 8);
    *ok = pass;
    return BZ_OK;
}

}  // extern "C"
