/*
 * CPU oracle for the BitZ / flock Ligerito commitment path -- TEST
 * INFRASTRUCTURE ONLY (see oracle.h for the parity status and the rule that
 * nothing in the GPU library links this file).
 *
 * Every function cites the reference file:line it restates.  Paths are given
 * relative to the BitZ-PoC project root; "flock-core/" abbreviates
 * vendor/flock-mod/crates/flock-core/.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdint.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ========================================================================
 * GF(2^128) -- vendor/field/src/gf128.rs:80-180, gf128/portable.rs:10-96
 * Bit i of the little-endian 128-bit value is the coefficient of X^i and
 * X^128 = X^7 + X^2 + X + 1.
 * ======================================================================== */

/* 64x64 carry-less product.  On aarch64 with the crypto extension this is
 * the PMULL instruction (the instruction the reference's aarch64 kernels use,
 * vendor/field/src/gf128/kernels/aarch64.rs), so the CPU baseline measured on
 * the Grace host is not handicapped; elsewhere a 4-bit window formulation of
 * the schoolbook product: the 16 multiples of `a` by polynomials of degree < 4
 * are tabled, then each nibble of `b` selects one multiple shifted into
 * place.  Both are exact, so results are identical on every host. */
#if defined(__aarch64__) && defined(__ARM_FEATURE_AES)
#include <arm_neon.h>
static inline u128 clmul64(uint64_t a, uint64_t b) {
    poly128_t p = vmull_p64((poly64_t)a, (poly64_t)b);
    u128 r;
    memcpy(&r, &p, sizeof r);
    return r;
}
#else
static inline u128 clmul64(uint64_t a, uint64_t b) {
    u128 tbl[16];
    tbl[0] = 0;
    tbl[1] = a;
    for (int i = 2; i < 16; i += 2) {
        tbl[i] = tbl[i >> 1] << 1;
        tbl[i + 1] = tbl[i] ^ a;
    }
    u128 acc = 0;
    for (int n = 15; n >= 0; --n) {
        acc = (acc << 4) ^ tbl[(b >> (4 * n)) & 15];
    }
    return acc;
}
#endif

const char *orc_clmul_kind(void) {
#if defined(__aarch64__) && defined(__ARM_FEATURE_AES)
    return "pmull";
#else
    return "portable";
#endif
}

/* Karatsuba 128x128 -> 256 (portable.rs:62-68). */
static inline void clmul128(const uint64_t a[2], const uint64_t b[2], uint64_t r[4]) {
    u128 lo = clmul64(a[0], b[0]);
    u128 hi = clmul64(a[1], b[1]);
    u128 mid = clmul64(a[0] ^ a[1], b[0] ^ b[1]) ^ lo ^ hi;
    r[0] = (uint64_t)lo;
    r[1] = (uint64_t)(lo >> 64) ^ (uint64_t)mid;
    r[2] = (uint64_t)hi ^ (uint64_t)(mid >> 64);
    r[3] = (uint64_t)(hi >> 64);
}

/* w * g for g = X^7 + X^2 + X + 1, as a 128-bit value. */
static inline u128 times_g(uint64_t w) {
    u128 x = w;
    return x ^ (x << 1) ^ (x << 2) ^ (x << 7);
}

/* Reduce a 256-bit product modulo X^128 + g (portable.rs:70-96): substitute
 * X^128 = g for the two high words, then once more for the <= 7 bits that
 * spill back above X^128. */
static inline void reduce256(const uint64_t r[4], uint64_t out[2]) {
    u128 f2 = times_g(r[2]);
    u128 f3 = times_g(r[3]);
    uint64_t w0 = r[0] ^ (uint64_t)f2;
    uint64_t w1 = r[1] ^ (uint64_t)(f2 >> 64) ^ (uint64_t)f3;
    uint64_t spill = (uint64_t)(f3 >> 64);
    w0 ^= (uint64_t)times_g(spill);
    out[0] = w0;
    out[1] = w1;
}

void orc_gf_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]) {
    uint64_t r[4];
    clmul128(a, b, r);
    reduce256(r, out);
}

/* Shift-and-add multiply, structurally unlike the windowed path; the tests
 * compare the two. */
void orc_gf_mul_bitwise(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]) {
    uint64_t x0 = a[0], x1 = a[1], z0 = 0, z1 = 0;
    for (int i = 0; i < 128; ++i) {
        uint64_t bit = (i < 64 ? b[0] >> i : b[1] >> (i - 64)) & 1;
        if (bit) {
            z0 ^= x0;
            z1 ^= x1;
        }
        uint64_t carry = x1 >> 63;
        x1 = (x1 << 1) | (x0 >> 63);
        x0 = (x0 << 1) ^ (carry ? 0x87ULL : 0);
    }
    out[0] = z0;
    out[1] = z1;
}

static inline void gf_mul(const uint64_t *a, const uint64_t *b, uint64_t *out) {
    uint64_t t[2];
    orc_gf_mul(a, b, t);
    out[0] = t[0];
    out[1] = t[1];
}

void orc_gf_mul_many(const uint64_t *a, const uint64_t *b, uint64_t *out, size_t n) {
    for (size_t i = 0; i < n; ++i) gf_mul(a + 2 * i, b + 2 * i, out + 2 * i);
}

/* Inverse as a^(2^128 - 2) (any correct inverse agrees with the reference's
 * fixed-schedule inverse_or_zero, gf128.rs:122-126; zero maps to zero). */
void orc_gf_inv(const uint64_t a[2], uint64_t out[2]) {
    /* a^(2^128-2) = (a^(2^127-1))^2 ; build a^(2^k-1) by doubling. */
    uint64_t acc[2] = {a[0], a[1]}; /* a^(2^1-1) */
    for (int k = 1; k < 127; ++k) {
        uint64_t sq[2];
        gf_mul(acc, acc, sq);    /* a^(2^(k+1)-2) */
        gf_mul(sq, a, acc);      /* a^(2^(k+1)-1) */
    }
    gf_mul(acc, acc, out);       /* a^(2^128-2) */
}

void orc_ghash_chain(const uint64_t h[2], const uint64_t *blocks, size_t n, uint64_t out[2]) {
    uint64_t x[2] = {0, 0};
    for (size_t i = 0; i < n; ++i) {
        x[0] ^= blocks[2 * i];
        x[1] ^= blocks[2 * i + 1];
        gf_mul(x, h, x);
    }
    out[0] = x[0];
    out[1] = x[1];
}

/* ========================================================================
 * Tiny parallel-for over [0, n) in contiguous ranges.
 * ======================================================================== */
typedef void (*range_fn)(void *ctx, size_t lo, size_t hi);
struct pf_job { range_fn fn; void *ctx; size_t lo, hi; };
static void *pf_tramp(void *p) {
    struct pf_job *j = (struct pf_job *)p;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}
static void parallel_for(size_t n, int n_threads, range_fn fn, void *ctx) {
    if (n_threads <= 1 || n < 2) {
        fn(ctx, 0, n);
        return;
    }
    if ((size_t)n_threads > n) n_threads = (int)n;
    pthread_t th[256];
    struct pf_job jobs[256];
    if (n_threads > 256) n_threads = 256;
    size_t per = (n + n_threads - 1) / n_threads;
    int started = 0;
    jobs[0] = (struct pf_job){fn, ctx, 0, per < n ? per : n};
    for (int t = 0; t < n_threads; ++t) {
        size_t lo = (size_t)t * per, hi = lo + per;
        if (lo >= n) break;
        if (hi > n) hi = n;
        jobs[t] = (struct pf_job){fn, ctx, lo, hi};
        if (t == 0) continue;
        if (pthread_create(&th[t], NULL, pf_tramp, &jobs[t]) != 0) {
            fn(ctx, lo, hi);
            jobs[t].fn = NULL;
        }
        started = t + 1;
    }
    fn(ctx, jobs[0].lo, jobs[0].hi);
    for (int t = 1; t < started; ++t)
        if (jobs[t].fn) pthread_join(th[t], NULL);
}

/* ========================================================================
 * Additive NTT -- flock-core/src/ntt/additive_ntt_f128.rs
 * ======================================================================== */

/* generate_evals_from_subspace (:66-100) for the basis {1, x, .., x^(l-1)}
 * (:136-140).  Row i has length l - i; row i, entry k is stored at
 * out[2*(i*l + k)].  Rows are built from the unnormalized previous row, then
 * every row is divided by its 0-th entry. */
void orc_ntt_evals(int l, uint64_t *out) {
    if (l <= 0) return;
    memset(out, 0, sizeof(uint64_t) * 2 * (size_t)l * (size_t)l);
    for (int k = 0; k < l; ++k) {
        out[2 * k] = (k < 64) ? (1ULL << k) : 0;
        out[2 * k + 1] = (k >= 64) ? (1ULL << (k - 64)) : 0;
    }
    for (int i = 1; i < l; ++i) {
        const uint64_t *prev = out + 2 * (size_t)(i - 1) * l;
        uint64_t *row = out + 2 * (size_t)i * l;
        int prev_len = l - (i - 1);
        for (int k = 1; k < prev_len; ++k) {
            uint64_t s[2] = {prev[2 * k] ^ prev[0], prev[2 * k + 1] ^ prev[1]};
            gf_mul(prev + 2 * k, s, row + 2 * (k - 1));
        }
    }
    for (int i = 0; i < l; ++i) {
        uint64_t *row = out + 2 * (size_t)i * l;
        uint64_t inv[2];
        orc_gf_inv(row, inv);
        for (int k = 0; k < l - i; ++k) gf_mul(row + 2 * k, inv, row + 2 * k);
    }
}

/* twiddle(layer, block) = span_get(evals[l-layer-1][1..], block) (:150-156,
 * span_get :105-113). */
static void twiddle_from_evals(const uint64_t *evals, int l, int layer, uint64_t block,
                               uint64_t out[2]) {
    const uint64_t *row = evals + 2 * (size_t)(l - layer - 1) * l;
    uint64_t a0 = 0, a1 = 0;
    for (int j = 0; j < layer && j < 64; ++j) {
        if ((block >> j) & 1) {
            a0 ^= row[2 * (1 + j)];
            a1 ^= row[2 * (1 + j) + 1];
        }
    }
    out[0] = a0;
    out[1] = a1;
}

void orc_ntt_twiddle(int log_domain, int layer, uint64_t block, uint64_t out[2]) {
    uint64_t *ev = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)log_domain * log_domain);
    orc_ntt_evals(log_domain, ev);
    twiddle_from_evals(ev, log_domain, layer, block, out);
    free(ev);
}

struct ntt_layer_ctx {
    uint64_t *data;
    const uint64_t *evals;
    size_t num_ntts;
    int l, layer;
};

/* One layer of forward_transform_interleaved_scalar_from_layer (:243-274):
 * blocks of 2^(l-layer) positions, pairs (row, row + half), every lane:
 * u <- u + t*v ; v <- v + u.  Parallel over blocks. */
static void ntt_layer_blocks(void *p, size_t lo, size_t hi) {
    struct ntt_layer_ctx *c = (struct ntt_layer_ctx *)p;
    size_t block_size = (size_t)1 << (c->l - c->layer);
    size_t half = block_size >> 1;
    for (size_t blk = lo; blk < hi; ++blk) {
        uint64_t tw[2];
        twiddle_from_evals(c->evals, c->l, c->layer, blk, tw);
        uint64_t *base = c->data + 2 * blk * block_size * c->num_ntts;
        for (size_t row = 0; row < half; ++row) {
            uint64_t *top = base + 2 * row * c->num_ntts;
            uint64_t *bot = top + 2 * half * c->num_ntts;
            for (size_t lane = 0; lane < c->num_ntts; ++lane) {
                uint64_t *u = top + 2 * lane, *v = bot + 2 * lane, t[2];
                gf_mul(v, tw, t);
                u[0] ^= t[0];
                u[1] ^= t[1];
                v[0] ^= u[0];
                v[1] ^= u[1];
            }
        }
    }
}

/* Same layer, parallel over rows inside each block (top layers have few
 * blocks). */
struct ntt_rows_ctx {
    struct ntt_layer_ctx *c;
    size_t blk;
    uint64_t tw[2];
};
static void ntt_layer_rows(void *p, size_t lo, size_t hi) {
    struct ntt_rows_ctx *r = (struct ntt_rows_ctx *)p;
    struct ntt_layer_ctx *c = r->c;
    size_t block_size = (size_t)1 << (c->l - c->layer);
    size_t half = block_size >> 1;
    uint64_t *base = c->data + 2 * r->blk * block_size * c->num_ntts;
    for (size_t row = lo; row < hi; ++row) {
        uint64_t *top = base + 2 * row * c->num_ntts;
        uint64_t *bot = top + 2 * half * c->num_ntts;
        for (size_t lane = 0; lane < c->num_ntts; ++lane) {
            uint64_t *u = top + 2 * lane, *v = bot + 2 * lane, t[2];
            gf_mul(v, r->tw, t);
            u[0] ^= t[0];
            u[1] ^= t[1];
            v[0] ^= u[0];
            v[1] ^= u[1];
        }
    }
}

void orc_ntt_forward_interleaved(uint64_t *data, size_t num_ntts, int log_d, int start_layer,
                                 int n_threads) {
    if (log_d <= 0) return;
    uint64_t *ev = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)log_d * log_d);
    orc_ntt_evals(log_d, ev);
    for (int layer = start_layer; layer < log_d; ++layer) {
        struct ntt_layer_ctx c = {data, ev, num_ntts, log_d, layer};
        size_t nblocks = (size_t)1 << layer;
        if (n_threads > 1 && nblocks < (size_t)n_threads * 4) {
            size_t half = (size_t)1 << (log_d - layer - 1);
            for (size_t blk = 0; blk < nblocks; ++blk) {
                struct ntt_rows_ctx r = {&c, blk, {0, 0}};
                twiddle_from_evals(ev, log_d, layer, blk, r.tw);
                parallel_for(half, n_threads, ntt_layer_rows, &r);
            }
        } else {
            parallel_for(nblocks, n_threads, ntt_layer_blocks, &c);
        }
    }
    free(ev);
}

/* ------------------------------------------------------------------------
 * The same transform with the reference's parallel structure
 * (forward_transform_interleaved_parallel_from_layer, :298-517): the top
 * layers sweep the whole buffer two at a time (the fused 2-layer row op of
 * :829-857, which is the two layers applied in order), and the deep layers
 * run sub-group by sub-group, each sub-group (a block of at most 2 MiB) held
 * in cache while all of its remaining layers are applied (:434-516).  Work is
 * handed to a persistent pool of threads instead of threads started per
 * layer.  Identical output to orc_ntt_forward_interleaved.
 * ------------------------------------------------------------------------ */
static struct {
    pthread_mutex_t mu;
    pthread_cond_t cv_work, cv_done;
    int n_workers;
    pthread_t th[256];
    unsigned gen;
    int pending;
    range_fn fn;
    void *ctx;
    size_t n, chunk;
    atomic_size_t next;
} g_pool = {PTHREAD_MUTEX_INITIALIZER, PTHREAD_COND_INITIALIZER, PTHREAD_COND_INITIALIZER};

static void pool_drain(void) {
    for (;;) {
        size_t i = atomic_fetch_add(&g_pool.next, g_pool.chunk);
        if (i >= g_pool.n) break;
        size_t hi = i + g_pool.chunk < g_pool.n ? i + g_pool.chunk : g_pool.n;
        g_pool.fn(g_pool.ctx, i, hi);
    }
}

/* arg: the generation current when the worker was created (before the job
 * that created it was published), so that job is the first one it runs */
static void *pool_worker(void *arg) {
    unsigned seen = (unsigned)(uintptr_t)arg;
    pthread_mutex_lock(&g_pool.mu);
    for (;;) {
        while (g_pool.gen == seen) pthread_cond_wait(&g_pool.cv_work, &g_pool.mu);
        seen = g_pool.gen;
        pthread_mutex_unlock(&g_pool.mu);
        pool_drain();
        pthread_mutex_lock(&g_pool.mu);
        if (--g_pool.pending == 0) pthread_cond_signal(&g_pool.cv_done);
    }
    return NULL;
}

/* fn over [0, n) in chunks of `chunk` items, by the calling thread and up to
 * n_threads - 1 pool workers (created once, kept for the process). */
static void pool_run(size_t n, size_t chunk, int n_threads, range_fn fn, void *ctx) {
    if (n_threads <= 1 || n <= chunk) {
        fn(ctx, 0, n);
        return;
    }
    if (n_threads > 256) n_threads = 256;
    pthread_mutex_lock(&g_pool.mu);
    while (g_pool.n_workers < n_threads - 1) {
        if (pthread_create(&g_pool.th[g_pool.n_workers], NULL, pool_worker,
                           (void *)(uintptr_t)g_pool.gen) != 0)
            break;
        g_pool.n_workers++;
    }
    g_pool.fn = fn;
    g_pool.ctx = ctx;
    g_pool.n = n;
    g_pool.chunk = chunk ? chunk : 1;
    atomic_store(&g_pool.next, 0);
    g_pool.pending = g_pool.n_workers;
    g_pool.gen++;
    pthread_cond_broadcast(&g_pool.cv_work);
    pthread_mutex_unlock(&g_pool.mu);
    pool_drain();
    pthread_mutex_lock(&g_pool.mu);
    while (g_pool.pending > 0) pthread_cond_wait(&g_pool.cv_done, &g_pool.mu);
    pthread_mutex_unlock(&g_pool.mu);
}

/* u <- u + t v ; v <- v + u over `lanes` lanes of rows u and v */
static inline void butterfly_rows(uint64_t *u, uint64_t *v, size_t lanes, const uint64_t t[2]) {
    const int zero = (t[0] | t[1]) == 0;
    for (size_t lane = 0; lane < lanes; ++lane) {
        uint64_t *a = u + 2 * lane, *b = v + 2 * lane;
        if (!zero) {
            uint64_t p[2];
            gf_mul(b, t, p);
            a[0] ^= p[0];
            a[1] ^= p[1];
        }
        b[0] ^= a[0];
        b[1] ^= a[1];
    }
}

struct ntt_blk_ctx {
    uint64_t *data;
    const uint64_t *evals;
    size_t lanes;
    int l, layer, deep_start;
};

/* Fused pair of top layers (layer, layer+1): item = (block B, row rr) of the
 * quads at positions B*4Q + g*Q + rr, g = 0..3. */
static void ntt_pair_items(void *p, size_t lo, size_t hi) {
    struct ntt_blk_ctx *c = (struct ntt_blk_ctx *)p;
    const int log_q = c->l - c->layer - 2;
    const size_t Q = (size_t)1 << log_q, row = 2 * c->lanes;
    for (size_t it = lo; it < hi; ++it) {
        const size_t B = it >> log_q, rr = it & (Q - 1);
        uint64_t to[2], ta[2], tb[2];
        twiddle_from_evals(c->evals, c->l, c->layer, B, to);
        twiddle_from_evals(c->evals, c->l, c->layer + 1, 2 * B, ta);
        twiddle_from_evals(c->evals, c->l, c->layer + 1, 2 * B + 1, tb);
        uint64_t *x0 = c->data + (B * 4 * Q + rr) * row;
        uint64_t *x1 = x0 + Q * row, *x2 = x1 + Q * row, *x3 = x2 + Q * row;
        butterfly_rows(x0, x2, c->lanes, to);
        butterfly_rows(x1, x3, c->lanes, to);
        butterfly_rows(x0, x1, c->lanes, ta);
        butterfly_rows(x2, x3, c->lanes, tb);
    }
}

/* A single top layer: item = (block B, row rr) of the pair (rr, rr + half). */
static void ntt_single_items(void *p, size_t lo, size_t hi) {
    struct ntt_blk_ctx *c = (struct ntt_blk_ctx *)p;
    const int log_h = c->l - c->layer - 1;
    const size_t H = (size_t)1 << log_h, row = 2 * c->lanes;
    for (size_t it = lo; it < hi; ++it) {
        const size_t B = it >> log_h, rr = it & (H - 1);
        uint64_t t[2];
        twiddle_from_evals(c->evals, c->l, c->layer, B, t);
        uint64_t *u = c->data + (B * 2 * H + rr) * row;
        butterfly_rows(u, u + H * row, c->lanes, t);
    }
}

/* Deep layers of one cache-resident sub-group: item = sub-group index G (the
 * block of layer deep_start), every layer from deep_start down to the last. */
static void ntt_subgroup_items(void *p, size_t lo, size_t hi) {
    struct ntt_blk_ctx *c = (struct ntt_blk_ctx *)p;
    const size_t row = 2 * c->lanes;
    for (size_t G = lo; G < hi; ++G) {
        for (int layer = c->deep_start; layer < c->l; ++layer) {
            const int d = layer - c->deep_start;          /* sub-blocks of G at this layer */
            const size_t H = (size_t)1 << (c->l - layer - 1);
            for (size_t sb = 0; sb < ((size_t)1 << d); ++sb) {
                const size_t B = (G << d) | sb;
                uint64_t t[2];
                twiddle_from_evals(c->evals, c->l, layer, B, t);
                uint64_t *base = c->data + B * 2 * H * row;
                for (size_t rr = 0; rr < H; ++rr)
                    butterfly_rows(base + rr * row, base + (rr + H) * row, c->lanes, t);
            }
        }
    }
}

void orc_ntt_forward_interleaved_blocked(uint64_t *data, size_t num_ntts, int log_d,
                                         int start_layer, int n_threads) {
    if (log_d <= 0 || start_layer >= log_d) return;
    uint64_t *ev = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)log_d * log_d);
    orc_ntt_evals(log_d, ev);
    /* sub-groups of 2^s positions, at most 2 MiB (at least one pair) */
    int s = 1;
    while (s < log_d - start_layer && ((size_t)2 << s) * num_ntts * 16 <= ((size_t)2 << 20)) ++s;
    struct ntt_blk_ctx c = {data, ev, num_ntts, log_d, start_layer, log_d - s};
    int layer = start_layer;
    while (layer < c.deep_start) {
        c.layer = layer;
        if (layer + 1 < c.deep_start) {
            pool_run((size_t)1 << (log_d - 2), 16, n_threads, ntt_pair_items, &c);
            layer += 2;
        } else {
            pool_run((size_t)1 << (log_d - 1), 16, n_threads, ntt_single_items, &c);
            layer += 1;
        }
    }
    pool_run((size_t)1 << c.deep_start, 1, n_threads, ntt_subgroup_items, &c);
    free(ev);
}

void orc_ntt_forward(uint64_t *data, int log_d) {
    orc_ntt_forward_interleaved(data, 1, log_d, 0, 1);
}

/* ========================================================================
 * SHA-256 (FIPS 180-4) -- the `sha2` 0.10 crate used by flock-core/src/merkle.rs
 * ======================================================================== */
static const uint32_t SHA_K[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};
static const uint32_t IV8[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};

static inline uint32_t rotr32(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static void sha256_block(uint32_t st[8], const uint8_t blk[64]) {
    uint32_t w[64];
    for (int i = 0; i < 16; ++i)
        w[i] = ((uint32_t)blk[4 * i] << 24) | ((uint32_t)blk[4 * i + 1] << 16) |
               ((uint32_t)blk[4 * i + 2] << 8) | blk[4 * i + 3];
    for (int i = 16; i < 64; ++i) {
        uint32_t s0 = rotr32(w[i - 15], 7) ^ rotr32(w[i - 15], 18) ^ (w[i - 15] >> 3);
        uint32_t s1 = rotr32(w[i - 2], 17) ^ rotr32(w[i - 2], 19) ^ (w[i - 2] >> 10);
        w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6],
             h = st[7];
    for (int i = 0; i < 64; ++i) {
        uint32_t S1 = rotr32(e, 6) ^ rotr32(e, 11) ^ rotr32(e, 25);
        uint32_t ch = (e & f) ^ (~e & g);
        uint32_t t1 = h + S1 + ch + SHA_K[i] + w[i];
        uint32_t S0 = rotr32(a, 2) ^ rotr32(a, 13) ^ rotr32(a, 22);
        uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
        uint32_t t2 = S0 + mj;
        h = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    st[0] += a; st[1] += b; st[2] += c; st[3] += d;
    st[4] += e; st[5] += f; st[6] += g; st[7] += h;
}

void orc_sha256(const uint8_t *data, size_t len, uint8_t out[32]) {
    uint32_t st[8];
    memcpy(st, IV8, sizeof st);
    size_t off = 0;
    while (len - off >= 64) {
        sha256_block(st, data + off);
        off += 64;
    }
    uint8_t tail[128];
    size_t rem = len - off;
    memset(tail, 0, sizeof tail);
    memcpy(tail, data + off, rem);
    tail[rem] = 0x80;
    size_t tl = (rem + 9 <= 64) ? 64 : 128;
    uint64_t bits = (uint64_t)len * 8;
    for (int i = 0; i < 8; ++i) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
    sha256_block(st, tail);
    if (tl == 128) sha256_block(st, tail + 64);
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)(st[i] >> 24);
        out[4 * i + 1] = (uint8_t)(st[i] >> 16);
        out[4 * i + 2] = (uint8_t)(st[i] >> 8);
        out[4 * i + 3] = (uint8_t)st[i];
    }
}

/* ========================================================================
 * BLAKE3 (the `blake3` 1.8.7 crate; specification restated).  Used with
 * the crate's tree semantics by flock-core/src/merkle.rs:160-201:
 *   leaf   = Hasher::new().update(leaf).finalize_non_root()
 *   parent = merge_subtrees_non_root(l, r, Mode::Hash)
 * ======================================================================== */
enum { B3_CHUNK_START = 1, B3_CHUNK_END = 2, B3_PARENT = 4, B3_ROOT = 8 };
static const int B3_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

#define B3G(a, b, c, d, x, y)                 \
    do {                                      \
        s[a] = s[a] + s[b] + (x);             \
        s[d] = rotr32(s[d] ^ s[a], 16);       \
        s[c] = s[c] + s[d];                   \
        s[b] = rotr32(s[b] ^ s[c], 12);       \
        s[a] = s[a] + s[b] + (y);             \
        s[d] = rotr32(s[d] ^ s[a], 8);        \
        s[c] = s[c] + s[d];                   \
        s[b] = rotr32(s[b] ^ s[c], 7);        \
    } while (0)

static void b3_compress(const uint32_t cv[8], const uint8_t block[64], uint64_t counter,
                        uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t m[16], s[16];
    for (int i = 0; i < 16; ++i)
        m[i] = (uint32_t)block[4 * i] | ((uint32_t)block[4 * i + 1] << 8) |
               ((uint32_t)block[4 * i + 2] << 16) | ((uint32_t)block[4 * i + 3] << 24);
    for (int i = 0; i < 8; ++i) s[i] = cv[i];
    s[8] = IV8[0]; s[9] = IV8[1]; s[10] = IV8[2]; s[11] = IV8[3];
    s[12] = (uint32_t)counter;
    s[13] = (uint32_t)(counter >> 32);
    s[14] = block_len;
    s[15] = flags;
    for (int r = 0; r < 7; ++r) {
        B3G(0, 4, 8, 12, m[0], m[1]);
        B3G(1, 5, 9, 13, m[2], m[3]);
        B3G(2, 6, 10, 14, m[4], m[5]);
        B3G(3, 7, 11, 15, m[6], m[7]);
        B3G(0, 5, 10, 15, m[8], m[9]);
        B3G(1, 6, 11, 12, m[10], m[11]);
        B3G(2, 7, 8, 13, m[12], m[13]);
        B3G(3, 4, 9, 14, m[14], m[15]);
        if (r < 6) {
            uint32_t p[16];
            for (int i = 0; i < 16; ++i) p[i] = m[B3_PERM[i]];
            memcpy(m, p, sizeof p);
        }
    }
    for (int i = 0; i < 8; ++i) {
        out[i] = s[i] ^ s[i + 8];
        out[i + 8] = s[i + 8] ^ cv[i];
    }
}

static void cv_to_bytes(const uint32_t w[8], uint8_t out[32]) {
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)w[i];
        out[4 * i + 1] = (uint8_t)(w[i] >> 8);
        out[4 * i + 2] = (uint8_t)(w[i] >> 16);
        out[4 * i + 3] = (uint8_t)(w[i] >> 24);
    }
}
static void cv_from_bytes(const uint8_t b[32], uint32_t w[8]) {
    for (int i = 0; i < 8; ++i)
        w[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) |
               ((uint32_t)b[4 * i + 2] << 16) | ((uint32_t)b[4 * i + 3] << 24);
}

/* Output CV of one chunk (<= 1024 bytes) with chunk counter `counter`;
 * `extra_flags` is ORed into the last block (ROOT for a one-chunk root). */
static void b3_chunk(const uint8_t *data, size_t len, uint64_t counter, uint32_t extra_flags,
                     uint32_t out[8]) {
    uint32_t cv[8];
    memcpy(cv, IV8, sizeof cv);
    size_t nblocks = len == 0 ? 1 : (len + 63) / 64;
    for (size_t b = 0; b < nblocks; ++b) {
        uint8_t blk[64];
        memset(blk, 0, 64);
        size_t off = b * 64, bl = len - off < 64 ? len - off : 64;
        if (len == 0) bl = 0;
        memcpy(blk, data + off, bl);
        uint32_t flags = 0;
        if (b == 0) flags |= B3_CHUNK_START;
        if (b == nblocks - 1) flags |= B3_CHUNK_END | extra_flags;
        uint32_t o[16];
        b3_compress(cv, blk, counter, (uint32_t)bl, flags, o);
        memcpy(cv, o, 32);
    }
    memcpy(out, cv, 32);
}

static void b3_parent(const uint32_t l[8], const uint32_t r[8], uint32_t flags, uint32_t out[8]) {
    uint8_t blk[64];
    cv_to_bytes(l, blk);
    cv_to_bytes(r, blk + 32);
    uint32_t o[16];
    b3_compress(IV8, blk, 0, 64, B3_PARENT | flags, o);
    memcpy(out, o, 32);
}

/* CV of the subtree over chunks [first_chunk, first_chunk + n) of `data`
 * (BLAKE3 tree: the left subtree holds the largest power of two number of
 * chunks that is smaller than n).  `root_flags` applies to the top node. */
static void b3_subtree(const uint8_t *data, size_t len, uint64_t first_chunk, uint32_t root_flags,
                       uint32_t out[8]) {
    size_t n = len <= 1024 ? 1 : (len + 1023) / 1024;
    if (n == 1) {
        b3_chunk(data, len, first_chunk, root_flags, out);
        return;
    }
    size_t left = 1;
    while (left * 2 < n) left *= 2;
    uint32_t l[8], r[8];
    b3_subtree(data, left * 1024, first_chunk, 0, l);
    b3_subtree(data + left * 1024, len - left * 1024, first_chunk + left, 0, r);
    b3_parent(l, r, root_flags, out);
}

void orc_blake3_hash(const uint8_t *data, size_t len, uint8_t out[32]) {
    uint32_t w[8];
    b3_subtree(data, len, 0, B3_ROOT, w);
    cv_to_bytes(w, out);
}

/* Extended output (XOF) of the unkeyed hash: the root node -- the last block
 * of a one-chunk input, else the top parent -- compressed with the ROOT flag
 * and the output block index as its counter; every output block is all 16
 * state words (the `blake3` crate's finalize_xof used by BitZ's
 * Blake3Transcript, src/transcript/mod.rs:49-52). */
void orc_blake3_xof(const uint8_t *data, size_t len, uint8_t *out, size_t out_len) {
    uint32_t cv[8];
    uint8_t blk[64];
    uint32_t block_len, flags;
    memset(blk, 0, 64);
    if (len <= 1024) {
        memcpy(cv, IV8, sizeof cv);
        size_t nblocks = len == 0 ? 1 : (len + 63) / 64;
        for (size_t b = 0; b + 1 < nblocks; ++b) {
            uint32_t o[16];
            b3_compress(cv, data + 64 * b, 0, 64, b == 0 ? B3_CHUNK_START : 0, o);
            memcpy(cv, o, 32);
        }
        size_t off = 64 * (nblocks - 1);
        block_len = (uint32_t)(len - off);
        memcpy(blk, data + off, block_len);
        flags = (nblocks == 1 ? B3_CHUNK_START : 0) | B3_CHUNK_END;
    } else {
        size_t n = (len + 1023) / 1024, left = 1;
        while (left * 2 < n) left *= 2;
        uint32_t l[8], r[8];
        b3_subtree(data, left * 1024, 0, 0, l);
        b3_subtree(data + left * 1024, len - left * 1024, left, 0, r);
        memcpy(cv, IV8, sizeof cv);
        cv_to_bytes(l, blk);
        cv_to_bytes(r, blk + 32);
        block_len = 64;
        flags = B3_PARENT;
    }
    for (uint64_t t = 0; 64 * t < out_len; ++t) {
        uint32_t o[16];
        b3_compress(cv, blk, t, block_len, flags | B3_ROOT, o);
        for (int i = 0; i < 64 && 64 * t + i < out_len; ++i)
            out[64 * t + i] = (uint8_t)(o[i / 4] >> (8 * (i % 4)));
    }
}

/* Proof of work (BitZ src/utils/blake3x4.rs:42-60): blake3(prefix || nonce_le)
 * has at least `bits` leading zero bits, counted from the most significant bit
 * of byte 0. */
int orc_pow_ok(const uint8_t *prefix, size_t plen, uint64_t nonce, unsigned bits) {
    uint8_t buf[64], h[32];
    memcpy(buf, prefix, plen);
    for (int i = 0; i < 8; ++i) buf[plen + i] = (uint8_t)(nonce >> (8 * i));
    orc_blake3_hash(buf, plen + 8, h);
    unsigned acc = 0;
    for (int i = 0; i < 32; ++i) {
        if (h[i] == 0) {
            acc += 8;
            continue;
        }
        unsigned b = h[i], lz = 0;
        while (!(b & 0x80)) {
            ++lz;
            b <<= 1;
        }
        acc += lz;
        break;
    }
    return acc >= bits;
}

/* The smallest nonce in [start, end) passing orc_pow_ok (serial scan,
 * first_pow_nonce of blake3x4.rs); UINT64_MAX when none. */
uint64_t orc_pow_first_nonce(const uint8_t *prefix, size_t plen, uint64_t start, uint64_t end,
                             unsigned bits) {
    for (uint64_t n = start; n < end; ++n)
        if (orc_pow_ok(prefix, plen, n, bits)) return n;
    return UINT64_MAX;
}

void orc_blake3_leaf_cv(const uint8_t *data, size_t len, uint8_t out[32]) {
    uint32_t w[8];
    b3_subtree(data, len, 0, 0, w);
    cv_to_bytes(w, out);
}

/* Non-root CV of a power-of-two run of whole chunks that starts at chunk
 * `first_chunk` of a larger input (the BLAKE3 specification's tree: a chunk's
 * counter is its index in the whole input, and an aligned power-of-two run of
 * chunks is one node of the whole input's tree, merged non-root like the
 * PARENT nodes of merkle.rs:160-201).  One row of a lane shard is such a run
 * inside its leaf. */
void orc_blake3_subtree_cv(const uint8_t *data, size_t len, uint64_t first_chunk,
                           uint8_t out[32]) {
    uint32_t w[8];
    b3_subtree(data, len, first_chunk, 0, w);
    cv_to_bytes(w, out);
}

/* orc_blake3_subtree_cv of each of n_rows consecutive rows of row_len bytes. */
void orc_blake3_rows_subtree_cvs(const uint8_t *rows, size_t n_rows, size_t row_len,
                                 uint64_t first_chunk, uint8_t *out) {
    for (size_t i = 0; i < n_rows; ++i)
        orc_blake3_subtree_cv(rows + i * row_len, row_len, first_chunk, out + 32 * i);
}

void orc_blake3_parent_cv(const uint8_t l[32], const uint8_t r[32], uint8_t out[32]) {
    uint32_t lw[8], rw[8], o[8];
    cv_from_bytes(l, lw);
    cv_from_bytes(r, rw);
    b3_parent(lw, rw, 0, o);
    cv_to_bytes(o, out);
}

/* hash_leaf / hash_pair (merkle.rs:203-232). */
void orc_hash_leaf(const uint8_t *data, size_t len, int kind, uint8_t out[32]) {
    if (kind == 1) orc_blake3_leaf_cv(data, len, out);
    else orc_sha256(data, len, out);
}

void orc_hash_pair(const uint8_t l[32], const uint8_t r[32], int kind, uint8_t out[32]) {
    if (kind == 1) {
        orc_blake3_parent_cv(l, r, out);
    } else {
        uint8_t cat[64];
        memcpy(cat, l, 32);
        memcpy(cat + 32, r, 32);
        orc_sha256(cat, 64, out);
    }
}

/* ========================================================================
 * Merkle -- flock-core/src/merkle.rs:558-596 (tree), :688-741 (multi-proof),
 * :749-817 (multi-proof verify).
 * ======================================================================== */
struct leaves_ctx { const uint8_t *data; size_t leaf; int kind; uint8_t *tree; };
static void leaves_range(void *p, size_t lo, size_t hi) {
    struct leaves_ctx *c = (struct leaves_ctx *)p;
    for (size_t i = lo; i < hi; ++i)
        orc_hash_leaf(c->data + i * c->leaf, c->leaf, c->kind, c->tree + 32 * i);
}
struct pairs_ctx { const uint8_t *rd; uint8_t *wr; int kind; };
static void pairs_range(void *p, size_t lo, size_t hi) {
    struct pairs_ctx *c = (struct pairs_ctx *)p;
    for (size_t i = lo; i < hi; ++i)
        orc_hash_pair(c->rd + 64 * i, c->rd + 64 * i + 32, c->kind, c->wr + 32 * i);
}

void orc_merkle_tree(const uint8_t *data, size_t data_len, size_t num_leaves, int kind,
                     uint8_t *tree, int n_threads) {
    size_t leaf = data_len / num_leaves;
    struct leaves_ctx lc = {data, leaf, kind, tree};
    parallel_for(num_leaves, n_threads, leaves_range, &lc);
    size_t rd = 0, len = num_leaves;
    while (len > 1) {
        struct pairs_ctx pc = {tree + 32 * rd, tree + 32 * (rd + len), kind};
        parallel_for(len / 2, len >= 1024 ? n_threads : 1, pairs_range, &pc);
        rd += len;
        len >>= 1;
    }
}

/* The levels above given leaf hashes (tree[0 .. num_leaves) already holds
 * the leaves): the same flat layout and pair hashing as orc_merkle_tree. */
void orc_merkle_tree_from_leaves(uint8_t *tree, size_t num_leaves, int kind) {
    size_t rd = 0, len = num_leaves;
    while (len > 1) {
        struct pairs_ctx pc = {tree + 32 * rd, tree + 32 * (rd + len), kind};
        parallel_for(len / 2, 1, pairs_range, &pc);
        rd += len;
        len >>= 1;
    }
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

size_t orc_merkle_multi_proof(const uint8_t *tree, size_t num_leaves, const uint64_t *positions,
                              size_t q, uint8_t *out) {
    if (q == 0 || num_leaves == 1) return 0;
    uint64_t *act = (uint64_t *)malloc(sizeof(uint64_t) * q);
    memcpy(act, positions, sizeof(uint64_t) * q);
    qsort(act, q, sizeof(uint64_t), cmp_u64);
    size_t n = 0;
    for (size_t i = 0; i < q; ++i)
        if (n == 0 || act[n - 1] != act[i]) act[n++] = act[i];
    size_t emitted = 0, level_start = 0, level_len = num_leaves;
    while (level_len > 1) {
        size_t nn = 0, i = 0;
        while (i < n) {
            uint64_t p = act[i];
            int sib = (i + 1 < n) && act[i + 1] == (p ^ 1);
            if (sib) {
                i += 2;
            } else {
                memcpy(out + 32 * emitted, tree + 32 * (level_start + (p ^ 1)), 32);
                emitted++;
                i += 1;
            }
            act[nn++] = p >> 1;
        }
        n = nn;
        level_start += level_len;
        level_len >>= 1;
    }
    free(act);
    return emitted;
}

int orc_verify_merkle_multi_proof(const uint8_t root[32], size_t num_leaves,
                                  const uint64_t *pos, const uint8_t *leaf_hashes, size_t q,
                                  const uint8_t *proof, size_t n_proof, int kind) {
    if (num_leaves == 0 || (num_leaves & (num_leaves - 1))) return 0;
    if (q == 0) return n_proof == 0;
    for (size_t i = 0; i < q; ++i) {
        if (pos[i] >= num_leaves) return 0;
        if (i > 0 && pos[i - 1] >= pos[i]) return 0;
    }
    if (num_leaves == 1) return n_proof == 0 && memcmp(leaf_hashes, root, 32) == 0;
    uint64_t *p = (uint64_t *)malloc(sizeof(uint64_t) * q);
    uint8_t *h = (uint8_t *)malloc(32 * q);
    memcpy(p, pos, sizeof(uint64_t) * q);
    memcpy(h, leaf_hashes, 32 * q);
    size_t n = q, used = 0, level_len = num_leaves;
    int ok = 1;
    while (level_len > 1 && ok) {
        size_t nn = 0, i = 0;
        while (i < n) {
            uint8_t l[32], r[32];
            if (i + 1 < n && p[i + 1] == (p[i] ^ 1)) {
                memcpy(l, h + 32 * i, 32);
                memcpy(r, h + 32 * (i + 1), 32);
                i += 2;
            } else {
                if (used >= n_proof) { ok = 0; break; }
                const uint8_t *sib = proof + 32 * used++;
                if (p[i] & 1) { memcpy(l, sib, 32); memcpy(r, h + 32 * i, 32); }
                else { memcpy(l, h + 32 * i, 32); memcpy(r, sib, 32); }
                i += 1;
            }
            uint64_t parent = p[i - 1] >> 1;
            orc_hash_pair(l, r, kind, h + 32 * nn);
            p[nn++] = parent;
        }
        n = nn;
        level_len >>= 1;
    }
    if (ok) ok = (used == n_proof) && n == 1 && memcmp(h, root, 32) == 0;
    free(p);
    free(h);
    return ok;
}

/* ========================================================================
 * Commit -- flock-core/src/pcs/commit.rs:180-315
 * ======================================================================== */
int orc_commit(const uint64_t *msg, int log_msg_len, int log_inv_rate, int log_batch_size,
               int hash_kind, uint64_t *codeword, uint8_t *tree, uint8_t root[32],
               int n_threads) {
    /* validate (:125-136): log_batch_size <= log_msg_len, log_inv_rate >= 1 */
    if (log_batch_size > log_msg_len || log_inv_rate < 1) return -1;
    int log_dim = log_msg_len - log_batch_size;
    int k_code = log_dim + log_inv_rate;
    size_t num_ntts = (size_t)1 << log_batch_size;
    size_t msg_len = (size_t)1 << log_msg_len;
    size_t reps = (size_t)1 << log_inv_rate;
    /* replicate_message_fill (:239-258): 2^r copies == state after r layers */
    for (size_t r = 0; r < reps; ++r)
        memcpy(codeword + 2 * r * msg_len, msg, sizeof(uint64_t) * 2 * msg_len);
    /* finalize_commit (:262-315): NTT from layer r, Merkle over positions;
     * several threads run the reference's blocked structure */
    if (n_threads > 1)
        orc_ntt_forward_interleaved_blocked(codeword, num_ntts, k_code, log_inv_rate, n_threads);
    else
        orc_ntt_forward_interleaved(codeword, num_ntts, k_code, log_inv_rate, 1);
    size_t n_leaves = (size_t)1 << k_code;
    orc_merkle_tree((const uint8_t *)codeword, 16 * msg_len * reps, n_leaves, hash_kind, tree,
                    n_threads);
    memcpy(root, tree + 32 * (2 * n_leaves - 2), 32);
    return 0;
}

/* ========================================================================
 * Sumcheck folds -- flock-core/src/pcs/ligerito.rs
 * ======================================================================== */

/* partial_eval_lsb (:1678-1695): pair (2i, 2i+1) -> v0*(1+r) + v1*r. */
void orc_partial_eval_lsb(const uint64_t *evals, size_t n, const uint64_t *rs, size_t k,
                          uint64_t *out) {
    uint64_t *cur = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (n ? n : 1));
    memcpy(cur, evals, sizeof(uint64_t) * 2 * n);
    size_t len = n;
    for (size_t s = 0; s < k; ++s) {
        const uint64_t *r = rs + 2 * s;
        uint64_t opr[2] = {r[0] ^ 1, r[1]};
        size_t half = len / 2;
        for (size_t i = 0; i < half; ++i) {
            uint64_t a[2], b[2];
            gf_mul(cur + 4 * i, opr, a);
            gf_mul(cur + 4 * i + 2, r, b);
            cur[2 * i] = a[0] ^ b[0];
            cur[2 * i + 1] = a[1] ^ b[1];
        }
        len = half;
    }
    memcpy(out, cur, sizeof(uint64_t) * 2 * len);
    free(cur);
}

/* round_msg_lsb (:2500-2537): u0 = sum f0*b0, u2 = sum (f0+f1)*(b0+b1). */
void orc_round_msg_lsb(const uint64_t *f, const uint64_t *b, size_t n, uint64_t u0[2],
                       uint64_t u2[2]) {
    uint64_t a0[2] = {0, 0}, a2[2] = {0, 0};
    for (size_t j = 0; j < n / 2; ++j) {
        const uint64_t *f0 = f + 4 * j, *f1 = f0 + 2, *b0 = b + 4 * j, *b1 = b0 + 2;
        uint64_t p[2], fs[2] = {f0[0] ^ f1[0], f0[1] ^ f1[1]}, bs[2] = {b0[0] ^ b1[0], b0[1] ^ b1[1]};
        gf_mul(f0, b0, p);
        a0[0] ^= p[0]; a0[1] ^= p[1];
        gf_mul(fs, bs, p);
        a2[0] ^= p[0]; a2[1] ^= p[1];
    }
    u0[0] = a0[0]; u0[1] = a0[1];
    u2[0] = a2[0]; u2[1] = a2[1];
}

/* fold_and_msg_lsb (:2634-2735): nf[j] = f0 + (f0+f1)*r (same for b), then
 * the next-round message over the folded arrays (zero when half < 2). */
void orc_fold_and_msg_lsb(const uint64_t *f, const uint64_t *b, size_t n, const uint64_t r[2],
                          uint64_t *nf, uint64_t *nb, uint64_t u0[2], uint64_t u2[2]) {
    size_t half = n / 2;
    for (size_t j = 0; j < half; ++j) {
        uint64_t d[2], p[2];
        d[0] = f[4 * j] ^ f[4 * j + 2];
        d[1] = f[4 * j + 1] ^ f[4 * j + 3];
        gf_mul(d, r, p);
        nf[2 * j] = f[4 * j] ^ p[0];
        nf[2 * j + 1] = f[4 * j + 1] ^ p[1];
        d[0] = b[4 * j] ^ b[4 * j + 2];
        d[1] = b[4 * j + 1] ^ b[4 * j + 3];
        gf_mul(d, r, p);
        nb[2 * j] = b[4 * j] ^ p[0];
        nb[2 * j + 1] = b[4 * j + 1] ^ p[1];
    }
    if (half >= 2) {
        orc_round_msg_lsb(nf, nb, half, u0, u2);
    } else {
        u0[0] = u0[1] = u2[0] = u2[1] = 0;
    }
}

/* ========================================================================
 * Ring switch helpers -- BitZ src/ligerito.rs, src/poly/utils.rs
 * ======================================================================== */

/* build_eq_x_r_vec (src/poly/utils.rs:46-120): eq[sum x_i 2^i] =
 * prod_i (x_i ? r_i : 1 + r_i). */
void orc_build_eq_lsb(const uint64_t *point, size_t k, uint64_t *out) {
    out[0] = 1;
    out[1] = 0;
    for (size_t i = 0; i < k; ++i) {
        size_t half = (size_t)1 << i;
        for (size_t j = 0; j < half; ++j) {
            uint64_t one[2];
            gf_mul(out + 2 * j, point + 2 * i, one);
            out[2 * (half + j)] = one[0];
            out[2 * (half + j) + 1] = one[1];
            out[2 * j] ^= one[0];
            out[2 * j + 1] ^= one[1];
        }
    }
}

/* s_{i+1}(x) = s_i(x)^2 + s_i(v_i) s_i(x)  (ligerito.rs:1712-1715) */
static void next_s(const uint64_t s[2], const uint64_t s_root[2], uint64_t out[2]) {
    uint64_t a[2], b[2];
    gf_mul(s, s, a);
    gf_mul(s_root, s, b);
    out[0] = a[0] ^ b[0];
    out[1] = a[1] ^ b[1];
}

/* The basis a level's queries induce, in the dense form of
 * induce_sumcheck_poly (flock-core/src/pcs/ligerito.rs:1968-2072):
 * basis[j] = sum_i w[i] * W^_j(q_i), where W^_j(x) = prod_{k: bit_k(j)} W^_k(x)
 * are the normalized LCH novel-basis polynomials at the field element q_i
 * (= Gf128::new(q_i, 0)); s_k(v_k) from eval_sk_at_vks (:1720-1747), the
 * products as evaluate_scaled_basis_inplace (:1749-1785). */
void orc_induce_basis(int log_n, const uint64_t *queries, size_t nq, const uint64_t *w,
                      uint64_t *basis) {
    const size_t n = (size_t)1 << log_n;
    uint64_t sks_vks[2 * 65], inv[2 * 65];
    memset(sks_vks, 0, sizeof sks_vks);
    sks_vks[0] = 1;
    uint64_t layer[2 * 64];
    for (int i = 1; i <= log_n; ++i) {
        layer[2 * (i - 1)] = (uint64_t)1 << i;
        layer[2 * (i - 1) + 1] = 0;
    }
    int cur_len = log_n;
    for (int i = 0; i < log_n; ++i) {
        for (int j = 0; j < cur_len; ++j) {
            uint64_t t[2];
            next_s(layer + 2 * j, sks_vks + 2 * i, t);
            if (j == 0) {
                sks_vks[2 * (i + 1)] = t[0];
                sks_vks[2 * (i + 1) + 1] = t[1];
            } else {
                layer[2 * (j - 1)] = t[0];
                layer[2 * (j - 1) + 1] = t[1];
            }
        }
        --cur_len;
    }
    for (int k = 0; k <= log_n; ++k) {
        if (sks_vks[2 * k] | sks_vks[2 * k + 1])
            orc_gf_inv(sks_vks + 2 * k, inv + 2 * k);
        else
            inv[2 * k] = inv[2 * k + 1] = 0;
    }
    memset(basis, 0, 16 * n);
    uint64_t *local = (uint64_t *)malloc(16 * n);
    uint64_t sx[2 * 64];
    for (size_t qi = 0; qi < nq; ++qi) {
        if (log_n > 0) {
            sx[0] = queries[qi];
            sx[1] = 0;
            for (int i = 1; i < log_n; ++i) next_s(sx + 2 * (i - 1), sks_vks + 2 * (i - 1), sx + 2 * i);
            for (int i = 0; i < log_n; ++i) {
                uint64_t t[2];
                gf_mul(sx + 2 * i, inv + 2 * i, t);
                sx[2 * i] = t[0];
                sx[2 * i + 1] = t[1];
            }
        }
        local[0] = w[2 * qi];
        local[1] = w[2 * qi + 1];
        for (int k = 0; k < log_n; ++k) {
            const size_t len = (size_t)1 << k;
            for (size_t i = 0; i < len; ++i) gf_mul(sx + 2 * k, local + 2 * i, local + 2 * (i + len));
        }
        for (size_t j = 0; j < 2 * n; ++j) basis[j] ^= local[j];
    }
    free(local);
}

/* sv_fold_mfr (src/ligerito.rs:317-375) by its defining identity:
 * s[j] = sum_y eq[y] * bit_j(P[y]). */
void orc_sv_fold(const uint64_t *packed, size_t n, const uint64_t *eq, uint64_t *sv) {
    memset(sv, 0, sizeof(uint64_t) * 256);
    for (size_t y = 0; y < n; ++y) {
        for (int j = 0; j < 128; ++j) {
            uint64_t w = packed[2 * y + (j >> 6)];
            if ((w >> (j & 63)) & 1) {
                sv[2 * j] ^= eq[2 * y];
                sv[2 * j + 1] ^= eq[2 * y + 1];
            }
        }
    }
}

/* phi_from_words (src/ligerito.rs:384-427, slow form at :474-487):
 * out[y] = sum_{u : bit_u(eq_hi[y])} eq_r2[u]. */
void orc_phi_from_words(const uint64_t *eq_hi, size_t n, const uint64_t *eq_r2, uint64_t *out) {
    for (size_t y = 0; y < n; ++y) {
        uint64_t a0 = 0, a1 = 0;
        for (int u = 0; u < 128; ++u) {
            uint64_t w = eq_hi[2 * y + (u >> 6)];
            if ((w >> (u & 63)) & 1) {
                a0 ^= eq_r2[2 * u];
                a1 ^= eq_r2[2 * u + 1];
            }
        }
        out[2 * y] = a0;
        out[2 * y + 1] = a1;
    }
}

/* ========================================================================
 * ChaCha20 (RFC 8439 section 2.3) -- synthetic inputs.
 * ======================================================================== */
static inline uint32_t rotl32(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }
#define QR(a, b, c, d)                                  \
    do {                                                \
        x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16);   \
        x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12);   \
        x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);    \
        x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);    \
    } while (0)

void orc_chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3],
                        uint8_t out[64]) {
    uint32_t st[16] = {0x61707865, 0x3320646e, 0x79622d32, 0x6b206574};
    for (int i = 0; i < 8; ++i) st[4 + i] = key[i];
    st[12] = counter;
    st[13] = nonce[0];
    st[14] = nonce[1];
    st[15] = nonce[2];
    uint32_t x[16];
    memcpy(x, st, sizeof x);
    for (int i = 0; i < 10; ++i) {
        QR(0, 4, 8, 12); QR(1, 5, 9, 13); QR(2, 6, 10, 14); QR(3, 7, 11, 15);
        QR(0, 5, 10, 15); QR(1, 6, 11, 12); QR(2, 7, 8, 13); QR(3, 4, 9, 14);
    }
    for (int i = 0; i < 16; ++i) {
        uint32_t v = x[i] + st[i];
        out[4 * i] = (uint8_t)v;
        out[4 * i + 1] = (uint8_t)(v >> 8);
        out[4 * i + 2] = (uint8_t)(v >> 16);
        out[4 * i + 3] = (uint8_t)(v >> 24);
    }
}

void orc_chacha_words(uint64_t seed, uint64_t first_word, uint64_t *out, size_t n_words) {
    uint32_t key[8] = {(uint32_t)seed, (uint32_t)(seed >> 32), 0, 0, 0, 0, 0, 0};
    uint32_t nonce[3] = {0, 0, 0};
    uint8_t blk[64];
    uint64_t cached = ~0ULL;
    for (size_t i = 0; i < n_words; ++i) {
        uint64_t w = first_word + i;
        uint64_t b = w >> 2;
        if (b != cached) {
            orc_chacha20_block(key, (uint32_t)b, nonce, blk);
            cached = b;
        }
        const uint8_t *p = blk + 16 * (w & 3);
        uint64_t lo = 0, hi = 0;
        for (int k = 7; k >= 0; --k) {
            lo = (lo << 8) | p[k];
            hi = (hi << 8) | p[8 + k];
        }
        out[2 * i] = lo;
        out[2 * i + 1] = hi;
    }
}
