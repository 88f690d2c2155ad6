// Host runtime behind the C ABI (include/bitz_gpu.h): device context, memory
// budget, commit pipeline, openings (rows, multi-proofs), folds, batched
// CUDA-graph commits and the schedule autotuner.  Every entry point converts
// failures into a status code; nothing throws across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "bz_internal.h"
#include "runtime.h"

using namespace bz;

// ===========================================================================
// Host GF(2^128) (twiddle tables only).
// ===========================================================================
namespace bz {
typedef unsigned __int128 u128;
static inline u128 hclmul64(uint64_t a, uint64_t b) {
    u128 acc = 0;
    u128 aa = a;
    while (b) {
        if (b & 1) acc ^= aa;
        aa <<= 1;
        b >>= 1;
    }
    return acc;
}
void hgf_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]) {
    const u128 l = hclmul64(a[0], b[0]);
    const u128 h = hclmul64(a[1], b[1]);
    const u128 m = hclmul64(a[0] ^ a[1], b[0] ^ b[1]) ^ l ^ h;
    uint64_t r0 = (uint64_t)l, r1 = (uint64_t)(l >> 64) ^ (uint64_t)m;
    uint64_t r2 = (uint64_t)h ^ (uint64_t)(m >> 64), r3 = (uint64_t)(h >> 64);
    // fold r2, r3 by X^128 = X^7 + X^2 + X + 1
    auto tg = [](uint64_t w) -> u128 {
        u128 x = w;
        return x ^ (x << 1) ^ (x << 2) ^ (x << 7);
    };
    const u128 f2 = tg(r2), f3 = tg(r3);
    r0 ^= (uint64_t)f2;
    r1 ^= (uint64_t)(f2 >> 64) ^ (uint64_t)f3;
    r0 ^= (uint64_t)tg((uint64_t)(f3 >> 64));
    out[0] = r0;
    out[1] = r1;
}
void hgf_inv(const uint64_t a[2], uint64_t out[2]) {
    // a^(2^128 - 2) by the addition chain a^(2^k - 1) -> a^(2^(k+1) - 1)
    uint64_t acc[2] = {a[0], a[1]};
    for (int k = 1; k < 127; ++k) {
        uint64_t sq[2];
        hgf_mul(acc, acc, sq);
        hgf_mul(sq, a, acc);
    }
    hgf_mul(acc, acc, out);
}
}  // namespace bz

// ===========================================================================
// Context helpers.
// ===========================================================================
namespace bz {

int set_err(bz_ctx *ctx, int code, const char *what, cudaError_t e) {
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->err_mu);
        ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return code;
}
int set_msg(bz_ctx *ctx, int code, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->err_mu);
        ctx->last_error = msg;
    }
    return code;
}

int shape_from_params(const bz_params *p, Shape &s, size_t n_words, std::string &why) {
    if (!p) {
        why = "params is null";
        return BZ_ERR_ARG;
    }
    if (p->hash_kind > 1) {
        why = "hash_kind must be 0 (SHA-256) or 1 (BLAKE3)";
        return BZ_ERR_ARG;
    }
    // PcsParams::validate (commit.rs:125-136) and the length assert (:182).
    if (p->log_batch_size > p->log_msg_len) {
        why = "m too small: need log_msg_len >= log_batch_size";
        return BZ_ERR_SHAPE;
    }
    if (p->log_inv_rate < 1) {
        why = "log_inv_rate must be >= 1 for a non-trivial RS code";
        return BZ_ERR_SHAPE;
    }
    if (p->log_msg_len + p->log_inv_rate > 40 || p->log_msg_len - p->log_batch_size > 62) {
        why = "shape too large";
        return BZ_ERR_SHAPE;
    }
    if (n_words != ((size_t)1 << p->log_msg_len)) {
        why = "message length must be 2^log_msg_len";
        return BZ_ERR_SHAPE;
    }
    s.log_msg_len = (int)p->log_msg_len;
    s.log_inv_rate = (int)p->log_inv_rate;
    s.log_lanes = (int)p->log_batch_size;
    s.hash_kind = (int)p->hash_kind;
    return BZ_OK;
}

int dev_alloc(bz_ctx *ctx, size_t bytes, void **p, bool budgeted) {
    if (bytes == 0) bytes = 16;
    if (budgeted) {
        uint64_t cur = ctx->in_use.load();
        if (cur + bytes > ctx->budget)
            return set_msg(ctx, BZ_ERR_NOMEM, "memory budget exceeded");
    }
    cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, BZ_ERR_NOMEM, "cudaMallocAsync", e);
    }
    if (budgeted) ctx->in_use += bytes;
    return BZ_OK;
}

void dev_free(bz_ctx *ctx, void *p, size_t bytes, bool budgeted) {
    if (!p) return;
    cudaFreeAsync(p, ctx->stream);
    if (budgeted) ctx->in_use -= (bytes == 0 ? 16 : bytes);
}

int ensure_scratch(bz_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return BZ_OK;
    if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->stream);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    void *p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, BZ_ERR_NOMEM, "scratch", e);
    }
    ctx->scratch = (uint8_t *)p;
    ctx->scratch_bytes = bytes;
    return BZ_OK;
}

int get_twiddles(bz_ctx *ctx, int ell, const uint4 **out) {
    std::lock_guard<std::mutex> g(ctx->tw_mu);
    auto it = ctx->twiddles.find(ell);
    if (it != ctx->twiddles.end()) {
        *out = it->second;
        return BZ_OK;
    }
    std::vector<uint64_t> heap = twiddle_heap(ell);
    void *d = nullptr;
    BZ_CUDA(ctx, cudaMalloc(&d, heap.size() * 8));
    BZ_CUDA(ctx, cudaMemcpy(d, heap.data(), heap.size() * 8, cudaMemcpyHostToDevice));
    ctx->twiddles[ell] = (const uint4 *)d;
    *out = (const uint4 *)d;
    return BZ_OK;
}

uint32_t schedule_for(bz_ctx *ctx, const Shape &s) {
    std::lock_guard<std::mutex> g(ctx->sched_mu);
    const uint64_t key = shape_key(s);
    auto it = ctx->schedules.find(key);
    if (it != ctx->schedules.end()) return it->second;
    return default_schedule(s);
}

// Every live commitment of every context: bz_commitment_free checks a handle
// here before touching it, so a handle whose context was destroyed (which
// frees the context's commitments) is refused instead of used after free.
static std::mutex g_handles_mu;
static std::set<const bz_commitment *> g_handles;

// Allocate a commitment's resident buffers (budgeted).  Without a codeword
// the handle holds only a tree (the global tree of a lane-sharded commit,
// whose codeword stays split over the ranks).
int alloc_commitment(bz_ctx *ctx, const Shape &s, bz_commitment **out, bool with_codeword) {
    bz_commitment *c = new bz_commitment();
    c->ctx = ctx;
    c->shape = s;
    c->cw_bytes = with_codeword ? s.cw_words() * 16 : 0;
    c->tree_bytes = s.tree_nodes() * 32;
    int rc = with_codeword ? dev_alloc(ctx, c->cw_bytes, (void **)&c->d_cw, true) : BZ_OK;
    if (rc) {
        delete c;
        return rc;
    }
    rc = dev_alloc(ctx, c->tree_bytes, (void **)&c->d_tree, true);
    if (rc) {
        dev_free(ctx, c->d_cw, c->cw_bytes, true);
        delete c;
        return rc;
    }
    {
        std::lock_guard<std::mutex> g(ctx->live_mu);
        ctx->live.insert(c);
    }
    {
        std::lock_guard<std::mutex> g(g_handles_mu);
        g_handles.insert(c);
    }
    *out = c;
    return BZ_OK;
}

// Enqueue NTT + Merkle for a commitment whose buffers exist.
int enqueue_commit(bz_ctx *ctx, const Shape &s, const uint4 *d_msg, bz_commitment *c,
                   cudaStream_t st, uint32_t schedule) {
    const uint4 *d_tw = nullptr;
    int rc = get_twiddles(ctx, s.k_code(), &d_tw);
    if (rc) return rc;
    const size_t need = merkle_scratch_bytes(s);
    if (need) {
        rc = ensure_scratch(ctx, need);
        if (rc) return rc;
    }
    int n = launch_commit_kernels(ctx, s, schedule, d_msg, c->d_cw, c->d_tree, d_tw, st, nullptr);
    ctx->launches += (uint64_t)n;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(ctx, BZ_ERR_CUDA, "kernel launch", e);
    c->root_ready = false;
    return BZ_OK;
}

bz_aux_stream *get_aux(bz_ctx *ctx, cudaStream_t st) {
    std::lock_guard<std::mutex> g(ctx->aux_mu);
    auto it = ctx->aux.find(st);
    if (it != ctx->aux.end()) return &it->second;
    bz_aux_stream a;
    if (cudaStreamCreateWithFlags(&a.s, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    for (auto &e : a.ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return &(ctx->aux[st] = a);
}

int launch_commit_kernels(bz_ctx *ctx, const Shape &s, uint32_t schedule, const uint4 *d_msg,
                          uint4 *d_cw, uint8_t *d_tree, const uint4 *d_tw, cudaStream_t st,
                          LaunchLog *log) {
    if ((schedule >> SCHED_PIPE_SHIFT) & 3) {
        bz_aux_stream *ax = get_aux(ctx, st);
        if (ax) {
            const int n = launch_commit_pipelined(s, schedule, d_msg, d_cw, d_tree, d_tw, st, ax->s,
                                                  ax->ev, ctx->num_sms, log);
            if (n >= 0) return n;
        }
    }
    int n = launch_ntt(s, schedule, d_msg, d_cw, d_tw, st, ctx->num_sms, log);
    n += launch_merkle(s, d_cw, d_tree, ctx->scratch, st, ctx->num_sms, log);
    return n;
}

int commitment_rows_on(bz_commitment *c, const uint64_t *positions, size_t q, uint64_t *out,
                       cudaStream_t st) {
    bz_ctx *ctx = c->ctx;
    if (!c->d_cw) return set_msg(ctx, BZ_ERR_STATE, "tree-only commitment: no codeword");
    const uint64_t n_pos = c->shape.n_leaves();
    for (size_t i = 0; i < q; ++i)
        if (positions[i] >= n_pos) return set_msg(ctx, BZ_ERR_ARG, "position out of range");
    if (q == 0) return BZ_OK;
    const size_t row_bytes = c->shape.leaf_bytes();
    void *d_pos = nullptr, *d_out = nullptr;
    if (cudaMallocAsync(&d_pos, q * 8, st) != cudaSuccess ||
        cudaMallocAsync(&d_out, q * row_bytes, st) != cudaSuccess) {
        cudaGetLastError();
        if (d_pos) cudaFreeAsync(d_pos, st);
        return set_msg(ctx, BZ_ERR_NOMEM, "opened rows buffer");
    }
    cudaMemcpyAsync(d_pos, positions, q * 8, cudaMemcpyHostToDevice, st);
    ctx->launches += launch_gather_rows(c->d_cw, c->shape.log_lanes, (const uint64_t *)d_pos, q,
                                        (uint4 *)d_out, st);
    cudaMemcpyAsync(out, d_out, q * row_bytes, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d_pos, st);
    cudaFreeAsync(d_out, st);
    BZ_CUDA(ctx, cudaStreamSynchronize(st));
    return BZ_OK;
}

int commitment_multiproof_on(bz_commitment *c, const uint64_t *positions, size_t q, uint8_t *out,
                             size_t cap, size_t *n_hashes, cudaStream_t st) {
    bz_ctx *ctx = c->ctx;
    const uint64_t num_leaves = c->shape.n_leaves();
    *n_hashes = 0;
    if (q == 0 || num_leaves == 1) return BZ_OK;
    // merkle_multi_proof (merkle.rs:688-741): sorted unique positions, walk
    // levels bottom-up, emit the sibling of every node whose sibling is not
    // itself active.
    std::vector<uint64_t> act(positions, positions + q);
    for (uint64_t p : act)
        if (p >= num_leaves) return set_msg(ctx, BZ_ERR_ARG, "position out of range");
    std::sort(act.begin(), act.end());
    act.erase(std::unique(act.begin(), act.end()), act.end());
    std::vector<uint64_t> idx;
    uint64_t level_start = 0, level_len = num_leaves;
    while (level_len > 1) {
        std::vector<uint64_t> next;
        next.reserve(act.size());
        size_t i = 0;
        while (i < act.size()) {
            const uint64_t p = act[i];
            const bool sib = i + 1 < act.size() && act[i + 1] == (p ^ 1);
            if (sib) {
                i += 2;
            } else {
                idx.push_back(level_start + (p ^ 1));
                i += 1;
            }
            next.push_back(p >> 1);
        }
        act.swap(next);
        level_start += level_len;
        level_len >>= 1;
    }
    *n_hashes = idx.size();
    if (!out) return BZ_OK;  // size query
    if (idx.size() > cap) return set_msg(ctx, BZ_ERR_ARG, "multiproof buffer too small");
    if (idx.empty()) return BZ_OK;
    void *d_idx = nullptr, *d_out = nullptr;
    if (cudaMallocAsync(&d_idx, idx.size() * 8, st) != cudaSuccess ||
        cudaMallocAsync(&d_out, idx.size() * 32, st) != cudaSuccess) {
        cudaGetLastError();
        if (d_idx) cudaFreeAsync(d_idx, st);
        return set_msg(ctx, BZ_ERR_NOMEM, "multiproof buffer");
    }
    cudaMemcpyAsync(d_idx, idx.data(), idx.size() * 8, cudaMemcpyHostToDevice, st);
    ctx->launches += launch_gather_nodes(c->d_tree, (const uint64_t *)d_idx, idx.size(),
                                         (uint8_t *)d_out, st);
    cudaMemcpyAsync(out, d_out, idx.size() * 32, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d_idx, st);
    cudaFreeAsync(d_out, st);
    BZ_CUDA(ctx, cudaStreamSynchronize(st));
    return BZ_OK;
}

std::future<int> side_async(bz_ctx *ctx, std::function<int()> job) {
    auto task = std::make_shared<std::packaged_task<int()>>(std::move(job));
    std::future<int> f = task->get_future();
    {
        std::lock_guard<std::mutex> g(ctx->side_mu);
        if (!ctx->side_thread.joinable()) {
            ctx->side_thread = std::thread([ctx] {
                cudaSetDevice(ctx->device);
                std::unique_lock<std::mutex> lk(ctx->side_mu);
                while (true) {
                    ctx->side_cv.wait(lk, [ctx] { return ctx->side_stop || !ctx->side_jobs.empty(); });
                    if (ctx->side_jobs.empty()) return;  // stopping, nothing left
                    std::function<void()> j = std::move(ctx->side_jobs.front());
                    ctx->side_jobs.pop_front();
                    lk.unlock();
                    j();
                    lk.lock();
                }
            });
        }
        ctx->side_jobs.emplace_back([task] { (*task)(); });
    }
    ctx->side_cv.notify_one();
    return f;
}

void side_shutdown(bz_ctx *ctx) {
    {
        std::lock_guard<std::mutex> g(ctx->side_mu);
        ctx->side_stop = true;
    }
    ctx->side_cv.notify_all();
    if (ctx->side_thread.joinable()) ctx->side_thread.join();
}

int fetch_root(bz_commitment *c) {
    bz_ctx *ctx = c->ctx;
    if (c->root_ready) return BZ_OK;
    if (c->done) {
        BZ_CUDA(ctx, cudaEventSynchronize(c->done));
        memcpy(c->root, c->root_slot, 32);
        c->root_ready = true;
        return BZ_OK;
    }
    const uint8_t *src = c->d_tree + (c->shape.tree_nodes() - 1) * 32;
    BZ_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, src, 32, cudaMemcpyDeviceToHost, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    memcpy(c->root, ctx->h_small, 32);
    c->root_ready = true;
    return BZ_OK;
}

}  // namespace bz

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *bz_status_string(int s) {
    switch (s) {
        case BZ_OK: return "ok";
        case BZ_ERR_ARG: return "invalid argument";
        case BZ_ERR_SHAPE: return "invalid shape";
        case BZ_ERR_CUDA: return "CUDA error";
        case BZ_ERR_NOMEM: return "out of device memory / budget";
        case BZ_ERR_BUSY: return "busy";
        case BZ_ERR_TIMEOUT: return "timeout";
        case BZ_ERR_STATE: return "invalid state";
        case BZ_ERR_NOTFOUND: return "not found";
        case BZ_ERR_TRUNCATED: return "proof stream truncated";
        case BZ_ERR_NONCANONICAL: return "proof stream encoded non-minimally";
        case BZ_ERR_DECODE: return "LigeritoProof decode failed";
        default: return "unknown status";
    }
}

const char *bz_last_error(const bz_ctx *ctx) {
    if (!ctx) return "no context";
    return ctx->last_error.c_str();
}

int bz_abi_version(void) { return BZ_ABI_VERSION; }

int bz_ctx_create(int device, uint64_t mem_budget_bytes, bz_ctx **out) {
    if (!out) return BZ_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return BZ_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return BZ_ERR_CUDA;
    bz_ctx *ctx = new bz_ctx();
    ctx->device = device;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    ctx->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return BZ_ERR_CUDA;
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->budget = mem_budget_bytes ? mem_budget_bytes : (uint64_t)(free_b * 0.9);
    init_ntt_kernels();
    init_fold_kernels();
    cudaEventCreate(&ctx->ev0);
    cudaEventCreate(&ctx->ev1);
    if (cudaMallocHost(&ctx->h_small, 4096) != cudaSuccess) {
        delete ctx;
        return BZ_ERR_CUDA;
    }
    if (cudaMalloc(&ctx->d_small, 4096) != cudaSuccess ||
        cudaMemset(ctx->d_small, 0, 4096) != cudaSuccess ||
        cudaHostAlloc(&ctx->h_mbox, 4096, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&ctx->d_mbox, ctx->h_mbox, 0) != cudaSuccess) {
        cudaGetLastError();
        if (ctx->d_small) cudaFree(ctx->d_small);
        if (ctx->h_mbox) cudaFreeHost(ctx->h_mbox);
        cudaFreeHost(ctx->h_small);
        delete ctx;
        return BZ_ERR_CUDA;
    }
    memset(ctx->h_mbox, 0, 4096);
    *out = ctx;
    return BZ_OK;
}

int bz_ctx_destroy(bz_ctx *ctx) {
    if (!ctx) return BZ_ERR_ARG;
    cudaSetDevice(ctx->device);
    side_shutdown(ctx);  // finishes queued side-stream openings first
    cudaStreamSynchronize(ctx->stream);
    std::vector<bz_commitment *> live;
    {
        std::lock_guard<std::mutex> g(ctx->live_mu);
        live.assign(ctx->live.begin(), ctx->live.end());
    }
    for (auto *c : live) bz_commitment_free(c);
    for (auto &kv : ctx->twiddles) cudaFree((void *)kv.second);
    for (auto &kv : ctx->aux) {
        cudaStreamSynchronize(kv.second.s);
        for (auto e : kv.second.ev) cudaEventDestroy(e);
        cudaStreamDestroy(kv.second.s);
    }
    if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_small);
    cudaFreeHost(ctx->h_small);
    cudaFreeHost(ctx->h_mbox);
    cudaEventDestroy(ctx->ev0);
    cudaEventDestroy(ctx->ev1);
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
    cudaStreamSynchronize(ctx->side_stream);
    cudaStreamDestroy(ctx->side_stream);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BZ_OK;
}

void *bz_ctx_stream(bz_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int bz_ctx_synchronize(bz_ctx *ctx) {
    if (!ctx) return BZ_ERR_ARG;
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_ctx_memory(const bz_ctx *ctx, uint64_t *in_use, uint64_t *budget) {
    if (!ctx) return BZ_ERR_ARG;
    if (in_use) *in_use = ctx->in_use.load();
    if (budget) *budget = ctx->budget;
    return BZ_OK;
}

// Stream-ordered on the context stream (the context's memory pool): the
// memory is valid for work enqueued on that stream after the allocation and
// is recycled once the work enqueued before the free has finished.
int bz_device_alloc(bz_ctx *ctx, size_t bytes, void **dptr) {
    if (!ctx || !dptr) return BZ_ERR_ARG;
    BZ_CUDA(ctx, cudaMallocAsync(dptr, bytes ? bytes : 16, ctx->stream));
    return BZ_OK;
}
int bz_device_free(bz_ctx *ctx, void *dptr) {
    if (!ctx) return BZ_ERR_ARG;
    if (dptr) BZ_CUDA(ctx, cudaFreeAsync(dptr, ctx->stream));
    return BZ_OK;
}
int bz_memcpy_h2d(bz_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!ctx) return BZ_ERR_ARG;
    BZ_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}
int bz_memcpy_d2h(bz_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!ctx) return BZ_ERR_ARG;
    BZ_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}
int bz_host_alloc_pinned(size_t bytes, void **hptr) {
    if (!hptr) return BZ_ERR_ARG;
    return cudaMallocHost(hptr, bytes ? bytes : 16) == cudaSuccess ? BZ_OK : BZ_ERR_NOMEM;
}
int bz_host_free_pinned(void *hptr) { return cudaFreeHost(hptr) == cudaSuccess ? BZ_OK : BZ_ERR_CUDA; }

int bz_timer_begin(bz_ctx *ctx) {
    if (!ctx) return BZ_ERR_ARG;
    BZ_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    return BZ_OK;
}
int bz_timer_end(bz_ctx *ctx, float *ms) {
    if (!ctx || !ms) return BZ_ERR_ARG;
    BZ_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    BZ_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    BZ_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return BZ_OK;
}
uint64_t bz_kernel_launches(const bz_ctx *ctx) { return ctx ? ctx->launches.load() : 0; }

// ---- commit ---------------------------------------------------------------
int bz_commit_device_async(bz_ctx *ctx, const uint64_t *d_msg, size_t n_words,
                           const bz_params *params, bz_commitment **out) {
    if (!ctx || !d_msg || !out) return BZ_ERR_ARG;
    *out = nullptr;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, n_words, why);
    if (rc) return set_msg(ctx, rc, why);
    bz_commitment *c = nullptr;
    rc = alloc_commitment(ctx, s, &c);
    if (rc) return rc;
    rc = enqueue_commit(ctx, s, (const uint4 *)d_msg, c, ctx->stream, schedule_for(ctx, s));
    if (rc) {
        bz_commitment_free(c);
        return rc;
    }
    *out = c;
    return BZ_OK;
}

int bz_commit_device(bz_ctx *ctx, const uint64_t *d_msg, size_t n_words, const bz_params *params,
                     bz_commitment **out, uint8_t root[32]) {
    int rc = bz_commit_device_async(ctx, d_msg, n_words, params, out);
    if (rc) return rc;
    rc = fetch_root(*out);
    if (rc) {
        bz_commitment_free(*out);
        *out = nullptr;
        return rc;
    }
    if (root) memcpy(root, (*out)->root, 32);
    return BZ_OK;
}

int bz_commit(bz_ctx *ctx, const uint64_t *msg, size_t n_words, const bz_params *params,
              bz_commitment **out, uint8_t root[32]) {
    if (!ctx || !msg || !out) return BZ_ERR_ARG;
    *out = nullptr;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, n_words, why);
    if (rc) return set_msg(ctx, rc, why);
    void *d_msg = nullptr;
    const size_t bytes = n_words * 16;
    rc = dev_alloc(ctx, bytes, &d_msg, true);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(d_msg, msg, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        dev_free(ctx, d_msg, bytes, true);
        return set_err(ctx, BZ_ERR_CUDA, "H2D message", e);
    }
    rc = bz_commit_device(ctx, (const uint64_t *)d_msg, n_words, params, out, root);
    dev_free(ctx, d_msg, bytes, true);
    return rc;
}

int bz_commit_async(bz_ctx *ctx, const uint64_t *msg, size_t n_words, const bz_params *params,
                    bz_commitment **out) {
    if (!ctx || !msg || !out) return BZ_ERR_ARG;
    *out = nullptr;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, n_words, why);
    if (rc) return set_msg(ctx, rc, why);
    bz_commitment *c = nullptr;
    rc = alloc_commitment(ctx, s, &c);
    if (rc) return rc;
    const size_t bytes = n_words * 16;
    if (ctx->in_use.load() + bytes > ctx->budget) {
        bz_commitment_free(c);
        return set_msg(ctx, BZ_ERR_NOMEM, "memory budget exceeded");
    }
    void *d_msg = nullptr;
    cudaError_t e = cudaMallocAsync(&d_msg, bytes, ctx->copy_stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        bz_commitment_free(c);
        return set_err(ctx, BZ_ERR_NOMEM, "message staging", e);
    }
    cudaEvent_t copied = nullptr;
    cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming);
    e = cudaMemcpyAsync(d_msg, msg, bytes, cudaMemcpyHostToDevice, ctx->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(copied, ctx->copy_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, copied, 0);
    cudaEventDestroy(copied);  // the wait above already captured it
    if (e != cudaSuccess) {
        cudaFreeAsync(d_msg, ctx->copy_stream);
        bz_commitment_free(c);
        return set_err(ctx, BZ_ERR_CUDA, "H2D message", e);
    }
    rc = enqueue_commit(ctx, s, (const uint4 *)d_msg, c, ctx->stream, schedule_for(ctx, s));
    cudaFreeAsync(d_msg, ctx->stream);
    if (rc) {
        bz_commitment_free(c);
        return rc;
    }
    uint8_t *slot = (uint8_t *)ctx->h_small + 32 * (ctx->root_ring++ % 96) + 1024;
    c->root_slot = slot;
    cudaMemcpyAsync(slot, c->d_tree + (s.tree_nodes() - 1) * 32, 32, cudaMemcpyDeviceToHost,
                    ctx->stream);
    e = cudaEventRecord(c->done, ctx->stream);
    if (e != cudaSuccess) {
        bz_commitment_free(c);
        return set_err(ctx, BZ_ERR_CUDA, "record", e);
    }
    *out = c;
    return BZ_OK;
}

int bz_commitment_root(bz_commitment *c, uint8_t root[32]) {
    if (!c || !root) return BZ_ERR_ARG;
    int rc = fetch_root(c);
    if (rc) return rc;
    memcpy(root, c->root, 32);
    return BZ_OK;
}

int bz_commitment_params(const bz_commitment *c, bz_params *p) {
    if (!c || !p) return BZ_ERR_ARG;
    p->log_msg_len = (uint32_t)c->shape.log_msg_len;
    p->log_inv_rate = (uint32_t)c->shape.log_inv_rate;
    p->log_batch_size = (uint32_t)c->shape.log_lanes;
    p->hash_kind = (uint32_t)c->shape.hash_kind;
    return BZ_OK;
}

int bz_commitment_device_ptrs(const bz_commitment *c, const uint64_t **d_codeword,
                              const uint8_t **d_tree) {
    if (!c) return BZ_ERR_ARG;
    if (d_codeword) *d_codeword = (const uint64_t *)c->d_cw;
    if (d_tree) *d_tree = c->d_tree;
    return BZ_OK;
}

int bz_commitment_copy_codeword(bz_commitment *c, uint64_t *out, size_t n_words) {
    if (!c || !out) return BZ_ERR_ARG;
    bz_ctx *ctx = c->ctx;
    if (!c->d_cw) return set_msg(ctx, BZ_ERR_STATE, "tree-only commitment: no codeword");
    if (n_words != c->shape.cw_words()) return set_msg(ctx, BZ_ERR_ARG, "codeword size");
    BZ_CUDA(ctx, cudaMemcpyAsync(out, c->d_cw, n_words * 16, cudaMemcpyDeviceToHost, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_commitment_copy_tree(bz_commitment *c, uint8_t *out, size_t n_nodes) {
    if (!c || !out) return BZ_ERR_ARG;
    bz_ctx *ctx = c->ctx;
    if (n_nodes != c->shape.tree_nodes()) return set_msg(ctx, BZ_ERR_ARG, "tree size");
    BZ_CUDA(ctx, cudaMemcpyAsync(out, c->d_tree, n_nodes * 32, cudaMemcpyDeviceToHost, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_commitment_rows(bz_commitment *c, const uint64_t *positions, size_t q, uint64_t *out) {
    if (!c || (q && (!positions || !out))) return BZ_ERR_ARG;
    return bz::commitment_rows_on(c, positions, q, out, c->ctx->stream);
}

int bz_commitment_multiproof(bz_commitment *c, const uint64_t *positions, size_t q, uint8_t *out,
                             size_t cap, size_t *n_hashes) {
    if (!c || !n_hashes || (q && !positions)) return BZ_ERR_ARG;
    return bz::commitment_multiproof_on(c, positions, q, out, cap, n_hashes, c->ctx->stream);
}

int bz_commitment_free(bz_commitment *c) {
    if (!c) return BZ_ERR_ARG;
    {
        std::lock_guard<std::mutex> g(g_handles_mu);
        if (!g_handles.erase(c)) return BZ_ERR_STATE;  // freed, or its context destroyed
    }
    bz_ctx *ctx = c->ctx;
    {
        std::lock_guard<std::mutex> g(ctx->live_mu);
        if (!ctx->live.erase(c)) return BZ_ERR_STATE;
    }
    dev_free(ctx, c->d_cw, c->cw_bytes, true);
    dev_free(ctx, c->d_tree, c->tree_bytes, true);
    if (c->done) cudaEventDestroy(c->done);
    delete c;
    return BZ_OK;
}

int bz_commit_profile(bz_ctx *ctx, const uint64_t *d_msg, size_t n_words,
                      const bz_params *params, size_t cap, float *ms, char *names,
                      size_t *count, uint8_t root[32]) {
    if (!ctx || !d_msg || !count) return BZ_ERR_ARG;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, n_words, why);
    if (rc) return set_msg(ctx, rc, why);
    bz_commitment *c = nullptr;
    rc = alloc_commitment(ctx, s, &c);
    if (rc) return rc;
    const uint4 *d_tw = nullptr;
    rc = get_twiddles(ctx, s.k_code(), &d_tw);
    if (rc == BZ_OK && merkle_scratch_bytes(s)) rc = ensure_scratch(ctx, merkle_scratch_bytes(s));
    if (rc) {
        bz_commitment_free(c);
        return rc;
    }
    {
        LaunchLog log;
        log.st = ctx->stream;
        log.mark("start");
        int n = launch_commit_kernels(ctx, s, schedule_for(ctx, s), (const uint4 *)d_msg, c->d_cw,
                                      c->d_tree, d_tw, ctx->stream, &log);
        ctx->launches += (uint64_t)n;
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            bz_commitment_free(c);
            return set_err(ctx, BZ_ERR_CUDA, "profile", e);
        }
        const size_t k = log.events.size() - 1;
        *count = k;
        for (size_t i = 0; i < k && i < cap; ++i) {
            float t = 0;
            cudaEventElapsedTime(&t, log.events[i], log.events[i + 1]);
            if (ms) ms[i] = t;
            if (names) {
                strncpy(names + 32 * i, log.names[i + 1].c_str(), 31);
                names[32 * i + 31] = 0;
            }
        }
    }
    rc = fetch_root(c);
    if (rc == BZ_OK && root) memcpy(root, c->root, 32);
    bz_commitment_free(c);
    return rc;
}

int bz_ligero_commit_device(bz_ctx *ctx, const uint64_t *d_poly, uint32_t log_msg_cols,
                            uint32_t log_num_interleaved, uint32_t log_inv_rate,
                            uint32_t hash_kind, bz_commitment **out, uint8_t root[32]) {
    // ligero_commit (ligerito.rs:2390-2434) is commit_into with
    // log_msg_len = log_msg_cols + log_num_interleaved (same layout
    // poly[col * num_interleaved + lane]).
    bz_params p;
    p.log_msg_len = log_msg_cols + log_num_interleaved;
    p.log_inv_rate = log_inv_rate;
    p.log_batch_size = log_num_interleaved;
    p.hash_kind = hash_kind;
    return bz_commit_device(ctx, d_poly, (size_t)1 << p.log_msg_len, &p, out, root);
}

// ---- folds --------------------------------------------------------------
static uint4 to_u4(const uint64_t r[2]) {
    return make_uint4((uint32_t)r[0], (uint32_t)(r[0] >> 32), (uint32_t)r[1],
                      (uint32_t)(r[1] >> 32));
}

static bool pow2(size_t n) { return n && !(n & (n - 1)); }

}  // extern "C"

namespace bz {

// Mailbox post for the next message kernel on the context stream.
static MsgPost next_post(bz_ctx *ctx) {
    MsgPost p;
    p.ticket = (unsigned int *)((uint8_t *)ctx->d_small + 768);
    p.words = (uint64_t *)ctx->d_mbox;
    p.seq = (uint32_t *)((uint8_t *)ctx->d_mbox + 64);
    if (++ctx->mbox_seq == 0) ++ctx->mbox_seq;  // 0 is the initial mailbox value
    p.seq_val = ctx->mbox_seq;
    return p;
}

MsgPost next_msg_post(bz_ctx *ctx) { return next_post(ctx); }

void reset_msg_ticket(bz_ctx *ctx) {
    cudaMemsetAsync((uint8_t *)ctx->d_small + 768, 0, 4, ctx->stream);
}

// Wait for the message kernel to post sequence number seq, then read
// {u0, u2}.  The wait spins on the mailbox (no stream synchronisation on the
// critical path), checking the stream every few hundred spins so that a
// failed launch returns its error, and gives up after 60 s.
int mapped_wait(bz_ctx *ctx, size_t offset, uint32_t seq, const char *what) {
    volatile uint32_t *sp = (volatile uint32_t *)((uint8_t *)ctx->h_mbox + offset);
    const auto t0 = std::chrono::steady_clock::now();
    for (uint64_t spin = 1; *sp != seq; ++spin) {
        if ((spin & 255) == 0) {
            const cudaError_t e = cudaStreamQuery(ctx->stream);
            if (e != cudaSuccess && e != cudaErrorNotReady) return set_err(ctx, BZ_ERR_CUDA, what, e);
            if (e == cudaSuccess && *sp != seq)
                return set_msg(ctx, BZ_ERR_CUDA, std::string(what) + ": result not posted");
            if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60))
                return set_msg(ctx, BZ_ERR_TIMEOUT, std::string(what) + ": wait");
        }
    }
    std::atomic_thread_fence(std::memory_order_acquire);
    return BZ_OK;
}

int msg_wait(bz_ctx *ctx, uint32_t seq, uint64_t u0[2], uint64_t u2[2]) {
    const int rc = mapped_wait(ctx, 64, seq, "sumcheck message");
    if (rc) return rc;
    const volatile uint64_t *h = (const volatile uint64_t *)ctx->h_mbox;
    if (u0) {
        u0[0] = h[0];
        u0[1] = h[1];
    }
    if (u2) {
        u2[0] = h[2];
        u2[1] = h[3];
    }
    return BZ_OK;
}

int fold_launch(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb, uint32_t *msg_seq) {
    int rc = ensure_scratch(ctx, fold_partials_bytes(n));
    if (rc) return rc;
    const MsgPost post = next_post(ctx);
    ctx->launches += launch_fold_and_msg((const uint4 *)d_f, (const uint4 *)d_b, n, to_u4(r),
                                         (uint4 *)d_nf, (uint4 *)d_nb, (uint64_t *)ctx->scratch,
                                         nullptr, ctx->stream, ctx->num_sms, &post);
    BZ_CUDA(ctx, cudaGetLastError());
    *msg_seq = post.seq_val;
    return BZ_OK;
}

// The gate: r at byte 128 and the go word at byte 192 of the mapped mailbox;
// the kernel's time-out record at byte 832 of the small device buffer.
static uint8_t *gate_host(bz_ctx *ctx) { return (uint8_t *)ctx->h_mbox + 128; }

// Armed only while every CTA of the fold fits on the GPU at once, so that
// the CTAs that wait at the gate are few.
bool fold_armable(const bz_ctx *ctx, size_t n) {
    return ctx->arm_folds && n >= 2 && fold_grid(n, ctx->num_sms) <= 2 * ctx->num_sms;
}

bool gate_gave_up(bz_ctx *ctx) {
    uint32_t *d_err = (uint32_t *)((uint8_t *)ctx->d_small + 832);
    uint32_t err = 0;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
        cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost) != cudaSuccess || !err)
        return false;
    cudaMemset(d_err, 0, 4);
    ctx->arm_folds = false;
    return true;
}

int fold_arm(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n, uint64_t *d_nf,
             uint64_t *d_nb, ArmedFold *a, uint64_t limit_ns) {
    if (a->live) return set_msg(ctx, BZ_ERR_STATE, "a fold is already armed");
    int rc = ensure_scratch(ctx, fold_partials_bytes(n));
    if (rc) return rc;
    if (++ctx->gate_seq >= kGateCancel) ctx->gate_seq = 1;
    RGate g;
    g.r = (const uint64_t *)((uint8_t *)ctx->d_mbox + 128);
    g.go = (const uint32_t *)((uint8_t *)ctx->d_mbox + 192);
    g.seq = ctx->gate_seq;
    g.err = (uint32_t *)((uint8_t *)ctx->d_small + 832);
    g.limit_ns = limit_ns;
    const MsgPost post = next_post(ctx);
    ctx->launches += launch_fold_and_msg((const uint4 *)d_f, (const uint4 *)d_b, n,
                                         make_uint4(0, 0, 0, 0), (uint4 *)d_nf, (uint4 *)d_nb,
                                         (uint64_t *)ctx->scratch, nullptr, ctx->stream,
                                         ctx->num_sms, &post, &g);
    BZ_CUDA(ctx, cudaGetLastError());
    a->gate_seq = g.seq;
    a->msg_seq = post.seq_val;
    a->f = d_f;
    a->b = d_b;
    a->nf = d_nf;
    a->nb = d_nb;
    a->n = n;
    a->live = true;
    return BZ_OK;
}

// r first, then (release) the go word.
void fold_open(bz_ctx *ctx, ArmedFold *a, const uint64_t r[2]) {
    uint64_t *hr = (uint64_t *)gate_host(ctx);
    __atomic_store_n(&hr[0], r[0], __ATOMIC_RELAXED);
    __atomic_store_n(&hr[1], r[1], __ATOMIC_RELAXED);
    __atomic_store_n((uint32_t *)(gate_host(ctx) + 64), a->gate_seq, __ATOMIC_RELEASE);
    a->live = false;
}

// The cancelled CTAs return before touching the arrays or the ticket; the
// stream is drained so that nothing armed outlives the call.
int fold_cancel(bz_ctx *ctx, ArmedFold *a) {
    if (!a->live) return BZ_OK;
    __atomic_store_n((uint32_t *)(gate_host(ctx) + 64), a->gate_seq | kGateCancel,
                     __ATOMIC_RELEASE);
    a->live = false;
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

}  // namespace bz

extern "C" {

int bz_fold_and_msg_lsb(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                        const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb, uint64_t u0[2],
                        uint64_t u2[2]) {
    if (!ctx || !d_f || !d_b || !r || !d_nf || !d_nb) return BZ_ERR_ARG;
    if (!pow2(n) || n < 2) return set_msg(ctx, BZ_ERR_SHAPE, "n must be a power of two >= 2");
    uint32_t seq = 0;
    int rc = fold_launch(ctx, d_f, d_b, n, r, d_nf, d_nb, &seq);
    if (rc) return rc;
    return msg_wait(ctx, seq, u0, u2);
}

int bz_fold_gate_check(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                       const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb, int mode,
                       uint64_t limit_ns, uint64_t u0[2], uint64_t u2[2]) {
    if (!ctx || !d_f || !d_b || !d_nf || !d_nb || mode < 0 || mode > 2 || (mode == 0 && !r))
        return BZ_ERR_ARG;
    if (!pow2(n) || n < 2) return set_msg(ctx, BZ_ERR_SHAPE, "n must be a power of two >= 2");
    ArmedFold a;
    int rc = fold_arm(ctx, d_f, d_b, n, d_nf, d_nb, &a, limit_ns ? limit_ns : kGateLimitNs);
    if (rc) return rc;
    if (mode == 0) {
        fold_open(ctx, &a, r);
        return msg_wait(ctx, a.msg_seq, u0, u2);
    }
    if (mode == 1) return fold_cancel(ctx, &a);
    // mode 2: nothing is posted; the kernel's CTAs give up at the time limit
    a.live = false;
    const bool arming = ctx->arm_folds;
    const bool gave_up = gate_gave_up(ctx);
    ctx->arm_folds = arming;  // a deliberate time-out: the prover's arming is unchanged
    reset_msg_ticket(ctx);
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!gave_up) return set_msg(ctx, BZ_ERR_STATE, "the gate did not record its time-out");
    return set_msg(ctx, BZ_ERR_TIMEOUT, "fold gate: no challenge posted within the limit");
}

int bz_round_msg_lsb(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                     uint64_t u0[2], uint64_t u2[2]) {
    if (!ctx || !d_f || !d_b) return BZ_ERR_ARG;
    if (!pow2(n) || n < 2) return set_msg(ctx, BZ_ERR_SHAPE, "n must be a power of two >= 2");
    int rc = ensure_scratch(ctx, fold_partials_bytes(n));
    if (rc) return rc;
    const MsgPost post = next_post(ctx);
    ctx->launches += launch_round_msg((const uint4 *)d_f, (const uint4 *)d_b, n,
                                      (uint64_t *)ctx->scratch, nullptr, ctx->stream, ctx->num_sms,
                                      &post);
    BZ_CUDA(ctx, cudaGetLastError());
    return msg_wait(ctx, post.seq_val, u0, u2);
}

int bz_partial_eval_lsb(bz_ctx *ctx, const uint64_t *d_in, size_t n, const uint64_t *rs, size_t k,
                        uint64_t *d_out) {
    if (!ctx || !d_in || !d_out || (k && !rs)) return BZ_ERR_ARG;
    if (!pow2(n) || ((size_t)1 << k) > n) return set_msg(ctx, BZ_ERR_SHAPE, "bad n / k");
    if (k == 0) {
        BZ_CUDA(ctx, cudaMemcpyAsync(d_out, d_in, n * 16, cudaMemcpyDeviceToDevice, ctx->stream));
        BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return BZ_OK;
    }
    // ping-pong through one temporary of n/2 elements; last round into d_out
    void *tmp = nullptr;
    int rc = BZ_OK;
    if (k > 1) {
        rc = dev_alloc(ctx, (n / 2) * 16 * 2, &tmp, false);
        if (rc) return rc;
    }
    const uint4 *src = (const uint4 *)d_in;
    size_t len = n;
    uint4 *bufs[2] = {(uint4 *)tmp, tmp ? (uint4 *)tmp + n / 2 : nullptr};
    for (size_t i = 0; i < k; ++i) {
        uint4 *dst = (i == k - 1) ? (uint4 *)d_out : bufs[i & 1];
        ctx->launches += launch_partial_eval_round(src, len, to_u4(rs + 2 * i), dst, ctx->stream);
        src = dst;
        len /= 2;
    }
    if (tmp) dev_free(ctx, tmp, 0, false);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

// ---- ring switch -----------------------------------------------------------
int bz_build_eq_lsb(bz_ctx *ctx, const uint64_t *point, size_t k, uint64_t *d_out) {
    if (!ctx || !d_out || (k && !point)) return BZ_ERR_ARG;
    if (k > 40) return set_msg(ctx, BZ_ERR_SHAPE, "k too large");
    void *d_pt = nullptr;
    int rc = dev_alloc(ctx, (k ? k : 1) * 16, &d_pt, false);
    if (rc) return rc;
    if (k) cudaMemcpyAsync(d_pt, point, k * 16, cudaMemcpyHostToDevice, ctx->stream);
    ctx->launches +=
        launch_build_eq((const uint4 *)d_pt, k, (uint4 *)d_out, ctx->stream, ctx->num_sms);
    dev_free(ctx, d_pt, 0, false);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_sv_fold(bz_ctx *ctx, const uint64_t *d_packed, const uint64_t *d_eq, size_t n,
               uint64_t *sv) {
    if (!ctx || !d_packed || !d_eq || !sv) return BZ_ERR_ARG;
    int rc = ensure_scratch(ctx, sv_partials_bytes(n, ctx->num_sms) + 128 * 16);
    if (rc) return rc;
    uint4 *d_sv = (uint4 *)(ctx->scratch + sv_partials_bytes(n, ctx->num_sms));
    ctx->launches += launch_sv_fold((const uint4 *)d_packed, (const uint4 *)d_eq, n,
                                    (uint64_t *)ctx->scratch, d_sv, ctx->stream, ctx->num_sms);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaMemcpyAsync(sv, d_sv, 128 * 16, cudaMemcpyDeviceToHost, ctx->stream));
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

int bz_phi_from_words(bz_ctx *ctx, const uint64_t *d_eq_hi, size_t n, const uint64_t *eq_r2,
                      uint64_t *d_out) {
    if (!ctx || !d_eq_hi || !eq_r2 || !d_out) return BZ_ERR_ARG;
    void *d_r2 = nullptr;
    int rc = dev_alloc(ctx, 128 * 16, &d_r2, false);
    if (rc) return rc;
    cudaMemcpyAsync(d_r2, eq_r2, 128 * 16, cudaMemcpyHostToDevice, ctx->stream);
    ctx->launches += launch_phi((const uint4 *)d_eq_hi, n, (const uint4 *)d_r2, (uint4 *)d_out,
                                ctx->stream, ctx->num_sms);
    dev_free(ctx, d_r2, 0, false);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

// ---- inputs -----------------------------------------------------------------
int bz_chacha_fill_device(bz_ctx *ctx, uint64_t seed, uint64_t first_word, uint64_t *d_out,
                          size_t n_words) {
    if (!ctx || (n_words && !d_out)) return BZ_ERR_ARG;
    ctx->launches += launch_chacha(seed, first_word, (uint4 *)d_out, n_words, ctx->stream);
    BZ_CUDA(ctx, cudaGetLastError());
    BZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return BZ_OK;
}

}  // extern "C"
