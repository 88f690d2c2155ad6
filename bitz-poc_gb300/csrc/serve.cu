// Continuous-batching commit/open server.
//
// Requests are (1) commits of host messages of mixed sizes and (2) openings
// of earlier commits at query positions (rows + Merkle multi-proof).  A
// scheduler thread admits pending commits whenever an execution slot (a CUDA
// stream) is free AND the request's device memory (message staging +
// resident codeword + tree) fits in the server's budget, so requests that
// arrive while others run start as soon as slots and memory free up and their
// kernels overlap on the device.  Codewords and trees stay resident until
// the request is opened; the opening frees them.  Every device wait is an
// event query polled by the scheduler (no blocking call on the device), and
// host waits are bounded by caller timeouts.
//
// The server uses its own streams and its own scratch-free shapes (leaves up
// to 256 BLAKE3 chunks); while it runs, the owning context may still be used
// from other threads for unrelated work on the context stream.
//
// Scheduling: queued commits are admitted smallest first, except that a
// request that has waited longer than the aging bound goes first (so a large
// request is never starved), or in arrival order (bz_server_set_policy).
// The slots' streams have three priorities: a third of them the highest, for
// small requests of at most 2^small_log elements (2^20 by default) and for
// openings; a third a middle one, for medium requests of at most
// 2^(small_log + 3) elements; the rest the lowest, for the largest.  A request
// takes a slot of its own tier or, when those are busy, of a lower one, never a
// higher one.  Medium and large requests' table passes run as short CTAs, so a
// higher tier's kernels get SMs within a fraction of their pass.  A small or
// medium request's message is read from pinned host memory by a copy kernel,
// so it never queues behind a large upload on the copy engine; the largest
// requests' uploads go to the copy engine in 64 MiB pieces.  A commit-then-open
// request enqueues its opening (row gather, multi-proof nodes, the copies to
// the slot's pinned staging) right behind its commit on the same stream: one
// completion, no second trip through the scheduler.  Each slot's work ends
// with a host callback that wakes the scheduler.
//
// Nothing on the request path synchronises the device: device buffers come
// from the buffers of finished requests of the same size or else from the
// server's stream-ordered pool (cudaMallocFromPoolAsync / cudaFreeAsync on
// the slot's stream), and each slot owns its completion event and a grow-only pinned
// staging buffer for the root, rows and proof nodes, which the scheduler
// copies into the request when the slot's work completes.  A completion
// queue (bz_server_next_done) hands state changes to the caller without
// polling every request.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <deque>
#include <set>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "runtime.h"

using namespace bz;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState : int {
    RS_QUEUED = 0,
    RS_RUNNING = 1,
    RS_COMMITTED = 2,
    RS_OPEN_QUEUED = 3,
    RS_OPENING = 4,
    RS_OPENED = 5,
    RS_FAILED = 6,
};

struct Request {
    uint64_t id = 0;
    Shape shape;
    const uint64_t *host_msg = nullptr;
    int state = RS_QUEUED;
    int error = BZ_OK;
    // device resources
    uint4 *d_msg = nullptr;
    bz_commitment *commit = nullptr;
    int slot = -1;
    uint8_t root[32] = {0};
    // opening
    bool auto_open = false;  // open as soon as the commit is done
    bool fused_open = false; // the opening was enqueued behind the commit
    std::vector<uint64_t> positions;
    std::vector<uint64_t> node_idx;
    std::vector<uint64_t> rows;  // q rows of 2^log_lanes elements
    std::vector<uint8_t> nodes;  // n_hashes * 32 bytes
    // timestamps (ns since server start)
    int64_t t_submit = 0, t_start = 0, t_committed = 0, t_open_submit = 0, t_opened = 0;
    size_t bytes = 0;
};

}  // namespace

struct bz_server {
    bz_ctx *ctx = nullptr;
    int n_slots = 0;
    uint64_t budget = 0, in_use = 0;
    size_t queue_cap = 0;
    // one stream per slot: the first n_hi slots have the highest priority and
    // serve small requests (and openings), the next n_mid a middle priority
    // for medium requests, the rest the lowest for the largest; a request may
    // also take a slot of a lower tier than its own.  One stream per slot
    // keeps the streams within the device's hardware work queues, so no two
    // slots' kernels serialise behind each other.
    std::vector<cudaStream_t> streams;
    int n_hi = 0, n_mid = 0;
    std::vector<cudaEvent_t> slot_done;    // completion of the slot's work
    std::vector<uint8_t *> slot_host;      // pinned staging (root, rows, nodes)
    std::vector<size_t> slot_host_bytes;
    std::vector<bool> slot_busy;
    std::deque<std::pair<uint64_t, int>> completed;  // (id, new state) for bz_server_next_done
    bool notify = false;                   // completions are recorded once asked for
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    // queued commits: by arrival (ids increase with arrival) and by size
    std::set<uint64_t> pend_by_id;
    std::set<std::pair<uint64_t, uint64_t>> pend_by_size;  // (bytes, id)
    std::deque<uint64_t> pending_opens;
    int admit_order = BZ_ADMIT_SMALLEST;
    int64_t aging_ns = 500000000;      // 500 ms
    int small_log = 20;                // requests of <= 2^small_log elements: high priority
    std::atomic<uint64_t> wakes{0};    // bumped by the slots' host callbacks
    // The server's own stream-ordered pool.  Its memory is reused across the
    // slots' streams only once the freeing stream's work is known complete:
    // with the default pool's internal dependencies, a small request's
    // allocation could take memory a large request freed and be made to wait
    // for that request's stream.
    cudaMemPool_t pool = nullptr;
    // Device buffers of finished requests, by size, kept for the next request
    // of the same size (sizes are powers of two, so a few recur).  Taking
    // them does not block: a pool allocation that has to map more memory holds
    // the scheduler (and every completion behind it) for 5-7 ms at a 2^26
    // request, and the pool had to whenever its free blocks were too small
    // for the request or not yet known complete on another stream.
    std::map<size_t, std::vector<void *>> spare;
    uint64_t spare_bytes = 0;
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<uint64_t> running;  // commit or open in flight
    uint64_t next_id = 1;
    bool stop = false;
    std::thread thr;
    Clock::time_point t0;
    uint64_t n_committed = 0, n_opened = 0, n_failed = 0;
    int64_t ns() const {
        return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
    }
};

namespace {

size_t request_bytes(const Shape &s) {
    return s.msg_words() * 16 + s.cw_words() * 16 + s.tree_nodes() * 32;
}

// Multi-proof node indices of sorted unique positions
// (flock-core/src/merkle.rs:688-741).
std::vector<uint64_t> multiproof_nodes(std::vector<uint64_t> act, uint64_t n_leaves) {
    std::vector<uint64_t> idx;
    uint64_t level_start = 0, level_len = n_leaves;
    while (level_len > 1 && !act.empty()) {
        std::vector<uint64_t> next;
        size_t i = 0;
        while (i < act.size()) {
            const uint64_t p = act[i];
            if (i + 1 < act.size() && act[i + 1] == (p ^ 1)) {
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
    return idx;
}

// Sorted unique positions, all below n_leaves (else false).
bool set_positions(Request *r, const uint64_t *positions, size_t q) {
    const uint64_t n_leaves = r->shape.n_leaves();
    std::vector<uint64_t> act(positions, positions + q);
    for (uint64_t p : act)
        if (p >= n_leaves) return false;
    std::sort(act.begin(), act.end());
    act.erase(std::unique(act.begin(), act.end()), act.end());
    r->node_idx = multiproof_nodes(act, n_leaves);
    r->positions = std::move(act);
    return true;
}

// Grow slot's pinned staging to `bytes` (the slot is idle when called).
int ensure_slot_host(bz_server *S, int slot, size_t bytes) {
    if (S->slot_host_bytes[slot] >= bytes) return BZ_OK;
    const size_t want = std::max(bytes, (size_t)2 * S->slot_host_bytes[slot]);
    if (S->slot_host[slot]) cudaFreeHost(S->slot_host[slot]);
    S->slot_host[slot] = nullptr;
    S->slot_host_bytes[slot] = 0;
    if (cudaMallocHost(&S->slot_host[slot], want) != cudaSuccess) {
        cudaGetLastError();
        return BZ_ERR_NOMEM;
    }
    S->slot_host_bytes[slot] = want;
    return BZ_OK;
}

#ifndef BZ_SERVE_SHORT_CTAS
#define BZ_SERVE_SHORT_CTAS 1
#endif

bool is_large(const bz_server *S, const Shape &s) { return s.log_msg_len > S->small_log; }

// Priority tier of a request: 0 small, 1 medium, 2 the largest (everything
// tier 0 when priorities are off).
constexpr int kMidSpan = 3;  // medium: up to 2^(small_log + kMidSpan) elements
int tier_of(const bz_server *S, const Shape &s) {
    if (S->small_log < 0 || s.log_msg_len <= S->small_log) return 0;
    return s.log_msg_len <= S->small_log + kMidSpan ? 1 : 2;
}

// Wakes the scheduler once a slot's work is done (runs on a CUDA callback
// thread: no CUDA call and no lock here; the scheduler's wait has a short
// timeout as well, so a wakeup that races its check costs that timeout).
void CUDART_CB slot_done_cb(void *p) {
    bz_server *S = static_cast<bz_server *>(p);
    S->wakes.fetch_add(1, std::memory_order_release);
    S->cv_work.notify_one();
}

// Enqueue the gather of r's opened rows and multi-proof nodes and their copy
// into the slot's pinned staging at byte offset h_off (rows, then nodes).
int enqueue_open(bz_server *S, Request *r, cudaStream_t st, uint8_t *h) {
    bz_ctx *ctx = S->ctx;
    const Shape &s = r->shape;
    const size_t q = r->positions.size(), nn = r->node_idx.size();
    const size_t row_bytes = s.leaf_bytes();
    // device: positions, node indices, rows, nodes in one stream-ordered allocation
    const size_t o_idx = q * 8, o_rows = (o_idx + nn * 8 + 15) & ~(size_t)15;
    const size_t o_nodes = o_rows + q * row_bytes, dev_bytes = o_nodes + nn * 32 + 16;
    uint8_t *d = nullptr;
    if (cudaMallocFromPoolAsync((void **)&d, dev_bytes, S->pool, st) != cudaSuccess) {
        cudaGetLastError();
        return BZ_ERR_NOMEM;
    }
    uint64_t *d_pos = (uint64_t *)d, *d_idx = (uint64_t *)(d + o_idx);
    uint4 *d_rows = (uint4 *)(d + o_rows);
    uint8_t *d_nodes = d + o_nodes;
    if (q) cudaMemcpyAsync(d_pos, r->positions.data(), q * 8, cudaMemcpyHostToDevice, st);
    if (nn) cudaMemcpyAsync(d_idx, r->node_idx.data(), nn * 8, cudaMemcpyHostToDevice, st);
    int n = launch_gather_rows(r->commit->d_cw, s.log_lanes, d_pos, q, d_rows, st);
    n += launch_gather_nodes(r->commit->d_tree, d_idx, nn, d_nodes, st);
    ctx->launches += (uint64_t)n;
    if (q) cudaMemcpyAsync(h, d_rows, q * row_bytes, cudaMemcpyDeviceToHost, st);
    if (nn) cudaMemcpyAsync(h + q * row_bytes, d_nodes, nn * 32, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    return BZ_OK;
}

// dst[i] = src[i], src in host memory the device can read (pinned, mapped).
__global__ void __launch_bounds__(256) upload_kernel(const uint4 *__restrict__ src,
                                                     uint4 *__restrict__ dst, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride],
                    d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

// The device's view of a host buffer, if it is pinned and mapped (null for
// pageable memory or a failed query).
const void *mapped_view(const void *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

size_t open_staging_bytes(const Request *r) {
    return r->positions.size() * r->shape.leaf_bytes() + r->node_idx.size() * 32;
}

// Spare buffers back to the pool (their work is complete), freed in st's order.
void drop_spares(bz_server *S, cudaStream_t st) {
    for (auto &kv : S->spare)
        for (void *p : kv.second) cudaFreeAsync(p, st);
    S->spare.clear();
    S->spare_bytes = 0;
}

// A device buffer of the given size for work on st: a spare one if any, else
// one from the pool (after giving the spares back to it when the pool alone
// cannot serve the size).  Null when the device is out of memory.
void *take_buffer(bz_server *S, size_t bytes, cudaStream_t st) {
    auto it = S->spare.find(bytes);
    if (it != S->spare.end() && !it->second.empty()) {
        void *p = it->second.back();
        it->second.pop_back();
        S->spare_bytes -= bytes;
        return p;
    }
    // the live requests (this one included) and the spares stay within the budget
    if (S->in_use + S->spare_bytes > S->budget) drop_spares(S, st);
    void *p = nullptr;
    if (cudaMallocFromPoolAsync(&p, bytes, S->pool, st) == cudaSuccess) return p;
    cudaGetLastError();
    if (S->spare_bytes == 0) return nullptr;
    drop_spares(S, st);
    if (cudaMallocFromPoolAsync(&p, bytes, S->pool, st) == cudaSuccess) return p;
    cudaGetLastError();
    return nullptr;
}

// A buffer whose work is complete (its slot's event was seen): kept as a spare
// while the live requests and the spares fit in the budget, else back to the
// pool.
void give_buffer(bz_server *S, void *p, size_t bytes, cudaStream_t st) {
    if (!p) return;
    if (S->in_use + S->spare_bytes + bytes <= S->budget) {
        S->spare[bytes].push_back(p);
        S->spare_bytes += bytes;
    } else {
        cudaFreeAsync(p, st);
    }
}

// Start a commit on a free slot (caller holds the lock).  A commit-then-open
// request's opening follows on the same stream; the root lands in the first
// 32 bytes of the slot's staging, the opening's rows and nodes after it.
int start_commit(bz_server *S, Request *r, int slot) {
    bz_ctx *ctx = S->ctx;
    const Shape &s = r->shape;
    const bool large = is_large(S, s);
    cudaStream_t st = S->streams[slot];
    if (r->auto_open) {
        const int rc = ensure_slot_host(S, slot, 32 + open_staging_bytes(r));
        if (rc) return rc;
    }
    r->d_msg = static_cast<uint4 *>(take_buffer(S, s.msg_words() * 16, st));
    if (!r->d_msg) return BZ_ERR_NOMEM;
    bz_commitment *c = new bz_commitment();
    c->ctx = ctx;
    c->shape = s;
    c->cw_bytes = s.cw_words() * 16;
    c->tree_bytes = s.tree_nodes() * 32;
    c->d_cw = static_cast<uint4 *>(take_buffer(S, c->cw_bytes, st));
    if (c->d_cw) c->d_tree = static_cast<uint8_t *>(take_buffer(S, c->tree_bytes, st));
    if (!c->d_cw || !c->d_tree) {
        // nothing has used them yet: freed in st's order
        if (c->d_cw) cudaFreeAsync(c->d_cw, st);
        cudaFreeAsync(r->d_msg, st);
        r->d_msg = nullptr;
        delete c;
        return BZ_ERR_NOMEM;
    }
    r->commit = c;
    // A small or medium request's message is read from pinned host memory by
    // a copy kernel on its own stream (as fast as the copy engine, both being
    // limited by the host link), so it never waits on the copy engine behind
    // a large request's upload: through the copy engine, 2^21-2^23 requests
    // waited 15-80 ms behind the 0.5-1 GiB uploads of the largest.  The
    // largest tier's and pageable messages go through the copy engine, in
    // pieces that let the other streams' copies in between.
    const bool ce_upload = S->small_log < 0 || tier_of(S, s) == 2;
    const void *dev_view = ce_upload ? nullptr : mapped_view(r->host_msg);
    if (dev_view) {
        const uint64_t n = s.msg_words();
        const unsigned grid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>((uint64_t)ctx->num_sms, (n + 1023) / 1024));
        upload_kernel<<<grid, 256, 0, st>>>(static_cast<const uint4 *>(dev_view), r->d_msg, n);
        ctx->launches += 1;
    } else {
        const size_t total = s.msg_words() * 16, piece = (size_t)64 << 20;
        for (size_t off = 0; off < total; off += piece)
            cudaMemcpyAsync(reinterpret_cast<uint8_t *>(r->d_msg) + off,
                            reinterpret_cast<const uint8_t *>(r->host_msg) + off,
                            std::min(piece, total - off), cudaMemcpyHostToDevice, st);
    }
    const uint4 *d_tw = nullptr;
    int rc = get_twiddles(ctx, s.k_code(), &d_tw);
    if (rc) return rc;
    // The shape's default schedule, not one the context's autotuner picked:
    // those are timed alone and may run two streams of their own (pipelined
    // schedules), which would bypass the slot's priority.  A large request's
    // table passes run as short CTAs when small requests have priority, so
    // their kernels get SMs within a fraction of a pass.
    uint32_t schedule = default_schedule(s);
#if BZ_SERVE_SHORT_CTAS
    if (S->small_log >= 0 && large) schedule |= SCHED_SHORT_CTAS;
#endif
    int n = launch_commit_kernels(ctx, s, schedule, r->d_msg, c->d_cw, c->d_tree, d_tw, st,
                                  nullptr);
    ctx->launches += (uint64_t)n;
    cudaMemcpyAsync(S->slot_host[slot], c->d_tree + (s.tree_nodes() - 1) * 32, 32,
                    cudaMemcpyDeviceToHost, st);
    r->fused_open = false;
    if (r->auto_open) {
        rc = enqueue_open(S, r, st, S->slot_host[slot] + 32);
        if (rc) return rc;
        r->fused_open = true;
    }
    cudaEventRecord(S->slot_done[slot], st);
    cudaLaunchHostFunc(st, slot_done_cb, S);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

int start_open(bz_server *S, Request *r, int slot) {
    cudaStream_t st = S->streams[slot];
    int rc = ensure_slot_host(S, slot, open_staging_bytes(r) + 32);
    if (rc) return rc;
    rc = enqueue_open(S, r, st, S->slot_host[slot]);
    if (rc) return rc;
    cudaEventRecord(S->slot_done[slot], st);
    cudaLaunchHostFunc(st, slot_done_cb, S);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

// The codeword and tree of r.  complete: the slot's work on them is known
// complete (its event was seen), so they may become spares; otherwise (a
// failed request) they go back to the pool in the stream's order.
void free_commit_buffers(bz_server *S, Request *r, int slot, bool complete) {
    if (r->commit) {
        cudaStream_t st = S->streams[slot >= 0 ? slot : 0];
        if (complete) {
            give_buffer(S, r->commit->d_cw, r->commit->cw_bytes, st);
            give_buffer(S, r->commit->d_tree, r->commit->tree_bytes, st);
        } else {
            cudaFreeAsync(r->commit->d_cw, st);
            cudaFreeAsync(r->commit->d_tree, st);
        }
        delete r->commit;
        r->commit = nullptr;
    }
}

// First slot of a tier (slots of tiers t, t+1, .. follow it); every slot when
// priorities are off.  With too few slots for three tiers the lower tiers
// share the last slot.
int tier_first_slot(const bz_server *S, int tier) {
    if (S->small_log < 0 || tier == 0) return 0;
    return std::min(S->n_slots - 1, tier == 1 ? S->n_hi : S->n_hi + S->n_mid);
}

// A free slot for a request of the given tier (-1: none): its own tier's
// slots first, then those of lower priority.
int free_slot(bz_server *S, int tier) {
    for (int i = tier_first_slot(S, tier); i < S->n_slots; ++i)
        if (!S->slot_busy[i]) return i;
    return -1;
}

// The next queued commit to admit and its slot ({0, -1}: none now): the
// oldest when it has waited past the aging bound (or in arrival order), else
// the smallest; a request with no free slot in its tier or below gives way to
// the smallest queued one.
std::pair<uint64_t, int> next_commit(bz_server *S) {
    const uint64_t oldest = *S->pend_by_id.begin();
    uint64_t id = oldest;
    if (S->admit_order == BZ_ADMIT_SMALLEST && S->ns() - S->reqs[oldest]->t_submit <= S->aging_ns)
        id = S->pend_by_size.begin()->second;
    int slot = free_slot(S, tier_of(S, S->reqs[id]->shape));
    if (slot < 0) {
        id = S->pend_by_size.begin()->second;
        slot = free_slot(S, tier_of(S, S->reqs[id]->shape));
    }
    return slot < 0 ? std::make_pair((uint64_t)0, -1) : std::make_pair(id, slot);
}

void scheduler(bz_server *S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    uint64_t seen_wakes = 0;
    while (!S->stop) {
        bool progress = false;
        seen_wakes = S->wakes.load(std::memory_order_acquire);
        // 1. completions
        for (size_t i = 0; i < S->running.size();) {
            Request *r = S->reqs[S->running[i]].get();
            cudaError_t q = cudaEventQuery(S->slot_done[r->slot]);
            if (q == cudaErrorNotReady) {
                ++i;
                continue;
            }
            progress = true;
            S->slot_busy[r->slot] = false;
            const uint8_t *h = S->slot_host[r->slot];
            auto take_opening = [&](const uint8_t *src) {
                const size_t q_rows = r->positions.size(), nn = r->node_idx.size();
                const size_t row_words = (size_t)2 << r->shape.log_lanes;
                r->rows.assign((const uint64_t *)src, (const uint64_t *)src + q_rows * row_words);
                r->nodes.assign(src + q_rows * row_words * 8,
                                src + q_rows * row_words * 8 + nn * 32);
                r->state = RS_OPENED;
                r->t_opened = S->ns();
                S->in_use -= r->bytes - r->shape.msg_words() * 16;
                free_commit_buffers(S, r, r->slot, true);
                ++S->n_opened;
            };
            if (q != cudaSuccess) {
                cudaGetLastError();
                if (r->d_msg) {  // a failed commit: its message buffer goes back to the pool
                    cudaFreeAsync(r->d_msg, S->streams[r->slot]);
                    r->d_msg = nullptr;
                    S->in_use -= r->shape.msg_words() * 16;
                }
                r->state = RS_FAILED;
                r->error = BZ_ERR_CUDA;
                ++S->n_failed;
            } else if (r->state == RS_RUNNING) {
                memcpy(r->root, h, 32);
                r->commit->root_ready = true;
                memcpy(r->commit->root, r->root, 32);
                r->state = RS_COMMITTED;
                r->t_committed = S->ns();
                S->in_use -= r->shape.msg_words() * 16;  // the message buffer is free
                give_buffer(S, r->d_msg, r->shape.msg_words() * 16, S->streams[r->slot]);
                r->d_msg = nullptr;
                ++S->n_committed;
                if (r->fused_open) {
                    // the opening ran behind the commit on the same stream
                    if (S->notify) S->completed.emplace_back(r->id, RS_COMMITTED);
                    r->t_open_submit = r->t_committed;
                    take_opening(h + 32);
                } else if (r->auto_open) {
                    if (S->notify) S->completed.emplace_back(r->id, RS_COMMITTED);
                    r->state = RS_OPEN_QUEUED;
                    r->t_open_submit = r->t_committed;
                    S->pending_opens.push_back(r->id);
                }
            } else if (r->state == RS_OPENING) {
                take_opening(h);
            }
            if (S->notify && r->state != RS_OPEN_QUEUED)
                S->completed.emplace_back(r->id, r->state);
            S->running[i] = S->running.back();
            S->running.pop_back();
        }
        // 2. openings first (they free memory)
        while (!S->pending_opens.empty()) {
            const int slot = free_slot(S, 0);
            if (slot < 0) break;
            Request *r = S->reqs[S->pending_opens.front()].get();
            S->pending_opens.pop_front();
            r->slot = slot;
            r->state = RS_OPENING;
            const int rc = start_open(S, r, slot);
            if (rc) {
                r->state = RS_FAILED;
                r->error = rc;
                ++S->n_failed;
                if (S->notify) S->completed.emplace_back(r->id, r->state);
                progress = true;
                continue;
            }
            S->slot_busy[slot] = true;
            S->running.push_back(r->id);
            progress = true;
        }
        // 3. admit commits while a slot and memory are free
        while (!S->pend_by_id.empty()) {
            const auto next = next_commit(S);
            if (next.second < 0) break;  // no slot for any queued request now
            const uint64_t id = next.first;
            const int slot = next.second;
            Request *r = S->reqs[id].get();
            if (S->in_use + r->bytes > S->budget) break;  // wait for openings to free HBM
            S->pend_by_id.erase(id);
            S->pend_by_size.erase({r->bytes, id});
            S->in_use += r->bytes;
            r->slot = slot;
            r->state = RS_RUNNING;
            r->t_start = S->ns();
            const int rc = start_commit(S, r, slot);
            if (rc) {
                // whatever it allocated goes back to the pool behind what it enqueued
                free_commit_buffers(S, r, slot, false);
                if (r->d_msg) cudaFreeAsync(r->d_msg, S->streams[slot]);
                r->d_msg = nullptr;
                r->state = RS_FAILED;
                r->error = rc;
                S->in_use -= r->bytes;
                ++S->n_failed;
                if (S->notify) S->completed.emplace_back(r->id, r->state);
                progress = true;
                continue;
            }
            S->slot_busy[slot] = true;
            S->running.push_back(r->id);
            progress = true;
        }
        if (progress) S->cv_done.notify_all();
        if (S->running.empty() && S->pend_by_id.empty() && S->pending_opens.empty()) {
            S->cv_work.wait_for(lk, std::chrono::milliseconds(50));
        } else if (!progress) {
            // a slot's host callback or a submission wakes this; the timeout
            // covers a callback that ran between the check and the wait
            S->cv_work.wait_for(lk, std::chrono::microseconds(200), [&] {
                return S->stop || S->wakes.load(std::memory_order_acquire) != seen_wakes;
            });
        }
    }
}

}  // namespace

extern "C" {

int bz_server_create(bz_ctx *ctx, int n_slots, uint64_t mem_budget_bytes, size_t queue_cap,
                     bz_server **out) {
    if (!ctx || !out || n_slots < 1 || n_slots > 32) return BZ_ERR_ARG;
    bz_server *S = new bz_server();
    S->ctx = ctx;
    S->n_slots = n_slots;
    S->budget = mem_budget_bytes ? mem_budget_bytes : ctx->budget;
    S->queue_cap = queue_cap ? queue_cap : 1 << 20;
    S->streams.assign(n_slots, nullptr);
    S->n_hi = std::max(1, n_slots / 3);
    S->n_mid = (n_slots - S->n_hi) / 2;
    S->slot_done.assign(n_slots, nullptr);
    S->slot_host.assign(n_slots, nullptr);
    S->slot_host_bytes.assign(n_slots, 0);
    S->slot_busy.assign(n_slots, false);
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    uint64_t keep = UINT64_MAX;
    int no = 0;
    if (cudaMemPoolCreate(&S->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess ||
        cudaMemPoolSetAttribute(S->pool, cudaMemPoolReuseAllowInternalDependencies, &no) !=
            cudaSuccess) {
        cudaGetLastError();
        if (S->pool) cudaMemPoolDestroy(S->pool);
        delete S;
        return BZ_ERR_CUDA;
    }
    for (int i = 0; i < n_slots; ++i) {
        if (cudaStreamCreateWithPriority(&S->streams[i], cudaStreamNonBlocking,
                                         i < S->n_hi ? greatest
                                         : i < S->n_hi + S->n_mid ? (greatest + least) / 2
                                                                  : least) != cudaSuccess ||
            cudaEventCreateWithFlags(&S->slot_done[i], cudaEventDisableTiming) != cudaSuccess ||
            ensure_slot_host(S, i, 1 << 20) != BZ_OK) {
            cudaGetLastError();
            for (int j = 0; j <= i; ++j) {
                if (S->streams[j]) cudaStreamDestroy(S->streams[j]);
                if (S->slot_done[j]) cudaEventDestroy(S->slot_done[j]);
                if (S->slot_host[j]) cudaFreeHost(S->slot_host[j]);
            }
            cudaMemPoolDestroy(S->pool);
            delete S;
            return BZ_ERR_CUDA;
        }
    }
    S->t0 = Clock::now();
    S->thr = std::thread(scheduler, S);
    *out = S;
    return BZ_OK;
}

int bz_server_set_policy(bz_server *S, int admit_order, uint32_t aging_ms,
                         int high_priority_log_size) {
    if (!S || (admit_order != BZ_ADMIT_FIFO && admit_order != BZ_ADMIT_SMALLEST) ||
        high_priority_log_size < -1 || high_priority_log_size > 62)
        return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    S->admit_order = admit_order;
    S->aging_ns = (int64_t)aging_ms * 1000000;
    S->small_log = high_priority_log_size;
    return BZ_OK;
}

}  // extern "C"

namespace {

int submit(bz_server *S, const uint64_t *host_msg, size_t n_words, const bz_params *params,
           const uint64_t *positions, size_t q, bool auto_open, uint64_t *request_id) {
    if (!S || !host_msg || !request_id || (auto_open && q && !positions)) return BZ_ERR_ARG;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, n_words, why);
    if (rc) return set_msg(S->ctx, rc, why);
    if (merkle_scratch_bytes(s)) return set_msg(S->ctx, BZ_ERR_SHAPE, "leaf too wide for serving");
    auto r = std::make_unique<Request>();
    r->shape = s;
    r->host_msg = host_msg;
    r->bytes = request_bytes(s);
    if (r->bytes > S->budget) return set_msg(S->ctx, BZ_ERR_NOMEM, "request exceeds the budget");
    if (auto_open) {
        if (!set_positions(r.get(), positions, q)) return BZ_ERR_ARG;
        r->auto_open = true;
    }
    std::lock_guard<std::mutex> g(S->mu);
    if (S->pend_by_id.size() >= S->queue_cap) return BZ_ERR_BUSY;
    r->id = S->next_id++;
    r->t_submit = S->ns();
    *request_id = r->id;
    S->pend_by_id.insert(r->id);
    S->pend_by_size.insert({r->bytes, r->id});
    S->reqs[r->id] = std::move(r);
    S->cv_work.notify_one();
    return BZ_OK;
}

}  // namespace

extern "C" {

int bz_server_submit_commit(bz_server *S, const uint64_t *host_msg, size_t n_words,
                            const bz_params *params, uint64_t *request_id) {
    return submit(S, host_msg, n_words, params, nullptr, 0, false, request_id);
}

int bz_server_submit_commit_open(bz_server *S, const uint64_t *host_msg, size_t n_words,
                                 const bz_params *params, const uint64_t *positions, size_t q,
                                 uint64_t *request_id) {
    return submit(S, host_msg, n_words, params, positions, q, true, request_id);
}

int bz_server_submit_open(bz_server *S, uint64_t id, const uint64_t *positions, size_t q) {
    if (!S || (q && !positions)) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
    Request *r = it->second.get();
    if (r->state != RS_COMMITTED) return BZ_ERR_STATE;
    if (!set_positions(r, positions, q)) return BZ_ERR_ARG;
    r->state = RS_OPEN_QUEUED;
    r->t_open_submit = S->ns();
    S->pending_opens.push_back(id);
    S->cv_work.notify_one();
    return BZ_OK;
}

int bz_server_next_done(bz_server *S, uint64_t *ids, int *states, size_t cap, size_t *n,
                        uint32_t timeout_us) {
    if (!S || !n || (cap && (!ids || !states))) return BZ_ERR_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    S->notify = true;
    *n = 0;
    if (S->completed.empty() && timeout_us)
        S->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us),
                            [&] { return !S->completed.empty(); });
    while (*n < cap && !S->completed.empty()) {
        ids[*n] = S->completed.front().first;
        states[(*n)++] = S->completed.front().second;
        S->completed.pop_front();
    }
    return BZ_OK;
}

int bz_server_poll(bz_server *S, uint64_t id, int *state) {
    if (!S || !state) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
    *state = it->second->state;
    return it->second->state == RS_FAILED ? it->second->error : BZ_OK;
}

int bz_server_wait(bz_server *S, uint64_t id, int target_state, uint32_t timeout_ms) {
    if (!S) return BZ_ERR_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms);
    while (true) {
        auto it = S->reqs.find(id);
        if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
        if (it->second->state == RS_FAILED) return it->second->error ? it->second->error : BZ_ERR_CUDA;
        if (it->second->state >= target_state) return BZ_OK;
        if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) return BZ_ERR_TIMEOUT;
    }
}

int bz_server_root(bz_server *S, uint64_t id, uint8_t root[32]) {
    if (!S || !root) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
    if (it->second->state < RS_COMMITTED || it->second->state == RS_FAILED) return BZ_ERR_STATE;
    memcpy(root, it->second->root, 32);
    return BZ_OK;
}

int bz_server_open_result(bz_server *S, uint64_t id, uint64_t *rows, size_t rows_cap_words,
                          uint8_t *proof, size_t proof_cap, size_t *n_rows, size_t *n_hashes) {
    if (!S) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
    Request *r = it->second.get();
    if (r->state != RS_OPENED) return BZ_ERR_STATE;
    const size_t q = r->positions.size(), nn = r->node_idx.size();
    const size_t row_words = (size_t)2 << r->shape.log_lanes;
    if (n_rows) *n_rows = q;
    if (n_hashes) *n_hashes = nn;
    if (rows) {
        if (rows_cap_words < q * row_words) return BZ_ERR_ARG;
        if (q) memcpy(rows, r->rows.data(), q * row_words * 8);
    }
    if (proof) {
        if (proof_cap < nn) return BZ_ERR_ARG;
        if (nn) memcpy(proof, r->nodes.data(), nn * 32);
    }
    return BZ_OK;
}

// Timestamps in nanoseconds since server start: submit, start, committed,
// open submitted, opened.
int bz_server_times(bz_server *S, uint64_t id, int64_t times[5]) {
    if (!S || !times) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
    Request *r = it->second.get();
    times[0] = r->t_submit;
    times[1] = r->t_start;
    times[2] = r->t_committed;
    times[3] = r->t_open_submit;
    times[4] = r->t_opened;
    return BZ_OK;
}

// Forget a finished request (opened or failed) and its host buffers.
int bz_server_release(bz_server *S, uint64_t id) {
    if (!S) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return BZ_ERR_NOTFOUND;
    Request *r = it->second.get();
    if (r->state != RS_OPENED && r->state != RS_FAILED) return BZ_ERR_STATE;
    if (r->state == RS_FAILED && r->commit) {
        free_commit_buffers(S, r, r->slot, false);
        S->in_use -= r->bytes - r->shape.msg_words() * 16;
    }
    S->reqs.erase(it);
    return BZ_OK;
}

int bz_server_stats(bz_server *S, uint64_t *committed, uint64_t *opened, uint64_t *failed,
                    uint64_t *in_use, uint64_t *queued) {
    if (!S) return BZ_ERR_ARG;
    std::lock_guard<std::mutex> g(S->mu);
    if (committed) *committed = S->n_committed;
    if (opened) *opened = S->n_opened;
    if (failed) *failed = S->n_failed;
    if (in_use) *in_use = S->in_use;
    if (queued) *queued = S->pend_by_id.size() + S->pending_opens.size();
    return BZ_OK;
}

int bz_server_destroy(bz_server *S) {
    if (!S) return BZ_ERR_ARG;
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    S->thr.join();
    for (auto s : S->streams) cudaStreamSynchronize(s);
    for (auto &kv : S->reqs) {
        Request *r = kv.second.get();
        if (r->commit) free_commit_buffers(S, r, 0, false);
        if (r->d_msg) cudaFreeAsync(r->d_msg, S->streams[0]);
    }
    drop_spares(S, S->streams[0]);
    for (auto s : S->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    cudaMemPoolDestroy(S->pool);
    for (int i = 0; i < S->n_slots; ++i) {
        cudaEventDestroy(S->slot_done[i]);
        cudaFreeHost(S->slot_host[i]);
    }
    delete S;
    return BZ_OK;
}

}  // extern "C"
