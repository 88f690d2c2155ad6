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
// Nothing on the request path synchronises the device: device buffers come
// from the stream-ordered pool (cudaMallocAsync / cudaFreeAsync on the slot's
// stream), and each slot owns its completion event and a grow-only pinned
// staging buffer for the root, rows and proof nodes, which the scheduler
// copies into the request when the slot's work completes.  A completion
// queue (bz_server_next_done) hands state changes to the caller without
// polling every request.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <algorithm>
#include <deque>
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
    bool auto_open = false;  // queue the opening as soon as the commit is done
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
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> slot_done;    // completion of the slot's work
    std::vector<uint8_t *> slot_host;      // pinned staging (root, rows, nodes)
    std::vector<size_t> slot_host_bytes;
    std::vector<bool> slot_busy;
    std::deque<std::pair<uint64_t, int>> completed;  // (id, new state) for bz_server_next_done
    bool notify = false;                   // completions are recorded once asked for
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> pending_commits, pending_opens;
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

// Start a commit on a free slot (caller holds the lock).
int start_commit(bz_server *S, Request *r, int slot) {
    bz_ctx *ctx = S->ctx;
    cudaStream_t st = S->streams[slot];
    const Shape &s = r->shape;
    cudaError_t e = cudaMallocAsync((void **)&r->d_msg, s.msg_words() * 16, st);
    if (e != cudaSuccess) return BZ_ERR_NOMEM;
    bz_commitment *c = new bz_commitment();
    c->ctx = ctx;
    c->shape = s;
    c->cw_bytes = s.cw_words() * 16;
    c->tree_bytes = s.tree_nodes() * 32;
    e = cudaMallocAsync((void **)&c->d_cw, c->cw_bytes, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&c->d_tree, c->tree_bytes, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (c->d_cw) cudaFreeAsync(c->d_cw, st);
        cudaFreeAsync(r->d_msg, st);
        r->d_msg = nullptr;
        delete c;
        return BZ_ERR_NOMEM;
    }
    r->commit = c;
    cudaMemcpyAsync(r->d_msg, r->host_msg, s.msg_words() * 16, cudaMemcpyHostToDevice, st);
    const uint4 *d_tw = nullptr;
    int rc = get_twiddles(ctx, s.k_code(), &d_tw);
    if (rc) return rc;
    int n = launch_commit_kernels(ctx, s, schedule_for(ctx, s), r->d_msg, c->d_cw, c->d_tree,
                                  d_tw, st, nullptr);
    ctx->launches += (uint64_t)n;
    cudaFreeAsync(r->d_msg, st);
    r->d_msg = nullptr;
    cudaMemcpyAsync(S->slot_host[slot], c->d_tree + (s.tree_nodes() - 1) * 32, 32,
                    cudaMemcpyDeviceToHost, st);
    cudaEventRecord(S->slot_done[slot], st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return BZ_ERR_CUDA;
    return BZ_OK;
}

int start_open(bz_server *S, Request *r, int slot) {
    bz_ctx *ctx = S->ctx;
    cudaStream_t st = S->streams[slot];
    const Shape &s = r->shape;
    const size_t q = r->positions.size(), nn = r->node_idx.size();
    const size_t row_bytes = s.leaf_bytes();
    // pinned staging: rows then nodes; device: positions, node indices,
    // rows, nodes in one stream-ordered allocation
    int rc = ensure_slot_host(S, slot, q * row_bytes + nn * 32 + 32);
    if (rc) return rc;
    const size_t o_idx = q * 8, o_rows = (o_idx + nn * 8 + 15) & ~(size_t)15;
    const size_t o_nodes = o_rows + q * row_bytes, dev_bytes = o_nodes + nn * 32 + 16;
    uint8_t *d = nullptr;
    if (cudaMallocAsync((void **)&d, dev_bytes, st) != cudaSuccess) {
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
    uint8_t *h = S->slot_host[slot];
    if (q) cudaMemcpyAsync(h, d_rows, q * row_bytes, cudaMemcpyDeviceToHost, st);
    if (nn) cudaMemcpyAsync(h + q * row_bytes, d_nodes, nn * 32, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    cudaEventRecord(S->slot_done[slot], st);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

void free_commit_buffers(bz_server *S, Request *r, int slot) {
    if (r->commit) {
        cudaStream_t st = S->streams[slot >= 0 ? slot : 0];
        cudaFreeAsync(r->commit->d_cw, st);
        cudaFreeAsync(r->commit->d_tree, st);
        delete r->commit;
        r->commit = nullptr;
    }
}

int free_slot(bz_server *S) {
    for (int i = 0; i < S->n_slots; ++i)
        if (!S->slot_busy[i]) return i;
    return -1;
}

void scheduler(bz_server *S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop) {
        bool progress = false;
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
            if (q != cudaSuccess) {
                cudaGetLastError();
                r->state = RS_FAILED;
                r->error = BZ_ERR_CUDA;
                ++S->n_failed;
            } else if (r->state == RS_RUNNING) {
                memcpy(r->root, h, 32);
                r->commit->root_ready = true;
                memcpy(r->commit->root, r->root, 32);
                r->state = RS_COMMITTED;
                r->t_committed = S->ns();
                S->in_use -= r->shape.msg_words() * 16;  // staging buffer released
                ++S->n_committed;
                if (r->auto_open) {
                    if (S->notify) S->completed.emplace_back(r->id, RS_COMMITTED);
                    r->state = RS_OPEN_QUEUED;
                    r->t_open_submit = r->t_committed;
                    S->pending_opens.push_back(r->id);
                }
            } else if (r->state == RS_OPENING) {
                const size_t q_rows = r->positions.size(), nn = r->node_idx.size();
                const size_t row_words = (size_t)2 << r->shape.log_lanes;
                r->rows.assign((const uint64_t *)h, (const uint64_t *)h + q_rows * row_words);
                r->nodes.assign(h + q_rows * row_words * 8, h + q_rows * row_words * 8 + nn * 32);
                r->state = RS_OPENED;
                r->t_opened = S->ns();
                free_commit_buffers(S, r, r->slot);
                S->in_use -= r->bytes - r->shape.msg_words() * 16;
                ++S->n_opened;
            }
            if (S->notify && !(r->auto_open && r->state == RS_OPEN_QUEUED))
                S->completed.emplace_back(r->id, r->state);
            S->running[i] = S->running.back();
            S->running.pop_back();
        }
        // 2. openings first (they free memory)
        while (!S->pending_opens.empty()) {
            const int slot = free_slot(S);
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
        // 3. admit commits in arrival order while a slot and memory are free
        while (!S->pending_commits.empty()) {
            const int slot = free_slot(S);
            if (slot < 0) break;
            Request *r = S->reqs[S->pending_commits.front()].get();
            if (S->in_use + r->bytes > S->budget) break;  // wait for openings to free HBM
            S->pending_commits.pop_front();
            S->in_use += r->bytes;
            r->slot = slot;
            r->state = RS_RUNNING;
            r->t_start = S->ns();
            const int rc = start_commit(S, r, slot);
            if (rc) {
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
        if (S->running.empty() && S->pending_commits.empty() && S->pending_opens.empty()) {
            S->cv_work.wait_for(lk, std::chrono::milliseconds(50));
        } else if (!progress) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
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
    S->streams.resize(n_slots);
    S->slot_done.resize(n_slots);
    S->slot_host.assign(n_slots, nullptr);
    S->slot_host_bytes.assign(n_slots, 0);
    S->slot_busy.assign(n_slots, false);
    for (int i = 0; i < n_slots; ++i) {
        if (cudaStreamCreateWithFlags(&S->streams[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&S->slot_done[i], cudaEventDisableTiming) != cudaSuccess ||
            ensure_slot_host(S, i, 64 << 10) != BZ_OK) {
            cudaGetLastError();
            for (int j = 0; j <= i; ++j) {
                if (S->streams[j]) cudaStreamDestroy(S->streams[j]);
                if (S->slot_done[j]) cudaEventDestroy(S->slot_done[j]);
                if (S->slot_host[j]) cudaFreeHost(S->slot_host[j]);
            }
            delete S;
            return BZ_ERR_CUDA;
        }
    }
    S->t0 = Clock::now();
    S->thr = std::thread(scheduler, S);
    *out = S;
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
    if (S->pending_commits.size() >= S->queue_cap) return BZ_ERR_BUSY;
    r->id = S->next_id++;
    r->t_submit = S->ns();
    *request_id = r->id;
    S->pending_commits.push_back(r->id);
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
        free_commit_buffers(S, r, r->slot);
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
    if (queued) *queued = S->pending_commits.size() + S->pending_opens.size();
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
        if (r->commit) free_commit_buffers(S, r, 0);
    }
    for (auto s : S->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    for (int i = 0; i < S->n_slots; ++i) {
        cudaEventDestroy(S->slot_done[i]);
        cudaFreeHost(S->slot_host[i]);
    }
    delete S;
    return BZ_OK;
}

}  // extern "C"
