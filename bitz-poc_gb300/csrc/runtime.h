// Definitions of the opaque ABI handles and helpers shared by the host
// runtime translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <thread>
#include <future>
#include <functional>
#include <deque>
#include <condition_variable>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "bz_internal.h"

struct bz_commitment {
    bz_ctx *ctx = nullptr;
    bz::Shape shape;
    uint4 *d_cw = nullptr;
    uint8_t *d_tree = nullptr;
    size_t cw_bytes = 0, tree_bytes = 0;
    bool root_ready = false;
    uint8_t root[32] = {0};
    cudaEvent_t done = nullptr;       // async commits: root copied to root_slot
    const uint8_t *root_slot = nullptr;
};

// Auxiliary stream (and its events) paired with a launching stream for the
// two-stream pipelined commit.
struct bz_aux_stream {
    cudaStream_t s = nullptr;
    cudaEvent_t ev[16] = {};
};

struct bz_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0;
    std::atomic<uint64_t> in_use{0};
    std::atomic<uint64_t> launches{0};
    std::mutex err_mu, tw_mu, sched_mu, live_mu;
    std::string last_error;
    std::map<int, const uint4 *> twiddles;  // by k_code
    std::map<uint64_t, uint32_t> schedules;  // by shape key
    std::set<bz_commitment *> live;
    uint8_t *scratch = nullptr;
    size_t scratch_bytes = 0;
    void *h_small = nullptr;  // 4 KiB pinned
    void *d_small = nullptr;  // 4 KiB device (zeroed; word 192 is the message ticket)
    void *h_mbox = nullptr;   // 4 KiB mapped pinned: sumcheck message mailbox
    void *d_mbox = nullptr;   // its device view
    uint32_t mbox_seq = 0;    // last posted sequence number
    uint32_t gate_seq = 0;    // last armed fold's gate number
    bool arm_folds = true;    // cleared after a gate ran out (the prover stops arming)
    uint32_t pow_seq = 0;     // last proof-of-work search's mailbox number
    bool pow_ready = false;   // the search's device counters hold their idle values
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex aux_mu;
    std::map<cudaStream_t, bz_aux_stream> aux;
    cudaStream_t copy_stream = nullptr;  // host-to-device uploads of async commits
    cudaStream_t side_stream = nullptr;  // openings that overlap the context stream's work
    // One helper thread (started on first use) runs side-stream work queued by
    // side_async; reusing it spares a thread start per proof.
    std::mutex side_mu;
    std::condition_variable side_cv;
    std::deque<std::function<void()>> side_jobs;
    std::thread side_thread;
    bool side_stop = false;
    uint64_t root_ring = 0;              // next 32-byte slot of h_small for async roots
};

// A reusable batch plan (batch.cu; the persistent form is built in persist.cu).
struct bz_batch_plan {
    bz_ctx *ctx = nullptr;
    std::vector<bz::Shape> shapes;
    std::vector<const uint4 *> msgs;
    std::vector<bz_commitment *> commits;
    std::vector<uint32_t> schedules;
    uint8_t *d_roots = nullptr;
    int use_graph = 0;
    int n_branches = 1;
    std::vector<cudaStream_t> branches;
    std::vector<cudaEvent_t> fork_join;  // [0] fork, [1..n] joins
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // persistent plans: one device block holding the steps, the commit table
    // and the scheduler state; the graph resets the state and runs the kernel
    void *d_persist = nullptr;
    uint32_t *d_persist_err = nullptr;  // nonzero after a CTA gave up waiting
    std::vector<char> persist_args;      // the kernel's arguments (relaunch by the stall check)
    size_t persist_state_bytes = 0;
};

// Return BZ_ERR_CUDA (recording the failing call) when a CUDA call fails.
#define BZ_CUDA(ctx, call)                                                      \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) return bz::set_err((ctx), BZ_ERR_CUDA, #call, e_); \
    } while (0)

namespace bz {
inline uint64_t shape_key(const Shape &s) {
    return (uint64_t)s.log_msg_len | ((uint64_t)s.log_inv_rate << 8) |
           ((uint64_t)s.log_lanes << 16) | ((uint64_t)s.hash_kind << 24);
}
int set_err(bz_ctx *ctx, int code, const char *what, cudaError_t e);
int set_msg(bz_ctx *ctx, int code, const std::string &msg);
int shape_from_params(const bz_params *p, Shape &s, size_t n_words, std::string &why);
int dev_alloc(bz_ctx *ctx, size_t bytes, void **p, bool budgeted);
void dev_free(bz_ctx *ctx, void *p, size_t bytes, bool budgeted);
int ensure_scratch(bz_ctx *ctx, size_t bytes);
// Run job on the context's helper thread; the future holds its status.
std::future<int> side_async(bz_ctx *ctx, std::function<int()> job);
void side_shutdown(bz_ctx *ctx);
// Opened rows and multi-proof of a commitment on stream st (synchronised on
// return); the C ABI calls run them on the context stream.
int commitment_rows_on(bz_commitment *c, const uint64_t *positions, size_t q, uint64_t *out,
                       cudaStream_t st);
int commitment_multiproof_on(bz_commitment *c, const uint64_t *positions, size_t q, uint8_t *out,
                             size_t cap, size_t *n_hashes, cudaStream_t st);
int get_twiddles(bz_ctx *ctx, int ell, const uint4 **out);
uint32_t schedule_for(bz_ctx *ctx, const Shape &s);
int alloc_commitment(bz_ctx *ctx, const Shape &s, bz_commitment **out,
                     bool with_codeword = true);
int enqueue_commit(bz_ctx *ctx, const Shape &s, const uint4 *d_msg, bz_commitment *c,
                   cudaStream_t st, uint32_t schedule);
int fetch_root(bz_commitment *c);
// The auxiliary stream paired with `st` (created on first use; call before a
// stream capture that will use it).
bz_aux_stream *get_aux(bz_ctx *ctx, cudaStream_t st);
// NTT + Merkle kernels of one commit on `st`: the two-stream pipeline when the
// schedule asks for it and the shape allows it, else the plain sequence.
int launch_commit_kernels(bz_ctx *ctx, const Shape &s, uint32_t schedule, const uint4 *d_msg,
                          uint4 *d_cw, uint8_t *d_tree, const uint4 *d_tw, cudaStream_t st,
                          LaunchLog *log);

// Sumcheck rounds on the context stream.  fold_launch enqueues one
// fold-and-message round with a known challenge; msg_wait returns its
// message.  A fold can also be armed: enqueued before its challenge exists,
// behind the round in flight, so that its launch overlaps the host's wait and
// transcript work; fold_open posts the challenge, fold_cancel withdraws it.
// Between fold_arm and fold_open/fold_cancel the host must not wait on the
// context stream (the armed kernel would hold it until its time limit).
struct ArmedFold {
    uint32_t gate_seq = 0;
    uint32_t msg_seq = 0;
    const uint64_t *f = nullptr, *b = nullptr;
    uint64_t *nf = nullptr, *nb = nullptr;
    size_t n = 0;
    bool live = false;
};
int fold_launch(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb, uint32_t *msg_seq);
bool fold_armable(const bz_ctx *ctx, size_t n);
int fold_arm(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n, uint64_t *d_nf,
             uint64_t *d_nb, ArmedFold *a, uint64_t limit_ns = kGateLimitNs);
void fold_open(bz_ctx *ctx, ArmedFold *a, const uint64_t r[2]);
int fold_cancel(bz_ctx *ctx, ArmedFold *a);
// After a gated round's message failed to arrive: drains the stream and
// reports (and clears) whether a gate ran out, which then stops arming on the
// context.
bool gate_gave_up(bz_ctx *ctx);
int msg_wait(bz_ctx *ctx, uint32_t seq, uint64_t u0[2], uint64_t u2[2]);
// Spin until the 32-bit word at byte `offset` of the mapped mailbox reads
// seq, checking the context stream for errors (and for having gone idle
// without posting) every few hundred spins; 60 s limit.
int mapped_wait(bz_ctx *ctx, size_t offset, uint32_t seq, const char *what);
// Zero the message ticket (after a round that may have stopped part-way).
void reset_msg_ticket(bz_ctx *ctx);
// The mailbox post for the next message kernel on the context stream (its
// sequence number is what msg_wait then waits for).
MsgPost next_msg_post(bz_ctx *ctx);
}  // namespace bz
