/*
 * bitz_gpu.h -- C ABI of the GB300 (sm_103a) Ligerito / Reed-Solomon
 * commitment library.
 *
 * Every entry point returns a bz_status code; nothing unwinds across the ABI.
 * Buffers are plain pointers and sizes.  GF(2^128) elements are two
 * little-endian uint64 words {lo, hi} (the reference's repr(C) Gf128,
 * vendor/field/src/gf128.rs:91-96), so an array of n elements is uint64_t[2n]
 * and its byte image is the reference's codeword byte view
 * (flock-core/src/pcs/commit.rs:284-292).
 *
 * Reference paths are relative to the BitZ-PoC project root; "flock-core/"
 * abbreviates vendor/flock-mod/crates/flock-core/.
 */
#ifndef BITZ_GPU_H
#define BITZ_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BZ_ABI_VERSION 1

typedef enum {
    BZ_OK = 0,
    BZ_ERR_ARG = 1,      /* null pointer, bad size, bad enum */
    BZ_ERR_SHAPE = 2,    /* the reference's PcsParams::validate / commit asserts */
    BZ_ERR_CUDA = 3,     /* a CUDA runtime call failed (bz_last_error has text) */
    BZ_ERR_NOMEM = 4,    /* device allocation failed or the memory budget is exceeded */
    BZ_ERR_BUSY = 5,     /* server queue full */
    BZ_ERR_TIMEOUT = 6,  /* a bounded wait ran out */
    BZ_ERR_STATE = 7,    /* handle in the wrong state (e.g. opened twice, freed) */
    BZ_ERR_NOTFOUND = 8, /* unknown request id; no proof-of-work nonce in the range */
    /* proof codec (src/proof_codec.rs:14-25 CodecError) */
    BZ_ERR_TRUNCATED = 9,    /* the stream ended before a field */
    BZ_ERR_NONCANONICAL = 10, /* a field encoded non-minimally */
    BZ_ERR_DECODE = 11       /* the bincode LigeritoProof blob does not decode */
} bz_status;

/* Merkle hash (flock-core/src/hash.rs:21-27; merkle.rs:203-232). */
typedef enum { BZ_HASH_SHA256 = 0, BZ_HASH_BLAKE3 = 1 } bz_hash_kind;

/* flock-core PcsParams (commit.rs:31-137) expressed in the packed domain:
 *   log_msg_len    = m - LOG_PACKING (m - 7)
 *   log_inv_rate   = r  (>= 1)
 *   log_batch_size = log2 of the interleaved lanes (<= log_msg_len)
 * Derived: log_dim = log_msg_len - log_batch_size, k_code = log_dim + r,
 * n_leaves = 2^k_code, leaf bytes = 16 << log_batch_size. */
typedef struct {
    uint32_t log_msg_len;
    uint32_t log_inv_rate;
    uint32_t log_batch_size;
    uint32_t hash_kind; /* bz_hash_kind */
} bz_params;

typedef struct bz_ctx bz_ctx;
typedef struct bz_commitment bz_commitment; /* device-resident ProverData + root */
typedef struct bz_ligerito_proof bz_ligerito_proof; /* flock's LigeritoProof, host side */

/* ---- context ---------------------------------------------------------- */
const char *bz_status_string(int status);
/* Last error text recorded on this context (never NULL). */
const char *bz_last_error(const bz_ctx *ctx);
int bz_abi_version(void);
/* One context per device.  mem_budget_bytes caps what the context keeps on
 * the device for commitments and scratch (0 = 90 % of free memory). */
int bz_ctx_create(int device, uint64_t mem_budget_bytes, bz_ctx **out);
int bz_ctx_destroy(bz_ctx *ctx);
/* The cudaStream_t every entry point of this context enqueues on. */
void *bz_ctx_stream(bz_ctx *ctx);
int bz_ctx_synchronize(bz_ctx *ctx);
/* Bytes currently held by live commitments and scratch; budget. */
int bz_ctx_memory(const bz_ctx *ctx, uint64_t *in_use, uint64_t *budget);
/* Device allocation helpers for callers that hold no other CUDA runtime. */
int bz_device_alloc(bz_ctx *ctx, size_t bytes, void **dptr);
int bz_device_free(bz_ctx *ctx, void *dptr);
int bz_memcpy_h2d(bz_ctx *ctx, void *dst, const void *src, size_t bytes);
int bz_memcpy_d2h(bz_ctx *ctx, void *dst, const void *src, size_t bytes);
int bz_host_alloc_pinned(size_t bytes, void **hptr);
int bz_host_free_pinned(void *hptr);
/* Stream-ordered timing on the context stream: begin records an event, end
 * records a second one, synchronizes, and returns the elapsed milliseconds. */
int bz_timer_begin(bz_ctx *ctx);
int bz_timer_end(bz_ctx *ctx, float *ms);
/* Number of this library's kernels enqueued on the context so far. */
uint64_t bz_kernel_launches(const bz_ctx *ctx);

/* ---- commit ------------------------------------------------------------ */
/* Replaces flock_core::pcs::commit::commit(z_packed, params) -> (Commitment,
 * ProverData)  (flock-core/src/pcs/commit.rs:180-200; commit_into :209-232;
 * finalize_commit :262-315), reached from BitZ through BinaryPcs::commit
 * (src/binary_pcs.rs:313-318) and commit_rs_flock_from_rows
 * (src/ligerito_flock.rs:198-245).
 * `msg` is host memory of n_words = 2^log_msg_len elements, laid out
 * msg[col * 2^log_batch_size + lane].  The codeword and Merkle tree stay on
 * the device inside *out until bz_commitment_free.  root receives the 32-byte
 * Merkle root (Commitment::root).  Synchronous. */
int bz_commit(bz_ctx *ctx, const uint64_t *msg, size_t n_words, const bz_params *params,
              bz_commitment **out, uint8_t root[32]);
/* Same, with the message already in device memory (no host copies). */
int bz_commit_device(bz_ctx *ctx, const uint64_t *d_msg, size_t n_words,
                     const bz_params *params, bz_commitment **out, uint8_t root[32]);
/* Enqueue only: no synchronization, root readable after bz_ctx_synchronize
 * through bz_commitment_root.  Used by graph capture and the benchmark. */
int bz_commit_device_async(bz_ctx *ctx, const uint64_t *d_msg, size_t n_words,
                           const bz_params *params, bz_commitment **out);
/* Asynchronous bz_commit: the host message is uploaded on the context's copy
 * stream and the kernels follow on the context stream, so the upload of one
 * commit overlaps the kernels of the previous one.  Returns without waiting;
 * `msg` must stay valid (and should be pinned) until bz_commitment_root
 * returns for this handle.  At most 96 asynchronous commits may be pending
 * (their roots wait in a ring of pinned slots). */
int bz_commit_async(bz_ctx *ctx, const uint64_t *msg, size_t n_words, const bz_params *params,
                    bz_commitment **out);
/* Root of a commitment (waits for that commitment only). */
int bz_commitment_root(bz_commitment *c, uint8_t root[32]);
int bz_commitment_params(const bz_commitment *c, bz_params *params);
/* Device pointers of the resident codeword (2^(k_code+log_batch_size)
 * elements, cw[pos * lanes + lane]) and flat tree ((2 n_leaves - 1) * 32 B,
 * leaves first, root last -- flock-core/src/merkle.rs:15-22). */
int bz_commitment_device_ptrs(const bz_commitment *c, const uint64_t **d_codeword,
                              const uint8_t **d_tree);
int bz_commitment_copy_codeword(bz_commitment *c, uint64_t *out, size_t n_words);
int bz_commitment_copy_tree(bz_commitment *c, uint8_t *out, size_t n_nodes);
/* Opened rows for sorted query positions: out[i] = the 2^log_batch_size
 * lanes at position positions[i] (the open_initial row gather of
 * flock-core/src/pcs/ligerito.rs:3472-3482). */
int bz_commitment_rows(bz_commitment *c, const uint64_t *positions, size_t q, uint64_t *out);
/* merkle_multi_proof (flock-core/src/merkle.rs:688-741): sibling hashes in
 * the reference's bottom-up sorted order; *n_hashes receives the count.
 * out must hold cap hashes. */
int bz_commitment_multiproof(bz_commitment *c, const uint64_t *positions, size_t q,
                             uint8_t *out, size_t cap, size_t *n_hashes);
int bz_commitment_free(bz_commitment *c);

/* ---- lane-sharded BLAKE3 commit (one commit over several GPUs) ----------- */
/* No counterpart in the reference, which commits on one machine.  It splits
 * flock-core's commit (commit.rs:180-315) by lanes: every lane's NTT is
 * independent (flock-core/src/ntt/additive_ntt_f128.rs:176-191) and a BLAKE3
 * leaf is the tree over its 1 KiB chunks of 64 lanes, the chunk's index in
 * the leaf being its counter (flock-core/src/merkle.rs:160-201).
 *
 * Rank `rank` of `world` (a power of two; 2^log_batch_size / world >= 64
 * lanes; BLAKE3 only, else BZ_ERR_SHAPE) commits its lanes
 * [rank Ls, (rank+1) Ls), Ls = 2^log_batch_size / world, from its message
 * shard msg_shard[col * Ls + j] = msg[col * 2^log_batch_size + rank * Ls + j]
 * (n_words = 2^log_msg_len / world).  `params` are the whole commit's.  The
 * returned handle holds the shard's codeword (its lanes of every position,
 * cw[pos * Ls + j]: bz_commitment_rows gives the rank's slice of opened rows)
 * and as its leaves the CV of each position's run of chunks
 * (bz_commitment_leaf_cvs); its own root means nothing.  Synchronous. */
int bz_commit_shard(bz_ctx *ctx, const uint64_t *msg_shard, size_t n_words,
                    const bz_params *params, uint32_t world, uint32_t rank, bz_commitment **out);
/* Same with the shard in device memory; enqueue only. */
int bz_commit_shard_device(bz_ctx *ctx, const uint64_t *d_msg_shard, size_t n_words,
                           const bz_params *params, uint32_t world, uint32_t rank,
                           bz_commitment **out);
/* The n_leaves x 32-byte leaves of a commitment's tree (a shard's per-position
 * chunk-run CVs: what the ranks exchange, an all-gather of 32 bytes per
 * position per rank). */
int bz_commitment_leaf_cvs(bz_commitment *c, uint8_t *out, size_t n_leaves);
/* The whole commit's tree from every rank's leaf CVs (host, world x n_leaves
 * x 32 bytes in rank order): each leaf CV is the merge of its position's world
 * CVs, then the Merkle levels.  *out is a tree-only handle (root, copy_tree,
 * multiproof; its codeword stays split over the ranks, so bz_commitment_rows
 * and copy_codeword return BZ_ERR_STATE); root receives the commit's root. */
int bz_merkle_from_shards(bz_ctx *ctx, const uint8_t *cvs, uint32_t world,
                          const bz_params *params, bz_commitment **out, uint8_t root[32]);

/* Phase timing: one commit as bz_commit_device with a CUDA event after every
 * kernel; ms[i] is the device time of launch i and names + 32*i its kernel
 * name (NUL terminated).  At most cap entries; *count receives the number of
 * launches.  The commitment is freed before returning. */
int bz_commit_profile(bz_ctx *ctx, const uint64_t *d_msg, size_t n_words,
                      const bz_params *params, size_t cap, float *ms, char *names,
                      size_t *count, uint8_t root[32]);

/* ligero_commit (flock-core/src/pcs/ligerito.rs:2390-2434): the recursive
 * levels' commit -- same replicate + NTT + Merkle over `poly` of
 * 2^(log_msg_cols + log_num_interleaved) elements (device pointer). */
int bz_ligero_commit_device(bz_ctx *ctx, const uint64_t *d_poly, uint32_t log_msg_cols,
                            uint32_t log_num_interleaved, uint32_t log_inv_rate,
                            uint32_t hash_kind, bz_commitment **out, uint8_t root[32]);

/* ---- batched commit ----------------------------------------------------- */
/* count independent commits (device messages) recorded into one CUDA graph
 * and launched once; roots is count*32 bytes.  With use_graph = 0 the same
 * work is issued as plain per-polynomial launches (the comparison path). */
int bz_commit_batch_device(bz_ctx *ctx, size_t count, const uint64_t *const *d_msgs,
                           const bz_params *params, bz_commitment **outs, uint8_t *roots,
                           int use_graph);

/* Reusable batch plan: the resident buffers of count commits and, with
 * use_graph != 0, one CUDA graph holding every kernel of every commit (the
 * polynomials spread over n_branches parallel branches so small ones overlap
 * on the device).  Each launch recommits the same device messages (their
 * contents may change between launches).  The shapes' NTT schedules are the
 * context's (bz_autotune before creating the plan picks them per shape).
 * This is the batched path of the reference's many-commit callers; there is
 * no single reference function it replaces. */
typedef struct bz_batch_plan bz_batch_plan;
int bz_batch_plan_create(bz_ctx *ctx, size_t count, const uint64_t *const *d_msgs,
                         const bz_params *params, int use_graph, int n_branches,
                         bz_batch_plan **out);
/* The same resident commits run as the work items of ONE persistent kernel
 * (one 512-thread CTA per SM), launched through a CUDA graph together with the
 * reset of its scheduler state.  Every commit's NTT passes, leaf hashes and
 * tree levels are steps of items; a CTA takes an item of the first commit
 * (largest first) whose current step still has one, so small commits fill the
 * SMs while a large one finishes a step.  The context's per-shape schedules
 * (bz_autotune) pick the radix-8, radix-4 / radix-2 and deep passes; shapes
 * too small for the table passes take generic single layers.  BZ_ERR_SHAPE
 * for single-column messages and BLAKE3 leaves of more than 256 chunks
 * (2^14 lanes).  A CTA that finds no ready item for 2 s stops, and
 * bz_batch_plan_roots then returns BZ_ERR_TIMEOUT.  Launch, roots,
 * commitment and destroy are those of any plan. */
int bz_batch_plan_create_persistent(bz_ctx *ctx, size_t count, const uint64_t *const *d_msgs,
                                    const bz_params *params, bz_batch_plan **out);
/* Test hook for a persistent plan (no counterpart in the reference): one
 * launch that waits for a step the plan does not have, with a wait limit of
 * limit_ms.  The kernel runs the plan's items, gives up waiting after the
 * limit and reports it; returns BZ_ERR_TIMEOUT when it did (the plan's later
 * launches are unaffected), BZ_ERR_ARG for a plan that is not persistent. */
int bz_batch_plan_stall_check(bz_batch_plan *plan, uint32_t limit_ms);
/* Enqueue one launch of the plan on the context stream (no synchronization). */
int bz_batch_plan_launch(bz_batch_plan *plan);
/* Synchronize and copy the count roots (count * 32 bytes). */
int bz_batch_plan_roots(bz_batch_plan *plan, uint8_t *roots);
/* The i-th commitment (owned by the plan; valid until the plan is destroyed). */
bz_commitment *bz_batch_plan_commitment(bz_batch_plan *plan, size_t i);
int bz_batch_plan_destroy(bz_batch_plan *plan);

/* ---- serving: continuous-batching commit / open server ------------------- */
/* A scheduler thread admits queued commits whenever one of n_slots execution
 * slots (CUDA streams) is free and the request's device memory (message
 * staging + resident codeword + tree) fits in mem_budget_bytes (0 = the
 * context budget); later arrivals start as earlier ones finish or are opened,
 * and their kernels overlap on the device.  Codewords and trees stay resident
 * until opened.  A finished request's device buffers are kept for the next
 * request of the same size while the live requests and these spares fit in
 * the budget; bz_server_stats's in_use counts the live requests only, and
 * bz_server_destroy returns everything.  The serving counterpart of the reference's
 * commit-then-open flow (BinaryPcs::commit then open_*, src/binary_pcs.rs:
 * 313-431); the reference has no server of its own. */
typedef struct bz_server bz_server;
enum {
    BZ_REQ_QUEUED = 0,
    BZ_REQ_RUNNING = 1,
    BZ_REQ_COMMITTED = 2,
    BZ_REQ_OPEN_QUEUED = 3,
    BZ_REQ_OPENING = 4,
    BZ_REQ_OPENED = 5,
    BZ_REQ_FAILED = 6
};
int bz_server_create(bz_ctx *ctx, int n_slots, uint64_t mem_budget_bytes, size_t queue_cap,
                     bz_server **out);
/* Scheduling policy (no counterpart in the reference, which has no server).
 * admit_order: BZ_ADMIT_SMALLEST (the default) admits the smallest queued
 * commit first, unless the oldest has waited more than aging_ms (default 500),
 * which then goes first; BZ_ADMIT_FIFO admits in arrival order.  The slots'
 * streams have three priorities (a third each, the rest lowest): requests of
 * at most 2^high_priority_log_size elements (default 20; -1: no priorities)
 * and openings take the highest, medium requests of at most
 * 2^(high_priority_log_size + 3) elements the middle one, the largest the
 * lowest.  A request also takes a slot of a lower priority than its own when
 * its own are busy, never a higher one; medium and large requests' table
 * passes are cut into short CTAs, so a higher-priority request's kernels take
 * SMs within a fraction of their pass.  A commit-then-open request's opening
 * always runs right behind its commit on the same stream. */
enum { BZ_ADMIT_FIFO = 0, BZ_ADMIT_SMALLEST = 1 };
int bz_server_set_policy(bz_server *s, int admit_order, uint32_t aging_ms,
                         int high_priority_log_size);
/* host_msg must stay valid until the request reaches BZ_REQ_COMMITTED.
 * From pinned host memory, small and medium messages are read by a copy
 * kernel on the request's stream and the largest go through the copy engine
 * in 64 MiB pieces; a pageable message always takes the copy engine.
 * BZ_ERR_BUSY when the queue holds queue_cap commits. */
int bz_server_submit_commit(bz_server *s, const uint64_t *host_msg, size_t n_words,
                            const bz_params *params, uint64_t *request_id);
/* Commit-then-open as one request: the opening at the q positions runs right
 * behind the commit (same results as submit_commit followed by submit_open);
 * the completion queue reports COMMITTED and OPENED together.  BZ_ERR_ARG for
 * a position outside the codeword. */
int bz_server_submit_commit_open(bz_server *s, const uint64_t *host_msg, size_t n_words,
                                 const bz_params *params, const uint64_t *positions, size_t q,
                                 uint64_t *request_id);
/* Queue an opening of a committed request at q positions: the opened rows
 * and the multi-proof (merkle_multi_proof order); frees the resident
 * codeword and tree when done. */
int bz_server_submit_open(bz_server *s, uint64_t request_id, const uint64_t *positions,
                          size_t q);
int bz_server_poll(bz_server *s, uint64_t request_id, int *state);
/* Wait (bounded by timeout_ms) until the request reaches target_state;
 * BZ_ERR_TIMEOUT when the wait runs out. */
int bz_server_wait(bz_server *s, uint64_t request_id, int target_state, uint32_t timeout_ms);
/* Completion queue: up to cap state changes since the previous call, in
 * order, as (ids[i], states[i]) with the state entered (COMMITTED, OPENED or
 * FAILED); waits up to timeout_us microseconds while none is pending.
 * Recording starts with the first call. */
int bz_server_next_done(bz_server *s, uint64_t *ids, int *states, size_t cap, size_t *n,
                        uint32_t timeout_us);
int bz_server_root(bz_server *s, uint64_t request_id, uint8_t root[32]);
/* rows: q * 2^log_batch_size elements for the sorted unique positions;
 * proof: n_hashes * 32 bytes.  Either output may be NULL (size query). */
int bz_server_open_result(bz_server *s, uint64_t request_id, uint64_t *rows,
                          size_t rows_cap_words, uint8_t *proof, size_t proof_cap,
                          size_t *n_rows, size_t *n_hashes);
/* ns since server start: submit, start, committed, open submitted, opened */
int bz_server_times(bz_server *s, uint64_t request_id, int64_t times[5]);
int bz_server_release(bz_server *s, uint64_t request_id);
int bz_server_stats(bz_server *s, uint64_t *committed, uint64_t *opened, uint64_t *failed,
                    uint64_t *in_use, uint64_t *queued);
int bz_server_destroy(bz_server *s);

/* ---- batched grand-product GKR (BitZ src/bitz/gkr.rs) -------------------- */
/* The caller's transcript (the reference's spongefish ProverState stays on
 * the caller's side): absorb the prover message msg[0..3] (two field
 * elements, lo and hi words each) and write the next challenge; stage
 * BZ_GKR_ROUND is the reference's Stage::GkrRound, BZ_GKR_CLOSE
 * Stage::GkrClose (prover_message then native_scalar, gkr.rs:264-271).  A
 * nonzero return aborts the proof with BZ_ERR_STATE. */
enum { BZ_GKR_ROUND = 0, BZ_GKR_CLOSE = 1 };
typedef int (*bz_gkr_transcript_fn)(void *user, int stage, const uint64_t msg[4],
                                    uint64_t challenge[2]);
/* gpgkr_prove (src/bitz/gkr.rs:113-125) of
 * GrandProductCircuit::new(leaves).batched_eval(groups) (gkr.rs:80-108):
 * n_leaves a power of two (the reference pads with ones; so must the
 * caller), groups a power of two below it, point: log2(groups) field
 * elements (little-endian), the claim point on the roots.  Writes the groups
 * roots (NULL: skipped), the little-endian leaf point (log2(n_leaves)
 * elements) and the claimed leaf value.  Messages, challenges, point and
 * claim are the reference's for the same transcript.  Device memory: about
 * 1.5 x the leaves besides them.  Synchronous. */
int bz_gkr_prove(bz_ctx *ctx, const uint64_t *leaves, size_t n_leaves, size_t groups,
                 const uint64_t *point, bz_gkr_transcript_fn fn, void *user,
                 uint64_t *roots, uint64_t *out_point, uint64_t out_claim[2]);
/* Same with the leaves in device memory; they are overwritten (the rounds
 * fold the leaf layer in place, as the reference's batched_eval consumes
 * its leaves). */
int bz_gkr_prove_device(bz_ctx *ctx, uint64_t *d_leaves, size_t n_leaves, size_t groups,
                        const uint64_t *point, bz_gkr_transcript_fn fn, void *user,
                        uint64_t *roots, uint64_t *out_point, uint64_t out_claim[2]);
/* Forest::prove (src/bitz/forest.rs:246-300) from its inputs: 2^t rows of
 * 2^s columns, leaf (row, column) = images[row] where bit (column mod 64) of
 * packed[(column / 64) * 2^t + row] is set, else 1 (the leaf grid of
 * src/bitz/forest_tests.rs:42-68); zeta: s elements.  The same transcript
 * as bz_gkr_prove over those leaves with 2^s groups, which is what the
 * reference's forest matches byte for byte. */
int bz_gkr_forest_prove(bz_ctx *ctx, const uint64_t *packed, const uint64_t *images, int t,
                        int s, const uint64_t *zeta, bz_gkr_transcript_fn fn, void *user,
                        uint64_t *roots, uint64_t *out_point, uint64_t out_claim[2]);

/* ---- sumcheck folds (device buffers) ------------------------------------ */
/* fold_and_msg_lsb (flock-core/src/pcs/ligerito.rs:2634-2735), used by
 * SumcheckProver::fold (:3046-3057): nf[j] = f[2j] + (f[2j]+f[2j+1])*r (same
 * for b) and the next-round message (u0, u2) over the folded arrays. */
int bz_fold_and_msg_lsb(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                        const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb, uint64_t u0[2],
                        uint64_t u2[2]);
/* Allocation-free bz_fold_and_msg_lsb, for callers that cannot allocate
 * device memory (a host runtime that reserved the GPU's memory for its own
 * pool, or a fold loop that cannot afford cudaMalloc's synchronisation).  No
 * counterpart in the reference: it is the same fold with its per-block
 * scratch in a fixed 64 KiB device array instead of allocated memory.  The
 * caller passes device inputs/outputs and a stream (NULL = default stream) on
 * the current device; d_msg receives {u0.lo, u0.hi, u2.lo, u2.hi} on the
 * device.  Enqueue only: synchronize the stream before reading outputs.  n
 * must be a power of two in [2, 2^40] (BZ_ERR_SHAPE otherwise).  The first
 * call on each device resolves the array's device address; make it before any
 * stream capture.  That address is kept for the life of the process: a
 * cudaDeviceReset after the first call on a device is not supported.  A
 * launch error already pending on the calling thread gives BZ_ERR_CUDA before
 * anything is launched and stays pending for its owner.  Calls that overlap
 * on the GPU share the array and race.  Allocates nothing (no cudaMalloc,
 * cudaFree or allocating library call). */
int bz_fold_and_msg_lsb_static(const uint64_t *d_f, const uint64_t *d_b, size_t n,
                               const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb,
                               uint64_t *d_msg, void *stream);
/* round_msg_lsb (ligerito.rs:2500-2537). */
int bz_round_msg_lsb(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                     uint64_t u0[2], uint64_t u2[2]);
/* Check of the armed fold that the prover uses for its small rounds (no
 * counterpart in the reference).  The prover enqueues such a round before its
 * challenge exists; the kernel waits at its gate, for at most limit_ns (0 =
 * the prover's 100 ms), until the host posts r.  This call arms one
 * bz_fold_and_msg_lsb round of length n, then:
 *   mode 0: posts r and returns the round's message (as bz_fold_and_msg_lsb);
 *   mode 1: cancels it (BZ_OK, nothing written);
 *   mode 2: posts nothing, waits for the kernel to give up and returns
 *           BZ_ERR_TIMEOUT.
 * Every mode leaves the context ready for further rounds. */
int bz_fold_gate_check(bz_ctx *ctx, const uint64_t *d_f, const uint64_t *d_b, size_t n,
                       const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb, int mode,
                       uint64_t limit_ns, uint64_t u0[2], uint64_t u2[2]);
/* partial_eval_lsb (ligerito.rs:1678-1695): fold the k LSB variables by
 * rs[0..k) (host array of k elements); d_out holds n >> k elements. */
int bz_partial_eval_lsb(bz_ctx *ctx, const uint64_t *d_in, size_t n, const uint64_t *rs,
                        size_t k, uint64_t *d_out);

/* ---- ring switch (BitZ src/ligerito.rs) --------------------------------- */
/* build_eq_x_r_vec (src/poly/utils.rs:46-120) on the device: 2^k entries. */
int bz_build_eq_lsb(bz_ctx *ctx, const uint64_t *point, size_t k, uint64_t *d_out);
/* sv_fold_mfr (src/ligerito.rs:317-375): sv[j] = sum_y eq[y]*bit_j(P[y]);
 * sv is a host array of 128 elements. */
int bz_sv_fold(bz_ctx *ctx, const uint64_t *d_packed, const uint64_t *d_eq, size_t n,
               uint64_t *sv);
/* phi_byte_tables + phi_from_words (src/ligerito.rs:384-427):
 * d_out[y] = sum_{u in bits(eq_hi[y])} eq_r2[u]; eq_r2 is a host array of
 * 128 elements. */
int bz_phi_from_words(bz_ctx *ctx, const uint64_t *d_eq_hi, size_t n, const uint64_t *eq_r2,
                      uint64_t *d_out);

/* ---- Fiat-Shamir transcript (host) ----------------------------------------- */
/* BitZ's Blake3Transcript (src/transcript/mod.rs:18-96): an incremental
 * BLAKE3 hasher over everything absorbed; squeezes read its extended output
 * without consuming the state.  Host-only and cheap; not thread-safe per
 * handle. */
typedef struct bz_transcript bz_transcript;
int bz_transcript_create(bz_transcript **out);
int bz_transcript_clone(const bz_transcript *t, bz_transcript **out);
int bz_transcript_destroy(bz_transcript *t);
/* absorb_inner (mod.rs:81-95): a plain hasher update. */
int bz_transcript_absorb(bz_transcript *t, const uint8_t *data, size_t len);
/* absorb_slice (src/transcript/traits.rs:371-376): 0x06 || len u64 LE ||
 * data || 0x07.  Every ZincChallenger observation (src/ligerito_flock.rs:
 * 36-62) is one absorb_slice. */
int bz_transcript_absorb_slice(bz_transcript *t, const uint8_t *data, size_t len);
/* get_challenge of a len-byte type without padding bits (mod.rs:65-80):
 * squeeze len bytes, then absorb 0x12 || bytes || 0x34. */
int bz_transcript_challenge(bz_transcript *t, uint8_t *out, size_t len);
/* get_field_challenge::<Gf128> = ZincChallenger::sample_f128 (:64-67). */
int bz_transcript_sample_f128(bz_transcript *t, uint64_t out[2]);
/* ZincChallenger::observe_f128 (:41-46): absorb_slice of lo LE || hi LE. */
int bz_transcript_observe_f128(bz_transcript *t, const uint64_t v[2]);
/* fill_sampling_bytes (mod.rs:58-63). */
int bz_transcript_fill_sampling_bytes(bz_transcript *t, uint8_t *out, size_t len);
/* state_digest (mod.rs:40-42). */
int bz_transcript_state_digest(const bz_transcript *t, uint8_t out[32]);
/* BLAKE3 extended output of one message (the `blake3` crate's
 * finalize_xof().fill), on the host. */
int bz_blake3_xof(const uint8_t *data, size_t len, uint8_t *out, size_t out_len);

/* ---- proof of work (GPU) ---------------------------------------------------- */
/* first_pow_nonce (src/utils/blake3x4.rs:42-69; the parallel
 * smallest_pow_nonce :71-120 returns the same nonce): the smallest nonce in
 * [start, end) such that blake3(prefix || nonce u64 LE) has >= bits leading
 * zero bits (most significant bit of byte 0 first).  prefix_len + 8 <= 64;
 * bits <= 256; bits == 0 gives start.  BZ_ERR_NOTFOUND when no nonce in the
 * range passes.  Synchronous (launches on the context stream). */
int bz_pow_first_nonce(bz_ctx *ctx, const uint8_t *prefix, size_t prefix_len, uint32_t bits,
                       uint64_t start, uint64_t end, uint64_t *nonce);
/* ZincChallenger::grind_pow (src/ligerito_flock.rs:70-99): seed = one
 * sample_f128 as 16 LE bytes; nonce = 0 when bits == 0, else the smallest
 * passing nonce of blake3(seed || nonce) (searched on the GPU); then
 * absorb_slice(nonce LE). */
int bz_transcript_grind_pow(bz_ctx *ctx, bz_transcript *t, uint32_t bits, uint64_t *nonce);
/* ZincChallenger::verify_pow (:101-113), on the host; *ok = 0 or 1. */
int bz_transcript_verify_pow(bz_transcript *t, uint64_t nonce, uint32_t bits, int *ok);

/* ---- level-0 Ligerito opening ---------------------------------------------- */
/* The level-0 part of recursive_prover_with_basis_initial_impl
 * (flock-core/src/pcs/ligerito.rs:3566-3720; entered from
 * recursive_prover_with_basis, :3455-3487, by BinaryPcs::open_basis,
 * src/binary_pcs.rs:341-367) against a device-resident commitment: the
 * transcript prefix, the initial_k lane folds (with fold grinding), the
 * level-1 ligero_commit of the folded witness, the query grind, the sampled
 * queries and alpha_0, and the opened rows with their Merkle multi-proof.
 * Requires initial_k == the commitment's log_batch_size (>= 1). */
typedef struct {
    uint32_t initial_k;           /* ProverConfig::initial_k */
    uint32_t recursive_k0;        /* recursive_ks[0] */
    uint32_t log_inv_rate1;       /* log_inv_rates[1] */
    uint32_t fold_grinding_bits0; /* fold_grinding_bits[0] */
    uint32_t grinding_bits0;      /* grinding_bits[0] */
    uint32_t queries0;            /* queries[0] */
    uint32_t hash_kind;           /* merkle_hash of the level-1 commitment */
    uint32_t ood_samples1;        /* ood_samples[1]: OOD rounds after the level-1 root */
} bz_l0_config;
typedef struct {
    size_t n_sumcheck;     /* 1 + initial_k messages (u0, u2) */
    size_t n_fold_nonces;  /* rounds with fold_grinding_bits0 - j > 0 */
    size_t n_queries;
    size_t n_alpha;        /* ceil_log2(queries0) */
    size_t row_len;        /* 2^initial_k elements per opened row */
    size_t n_proof_hashes;
    size_t folded_len;     /* 2^(log_msg_len - initial_k) */
    size_t n_ood_values;   /* ood_samples1 claimed evaluations */
} bz_l0_sizes;
typedef struct bz_l0_opening bz_l0_opening;
/* d_packed / d_basis: 2^log_msg_len elements on the device (the packed
 * witness and the combined basis b_initial); the transcript is advanced in
 * place.  Both device arrays are only read. */
int bz_ligerito_open_l0(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                        const uint64_t *d_packed, const uint64_t *d_basis,
                        const uint64_t target[2], const bz_l0_config *cfg,
                        bz_l0_opening **out);
int bz_l0_opening_sizes(const bz_l0_opening *o, bz_l0_sizes *sizes);
/* Copy any subset of the results (NULL skips): sumcheck n_sumcheck x 4 words
 * {u0.lo, u0.hi, u2.lo, u2.hi}; fold challenges initial_k x 2 words; alpha
 * n_alpha x 2 words; rows n_queries x row_len x 2 words (row q = codeword
 * positions q * row_len ...); proof n_proof_hashes x 32 bytes. */
int bz_l0_opening_copy(const bz_l0_opening *o, uint64_t *sumcheck, uint64_t *fold_nonces,
                       uint64_t *challenges, uint8_t root1[32], uint64_t *grinding_nonce,
                       uint64_t *queries, uint64_t *alpha, uint64_t *rows, uint8_t *proof);
/* Move the opened rows out of the opening without a copy (the 9.7 MB of rows
 * at 2^24): *data points at n_queries x row_len x 2 words, valid until
 * bz_rows_free(*rows), independent of the opening's own lifetime.  Once
 * taken, bz_l0_opening_copy writes no rows.  The rows move out once: a
 * second take returns BZ_ERR_STATE (and a failed row fetch its own error),
 * with *rows and *data set to NULL.  No counterpart in the reference (its
 * opening returns the rows by value). */
typedef struct bz_rows bz_rows;
int bz_l0_opening_take_rows(bz_l0_opening *o, bz_rows **rows, const uint64_t **data);
int bz_rows_free(bz_rows *rows);
/* ood_samples1 x 2 words: the claimed evaluations, in transcript order. */
int bz_l0_opening_ood_values(const bz_l0_opening *o, uint64_t *values);
/* The level-1 commitment (owned by the opening). */
bz_commitment *bz_l0_opening_level1(bz_l0_opening *o);
/* The folded witness f^1 and basis (device, owned by the opening). */
int bz_l0_opening_folded(const bz_l0_opening *o, const uint64_t **d_f1, const uint64_t **d_b1,
                         size_t *n1);
int bz_l0_opening_free(bz_l0_opening *o);

/* ---- full recursive Ligerito opening ------------------------------------- */
/* recursive_prover_with_basis / _initial (flock-core/src/pcs/ligerito.rs:
 * 3455-3884) against a device-resident level-0 commitment: the level-0
 * opening above, then every recursive level -- basis induction from the
 * previous level's queries, introduce + glue, the level's folds, the next
 * ligero_commit with its OOD rounds, grind, queries and opened rows -- and
 * the final level's yr, grind and rows.  *out is the LigeritoProof
 * (bz_ligerito_proof_view_of / bz_ligerito_proof_encode read it; free it with
 * bz_ligerito_proof_free).  Array lengths follow ProverConfig
 * (ligerito.rs:124-160): recursive_ks has recursive_steps entries, the
 * others recursive_steps + 1; fold_grinding_bits / ood_samples may be NULL
 * (all zero). */
typedef struct {
    uint32_t initial_k;
    uint32_t recursive_steps;
    const uint32_t *recursive_ks;
    const uint32_t *log_inv_rates;      /* [0] must be the commitment's rate */
    const uint32_t *queries;
    const uint32_t *grinding_bits;
    const uint32_t *fold_grinding_bits;
    const uint32_t *ood_samples;        /* [0] must be 0 */
    uint32_t hash_kind;                 /* merkle_hash of the recursive commitments */
} bz_ligerito_config;
int bz_ligerito_prove(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                      const uint64_t *d_packed, const uint64_t *d_basis, const uint64_t target[2],
                      const bz_ligerito_config *cfg, bz_ligerito_proof **out);

/* ---- proof codec (host) ------------------------------------------------------ */
/* flock's LigeritoProof (flock-core/src/pcs/ligerito.rs:1509-1551) as the
 * bincode 1.3 fixed-int blob that BitZ embeds (src/binary_pcs.rs:527-544),
 * and the BitZ proof stream around it (src/proof_codec.rs:39-161,
 * binary_pcs.rs:487-557).  Rows are Vec<Vec<Gf128>>: n_rows lengths in
 * row_lens and the rows' elements concatenated in data (2 words each). */
typedef struct {
    size_t n_rows;
    const size_t *row_lens;
    const uint64_t *data;
} bz_rows_view;
/* RecursiveProof {opened_rows, merkle_proof}; FinalProof adds yr. */
typedef struct {
    bz_rows_view rows;
    size_t n_hashes;
    const uint8_t *hashes; /* n_hashes x 32 */
} bz_level_view;
typedef struct {
    uint8_t initial_root[32];
    bz_level_view initial_proof;
    size_t n_recursive_roots;
    const uint8_t *recursive_roots; /* x 32 */
    size_t n_recursive_proofs;
    const bz_level_view *recursive_proofs;
    size_t n_yr;
    const uint64_t *yr;             /* final_proof.yr, x 2 words */
    bz_level_view final_rows;       /* final_proof.opened_rows / merkle_proof */
    size_t n_sumcheck;
    const uint64_t *sumcheck;       /* {u_0.lo, u_0.hi, u_2.lo, u_2.hi} each */
    size_t n_grinding_nonces;
    const uint64_t *grinding_nonces;
    size_t n_ood_values;
    const uint64_t *ood_values;     /* x 2 words */
    size_t n_fold_grinding_nonces;
    const uint64_t *fold_grinding_nonces;
} bz_ligerito_proof_view;
/* bincode::serialize(&proof): *len receives the blob size; out may be NULL
 * (size query), else it must hold cap >= *len bytes. */
int bz_ligerito_proof_encode(const bz_ligerito_proof_view *view, uint8_t *out, size_t cap,
                             size_t *len);
/* bincode fixint decode bounded by len, trailing bytes rejected
 * (BZ_ERR_DECODE on any failure). */
int bz_ligerito_proof_decode(const uint8_t *blob, size_t len, bz_ligerito_proof **out);
/* A view whose pointers live as long as the proof (and stay valid until the
 * next view_of call on it). */
int bz_ligerito_proof_view_of(bz_ligerito_proof *p, bz_ligerito_proof_view *view);
int bz_ligerito_proof_free(bz_ligerito_proof *p);

/* Writer (proof_codec.rs:39-89): len = u64 LE, gf = lo LE || hi LE, bytes raw. */
typedef struct bz_writer bz_writer;
int bz_writer_create(bz_writer **out);
int bz_writer_destroy(bz_writer *w);
int bz_writer_len(bz_writer *w, uint64_t n);
int bz_writer_gf(bz_writer *w, const uint64_t g[2]);
int bz_writer_bytes(bz_writer *w, const uint8_t *data, size_t len);
/* The accumulated bytes (valid until the next write or destroy). */
int bz_writer_data(const bz_writer *w, const uint8_t **data, size_t *len);
/* write_round0 (binary_pcs.rs:487-496): gf(y) || len(0) | len(1) || len(nonce). */
int bz_write_round0(bz_writer *w, const uint64_t y[2], int has_nonce, uint64_t nonce);
/* write_ring_switch (:510-519): the 128 partial evaluations s_v. */
int bz_write_ring_switch(bz_writer *w, const uint64_t s_v[256]);
/* write_ligerito (:527-531): len(blob) || blob. */
int bz_write_ligerito(bz_writer *w, const bz_ligerito_proof_view *view);
/* Reader (proof_codec.rs:91-161) over a caller buffer that must outlive it;
 * BZ_ERR_TRUNCATED when a field runs past the end. */
typedef struct bz_reader bz_reader;
int bz_reader_create(const uint8_t *buf, size_t len, bz_reader **out);
int bz_reader_destroy(bz_reader *r);
size_t bz_reader_remaining(const bz_reader *r);
int bz_reader_len(bz_reader *r, uint64_t *n);
int bz_reader_gf(bz_reader *r, uint64_t g[2]);
int bz_reader_take(bz_reader *r, size_t n, const uint8_t **data);
/* read_round0 (:498-508): BZ_ERR_NONCANONICAL for a presence tag > 1. */
int bz_read_round0(bz_reader *r, uint64_t y[2], int *has_nonce, uint64_t *nonce);
int bz_read_ring_switch(bz_reader *r, uint64_t s_v[256]);
/* read_ligerito (:533-544): BZ_ERR_TRUNCATED when the length exceeds
 * 64 MiB or the bytes left; BZ_ERR_DECODE when the blob does not decode. */
int bz_read_ligerito(bz_reader *r, bz_ligerito_proof **out);

/* ---- BitZ BinaryPcs opening ------------------------------------------------ */
/* Round 0, the out-of-domain sample bound right after the commitment
 * (BinaryPcs::prove_round0, src/binary_pcs.rs:320-325;
 * prove_ood_round_packed, src/ligerito_flock.rs:1520-1557): header frame,
 * grinding when grinding_bits > 0, zeta, y = MLE[packed](zeta, zeta^2, ...)
 * on the device, y absorbed.  d_packed holds n = 2^vars elements. */
typedef struct bz_round0 bz_round0;
int bz_pcs_prove_round0(bz_ctx *ctx, bz_transcript *transcript, const uint64_t *d_packed,
                        size_t n, uint32_t grinding_bits, bz_round0 **out);
/* OodRound {y, nonce}: has_nonce = 1 iff grinding_bits > 0; vars = log2 n. */
int bz_round0_get(const bz_round0 *r, uint64_t y[2], int *has_nonce, uint64_t *nonce,
                  uint32_t *vars);
/* The point (zeta^(2^i)), vars x 2 words. */
int bz_round0_point(const bz_round0 *r, uint64_t *point);
int bz_round0_free(bz_round0 *r);
/* ring_switch_prove (src/ligerito.rs:445-496): r_hi has log2 n coordinates;
 * s_v receives the 128 partial evaluations (absorbed), d_basis (n elements,
 * device) the weight table B(y), target beta0. */
int bz_pcs_ring_switch(bz_ctx *ctx, bz_transcript *transcript, const uint64_t *d_packed, size_t n,
                       const uint64_t *r_hi, uint64_t s_v[256], uint64_t *d_basis,
                       uint64_t target[2]);
/* BinaryPcs::open_basis (src/binary_pcs.rs:341-367): eta, d_basis +=
 * eta * eq(round-0 point) in place, target + eta * y, then bz_ligerito_prove. */
int bz_pcs_open_basis(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                      const uint64_t *d_packed, const bz_round0 *round0, uint64_t *d_basis,
                      const uint64_t target[2], const bz_ligerito_config *cfg,
                      bz_ligerito_proof **out);
/* BinaryPcs::open_bit_mle (src/binary_pcs.rs:413-431): point has
 * point_len = log_msg_len + 7 coordinates (the low 7 select the bit of a
 * word); ring switch on point[7..], then open_basis.  The BitMleOpening is
 * (s_v, *out). */
int bz_pcs_open_bit_mle(bz_ctx *ctx, bz_transcript *transcript, bz_commitment *c0,
                        const uint64_t *d_packed, const bz_round0 *round0, const uint64_t *point,
                        size_t point_len, const bz_ligerito_config *cfg, uint64_t s_v[256],
                        bz_ligerito_proof **out);

/* ---- bit-matrix ingest ------------------------------------------------------ */
/* A 2^row_vars x 2^col_vars bit matrix (IntegerMatrixLayout, src/pcs.rs:14-41;
 * cell (b, c) at flat index (b << col_vars) | c).  "rows": per column c its
 * bits packed 64 per word, W = ceil(2^row_vars / 64) words per column;
 * "packed columns": ceil(2^col_vars / 64) groups of 2^row_vars words, bit k
 * of word i of group g = column 64g + k's bit i.  All buffers on the device. */
/* repack_leaf_bits (src/ligerito.rs:19-33): d_cells holds one u128 (2 words)
 * per cell, each 0 or 1 (BZ_ERR_ARG otherwise, as the reference asserts). */
int bz_repack_leaf_bits(bz_ctx *ctx, const uint64_t *d_cells, uint32_t row_vars,
                        uint32_t col_vars, uint64_t *d_rows);
/* pack_columns_from_rows / rows_from_packed_cols (src/ligerito.rs:655-717):
 * 64 x 64 bit transposes. */
int bz_pack_columns_from_rows(bz_ctx *ctx, const uint64_t *d_rows, uint32_t row_vars,
                              uint32_t col_vars, uint64_t *d_packed_cols);
int bz_rows_from_packed_cols(bz_ctx *ctx, const uint64_t *d_packed_cols, uint32_t row_vars,
                             uint32_t col_vars, uint64_t *d_rows);
/* commit_rs_flock_from_rows (src/ligerito_flock.rs:198-245): the packed
 * message is the rows buffer read as {lo, hi} pairs (2^(row_vars - 7 +
 * col_vars) elements); requires row_vars >= 7 and log_batch < that count's
 * log. */
int bz_commit_rows(bz_ctx *ctx, const uint64_t *d_rows, uint32_t row_vars, uint32_t col_vars,
                   uint32_t log_inv_rate, uint32_t log_batch, uint32_t hash_kind,
                   bz_commitment **out, uint8_t root[32]);

/* ---- synthetic inputs --------------------------------------------------- */
/* RFC 8439 ChaCha20 keystream words (key = seed LE u64 zero padded, nonce 0,
 * counter from 0), word i = keystream bytes [16 i, 16 i + 16). */
int bz_chacha_fill_device(bz_ctx *ctx, uint64_t seed, uint64_t first_word, uint64_t *d_out,
                          size_t n_words);
int bz_chacha_fill_host(uint64_t seed, uint64_t first_word, uint64_t *out, size_t n_words,
                        int n_threads);

/* ---- schedule autotuner ---------------------------------------------------- */
/* Times the candidate NTT schedules for this shape and keeps the fastest for
 * later commits of the same shape on this context. */
int bz_autotune(bz_ctx *ctx, const bz_params *params, int reps, uint32_t *chosen);
int bz_schedule_get(bz_ctx *ctx, const bz_params *params, uint32_t *schedule);
int bz_schedule_set(bz_ctx *ctx, const bz_params *params, uint32_t schedule);

#ifdef __cplusplus
}
#endif
#endif /* BITZ_GPU_H */
