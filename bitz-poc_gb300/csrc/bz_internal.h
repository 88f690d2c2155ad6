// Internal interfaces between the CUDA translation units and the host
// runtime (context, commit pipeline, batching, serving).  Not part of the ABI.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace bz {

// ---- shape of one commit (flock-core/src/pcs/commit.rs:53-92) -------------
struct Shape {
    int log_msg_len = 0;    // m - 7
    int log_inv_rate = 0;   // r
    int log_lanes = 0;      // log_batch_size (a)
    int hash_kind = 1;      // 0 sha256, 1 blake3
    // BLAKE3 chunk counter of lane 0's chunk inside its leaf: 0 for a whole
    // commit; rank * (lanes / 64) for one rank's lanes of a lane-sharded
    // commit, whose "leaves" are then the CVs of its aligned run of chunks
    uint64_t chunk0 = 0;
    int log_dim() const { return log_msg_len - log_lanes; }        // b
    int k_code() const { return log_dim() + log_inv_rate; }        // ell
    size_t msg_words() const { return (size_t)1 << log_msg_len; }
    size_t cw_words() const { return (size_t)1 << (log_msg_len + log_inv_rate); }
    size_t n_leaves() const { return (size_t)1 << k_code(); }
    size_t leaf_bytes() const { return (size_t)16 << log_lanes; }
    size_t tree_nodes() const { return 2 * n_leaves() - 1; }
};

// Optional per-launch event marks (phase timing for the benchmark).
struct LaunchLog {
    cudaStream_t st = nullptr;
    std::vector<std::string> names;
    std::vector<cudaEvent_t> events;
    void mark(const char *name) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        names.emplace_back(name);
        events.push_back(e);
    }
    ~LaunchLog() {
        for (auto e : events) cudaEventDestroy(e);
    }
};

// ---- NTT schedule ----------------------------------------------------------
// Packed as: bits 0..3 = number of deep (shift-and-XOR) layers D (0..4),
// bit 4 = use radix-2 passes only for the table layers, bit 5 = force the
// generic one-layer-per-launch kernels (reference / fallback path), bit 6 =
// fuse the last table layers with the deep layers into one tail pass, bits
// 7..8 = narrow-multiply variant (0 shifts, 1 wide multiplies, 2 alternate),
// bit 14 = radix-4 passes with narrow (<= 25-bit) twiddles use compact tables.
enum : uint32_t {
    SCHED_DEEP_MASK = 0xF,
    SCHED_RADIX2 = 0x10,
    SCHED_GENERIC = 0x20,
    SCHED_FUSED_TAIL = 0x40,
    SCHED_MODE_SHIFT = 7,
    SCHED_SMALL_CTA = 0x200,      // 256-thread table passes (room for co-resident CTAs)
    SCHED_PIPE_SHIFT = 10,        // bits 10..11: log2 of the pipeline chunk count
    SCHED_PREFETCH = 0x1000,      // radix-4 table passes double-buffer their loads
    SCHED_LEAN = 0x2000,          // cap table-pass registers (room for co-resident CTAs)
    SCHED_NARROW = 0x4000,        // compact 32-bit tables for the deepest layers' twiddles
    SCHED_RADIX8 = 0x8000,        // radix-8 passes (eight 32 KB byte tables per twiddle)
    SCHED_R8_HEAD = 0x10000,      // with SCHED_RADIX8: the 1-2 leftover layers run first
    SCHED_SHORT_CTAS = 0x200000,  // table passes in 16 CTAs per SM instead of one long one
};
uint32_t default_schedule(const Shape &s);

// Twiddle heap for AdditiveNttF128::standard(ell): tw[(1 << l) + b] =
// twiddle(l, b) for 0 <= l < ell, 0 <= b < 2^l (entry 0 unused).
std::vector<uint64_t> twiddle_heap(int ell);

// Enqueue the forward interleaved NTT from layer r with the replicate fill
// fused (reads d_msg, writes d_cw).  Returns the number of kernels launched.
int launch_ntt(const Shape &s, uint32_t schedule, const uint4 *d_msg, uint4 *d_cw,
               const uint4 *d_tw, cudaStream_t st, int num_sms, LaunchLog *log = nullptr);

// Range-restricted NTT passes over positions [p0, p1) (aligned to the pass's
// blocks), used by the pipelined commit.
int launch_table_pass(const Shape &s, int layer, int layers, const uint4 *src, int src_bits,
                      uint4 *dst, const uint4 *tw, uint64_t p0, uint64_t p1, int threads,
                      cudaStream_t st, int num_sms, uint32_t schedule);
// Bit length of the widest twiddle of `layer` in the ell-layer transform.
int twiddle_bits(int ell, int layer);
// Shapes whose whole transform runs in one ntt_small_kernel launch.
bool small_ntt_ok(const Shape &s);
int launch_deep_range(const Shape &s, int deep, int mode, const uint4 *src, int src_bits,
                      uint4 *dst, const uint4 *tw, uint64_t p0, uint64_t p1, cudaStream_t st,
                      int num_sms);
// Leaf hashes of positions [p0, p1) (BLAKE3 leaves of <= 256 chunks, SHA-256)
// and the parent levels above all leaves.
bool leaves_range_supported(const Shape &s);
int launch_leaves_range(const Shape &s, const uint4 *d_cw, uint8_t *d_tree, uint64_t p0,
                        uint64_t p1, cudaStream_t st, int num_sms);
int launch_merkle_levels(const Shape &s, uint8_t *d_tree, cudaStream_t st, LaunchLog *log);
// Two-stream software pipeline of one commit: after the first table pass,
// position chunks go through the remaining table passes on `st` while the
// previous chunk's deep layers and leaf hashes run on `aux` (the two kinds of
// kernels bind different units and share SMs).  `ev` holds >= chunks + 2
// events.  Returns kernels launched, or -1 when the shape/schedule does not
// pipeline (the caller then uses launch_ntt + launch_merkle).
int launch_commit_pipelined(const Shape &s, uint32_t schedule, const uint4 *d_msg, uint4 *d_cw,
                            uint8_t *d_tree, const uint4 *d_tw, cudaStream_t st,
                            cudaStream_t aux, cudaEvent_t *ev, int num_sms, LaunchLog *log);

// Leaf CVs of a lane-sharded BLAKE3 commit: leaf p = the merge of the world
// ranks' subtree CVs cvs[rank * n_leaves + p] (world a power of two), written
// to tree[0 .. n_leaves).
int launch_combine_shard_cvs(const uint8_t *d_cvs, uint32_t world, uint64_t n_leaves,
                             uint8_t *d_tree, cudaStream_t st);
// Merkle tree over the codeword rows (leaves = positions).  d_scratch must hold
// merkle_scratch_bytes(s).  Returns kernels launched.
size_t merkle_scratch_bytes(const Shape &s);
int launch_merkle(const Shape &s, const uint4 *d_cw, uint8_t *d_tree, uint8_t *d_scratch,
                  cudaStream_t st, int num_sms, LaunchLog *log = nullptr);

// Gathers: rows of the codeword and arbitrary tree nodes.
int launch_gather_rows(const uint4 *d_cw, int log_lanes, const uint64_t *d_pos, size_t q,
                       uint4 *d_out, cudaStream_t st);
int launch_gather_nodes(const uint8_t *d_tree, const uint64_t *d_idx, size_t n, uint8_t *d_out,
                        cudaStream_t st);

// Folds.  d_partials holds fold_partials_bytes(n) bytes.  With `post`, the
// last CTA of the fold (or message) kernel reduces the partials itself and
// posts {u0, u2} to mapped host memory, then the sequence number (no finish
// kernel, no copy); without it a finish kernel writes d_msg_out.
struct MsgPost {
    unsigned int *ticket;  // device counter, 0 between launches
    uint64_t *words;       // device view of mapped host memory (4 words)
    uint32_t *seq;         // device view of mapped host memory
    uint32_t seq_val;
};
// Challenge gate of a fold launched ahead of its challenge: the host writes r
// to mapped memory, then the sequence number to `go` (or seq | kGateCancel to
// cancel).  The kernel waits at most limit_ns, then sets bit 0 of *err.  The
// host posts r within microseconds; the limit only bounds a gate that nothing
// opens (an error path, or a tool that runs each launch to completion before
// returning), and the prover then runs the round again unarmed.
constexpr uint32_t kGateCancel = 0x80000000u;
constexpr uint64_t kGateLimitNs = 100000000ull;  // 100 ms
struct RGate {
    const uint32_t *go = nullptr;  // device view of mapped host memory
    const uint64_t *r = nullptr;   // device view of mapped host memory: r.lo, r.hi
    uint32_t seq = 0;              // 1 .. kGateCancel - 1
    uint32_t *err = nullptr;       // device memory
    uint64_t limit_ns = kGateLimitNs;
};
size_t fold_partials_bytes(size_t n);
int fold_grid(size_t n, int num_sms);
int launch_fold_and_msg(const uint4 *d_f, const uint4 *d_b, size_t n, uint4 r, uint4 *d_nf,
                        uint4 *d_nb, uint64_t *d_partials, uint64_t *d_msg_out, cudaStream_t st,
                        int num_sms, const MsgPost *post = nullptr,
                        const RGate *gate = nullptr);
int launch_round_msg(const uint4 *d_f, const uint4 *d_b, size_t n, uint64_t *d_partials,
                     uint64_t *d_msg_out, cudaStream_t st, int num_sms,
                     const MsgPost *post = nullptr);
int launch_partial_eval_round(const uint4 *d_in, size_t n, uint4 r, uint4 *d_out,
                              cudaStream_t st);
int launch_build_eq(const uint4 *d_point_dev, size_t k, uint4 *d_out, cudaStream_t st,
                    int num_sms);
int launch_sv_fold(const uint4 *d_packed, const uint4 *d_eq, size_t n, uint64_t *d_partials,
                   uint4 *d_sv, cudaStream_t st, int num_sms);
size_t sv_partials_bytes(size_t n, int num_sms);
int launch_phi(const uint4 *d_eq_hi, size_t n, const uint4 *d_eq_r2, uint4 *d_out,
               cudaStream_t st, int num_sms);

int launch_chacha(uint64_t seed, uint64_t first_word, uint4 *d_out, size_t n_words,
                  cudaStream_t st);

// Batched grand-product GKR (BitZ src/bitz/gkr.rs; fold.cu): one product
// layer (out[i] = in[i] * in[half + i]), one dense round over h slots of the
// two half tables (with the previous round's fold by rho first when `fold`;
// the reduced (sum_end, sum_inf) land in d_out[0..3]; d_w_next, when not
// null, gets the next round's weights), and the forest's leaf grid.
// d_partials holds fold_partials_bytes(0) bytes.  With `post` the round's
// last CTA posts the sums to the mapped mailbox (as the sumcheck rounds do)
// and d_out is unused.
int launch_gkr_product(const uint4 *d_in, size_t half, uint4 *d_out, cudaStream_t st,
                       int num_sms);
int launch_gkr_round(uint4 *d_l, uint4 *d_r, const uint4 *d_w, size_t h, bool fold, uint4 rho,
                     bool send_one, uint4 *d_w_next, uint64_t *d_partials, uint64_t *d_out,
                     cudaStream_t st, int num_sms, const MsgPost *post = nullptr);
int launch_gkr_forest_leaves(const uint64_t *d_packed, const uint4 *d_images, int t, int s,
                             uint4 *d_out, cudaStream_t st, int num_sms);

// Recursive Ligerito prover (ligerito.cu).  Induce: zero the 2^log_d domain,
// scatter the nq query weights d_w at d_pos, apply the transposed forward NTT
// with the twiddle heap of log_d; the low 2^log_msg_cols outputs are the
// induced basis.
int launch_induce_basis(uint4 *d_domain, int log_d, const uint64_t *d_pos, const uint4 *d_w,
                        int nq, const uint4 *d_tw, cudaStream_t st);
// d_b[j] += beta * d_nb[j]
int launch_glue(uint4 *d_b, const uint4 *d_nb, size_t n, uint4 beta, cudaStream_t st);
// d_out[0] = sum_j d_f[j] * d_b[j]; d_partial holds dot_partials_count(n) elements.
size_t dot_partials_count(size_t n, int num_sms);
int launch_dot(const uint4 *d_f, const uint4 *d_b, size_t n, uint4 *d_partial, uint4 *d_out,
               cudaStream_t st, int num_sms);
// d_out[0] = sum_h head[h] * sum_j p[h 2^lo + j] * tail[j] over n_blocks blocks;
// d_partial holds split_dot_partials(n_blocks) elements.
size_t split_dot_partials(size_t n_blocks, int num_sms);
int launch_split_dot(const uint4 *d_p, const uint4 *d_tail, int lo, const uint4 *d_head,
                     size_t n_blocks, uint4 *d_partial, uint4 *d_out, cudaStream_t st,
                     int num_sms);
// d_b[i] += eta * head[i >> lo] * tail[i mod 2^lo]
int launch_eq_axpy(uint4 *d_b, const uint4 *d_tail, int lo, const uint4 *d_head, uint4 eta,
                   size_t n, cudaStream_t st);

// Bit-matrix ingest (ingest.cu).
int launch_repack_leaf_bits(const uint4 *d_cells, int row_vars, int col_vars, uint64_t *d_rows,
                            unsigned int *d_bad, cudaStream_t st);
int launch_pack_columns(const uint64_t *d_rows, int row_vars, int col_vars, uint64_t *d_packed,
                        cudaStream_t st);
int launch_unpack_columns(const uint64_t *d_packed, int row_vars, int col_vars, uint64_t *d_rows,
                          cudaStream_t st);

// One-time kernel attributes (large dynamic shared memory), called when a
// context is created so no attribute call happens during graph capture.
void init_ntt_kernels();
void init_fold_kernels();

// Host GF(2^128) (twiddle tables, host-side checks of transcript values).
void hgf_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]);
void hgf_inv(const uint64_t a[2], uint64_t out[2]);

}  // namespace bz
