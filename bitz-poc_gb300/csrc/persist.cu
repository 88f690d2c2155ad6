// Persistent batch commit: every commit of a batch plan runs as the work items
// of ONE kernel launch.
//
// A commit is a chain of steps (its NTT passes, its leaf hashes, its tree
// levels).  A step is a set of independent items: ranges of task chunks
// (table and radix-8 passes), of tasks (deep and generic layers, short
// leaves), of 512-chunk groups (BLAKE3 leaves) or of 512-node groups (tree
// levels).  A step may start only when the previous step of its commit is
// done.  One 512-thread CTA per SM loops: its first warp looks for a commit
// whose current step still has an unclaimed item (commits in decreasing size,
// so the largest commit's chain goes first and the smaller ones fill the SMs
// while it waits on its last items), claims the item with an atomic ticket,
// and the CTA runs it through the same device bodies as the standalone
// kernels (ntt_kernels.cuh, merkle_kernels.cuh).  The CTA that finishes a
// step's last item advances its commit.
//
// Items never wait on one another: a CTA only starts an item whose step is
// open, so every claimed item finishes and no CTA can hold up one that has
// work.  A CTA that finds nothing ready sleeps between looks and gives up
// after kPersistWaitNs without progress, setting an error word the host reads
// with the roots (BZ_ERR_TIMEOUT).
//
// Memory ordering: a finished item's writes are published by a fence before
// its ticket on the step's done counter; the step's last finisher fences
// again before it advances the commit; a CTA that sees the advanced step
// fences before the barrier that releases the item to its threads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "merkle_kernels.cuh"
#include "ntt_kernels.cuh"
#include "runtime.h"

namespace bz {
namespace {

constexpr uint64_t kPersistWaitNs = 2000000000ull;  // 2 s without a ready item

enum PKind : int32_t {
    PK_PASS8 = 0,   // pass8_body<W0, W1, W2>, variant W0*100 + W1*10 + W2; units = chunks
    PK_PF,          // table_pass2_pf_body<WO, WAB>, variant WO*10 + WAB; units = chunks
    PK_TP,          // table_pass_body<LAYERS>, variant LAYERS; units = chunks
    PK_DEEP,        // deep_pass_body<D, 0>, variant D; units = tasks
    PK_GENERIC,     // generic_layer_body; units = tasks
    PK_B3_CHUNKED,  // b3_leaves_chunked_body; units = groups of 512 chunks
    PK_B3_SMALL,    // b3_leaves_small_body; units = leaves
    PK_SHA,         // sha_leaves_body; units = leaves
    PK_LEVELS,      // merkle_levels_body; units = groups of 512 input nodes
};

struct PStep {
    int32_t kind = 0;
    int32_t variant = 0;
    uint32_t commit = 0;   // slot in the commit table
    uint32_t n_items = 1;
    uint64_t units = 0;
    TablePassArgs tp{};    // PASS8, PF, TP
    DeepArgs dp{};         // DEEP; GENERIC (with `layer`)
    int32_t layer = 0;
    int32_t log_lanes = 0;  // B3_SMALL, SHA
    int32_t log_c = 0;      // B3_CHUNKED
    const uint4 *cw = nullptr;
    uint32_t *leaves = nullptr;
    uint64_t count = 0;     // chunks (B3_CHUNKED)
    uint64_t chunk0 = 0;
    LevelsArgs lv{};
    const uint32_t *root_src = nullptr;  // last step of a commit: its root node
    uint32_t *root_dst = nullptr;
};

struct PCommit {
    uint32_t first, n_steps;
};

struct PersistArgs {
    const PStep *steps;
    const PCommit *commits;
    uint32_t n_commits;
    uint32_t total_steps;
    uint32_t *cur;         // per commit: index of its current step
    uint32_t *claim;       // per step: items handed out
    uint32_t *done;        // per step: items finished
    uint32_t *steps_done;  // steps finished, all commits
    uint32_t *err;         // bit 0: a CTA gave up waiting
    uint64_t limit_ns;
};

// Dynamic shared memory of the kernel: the largest body's tables plus its
// twiddle window and window words (the radix-8 pass).
constexpr size_t kPersistSmem = kPass8Smem + kTw8Window * 7 * 16 + 16;
static_assert(kPersistSmem >= table_smem(2) + kTwWindow * 3 * 16 + 16 + 16, "table pass scratch");
static_assert(kPersistSmem >= pf_smem(4, 4) + kTwWindow * 3 * 16 + 16, "prefetch pass scratch");
static_assert(kPersistSmem >= 512 * 9 * 4, "leaf CVs");

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
    return *reinterpret_cast<const volatile uint32_t *>(p);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Warp 0: claim an item of the first commit (in table order) whose current
// step has one left.  Returns false when none is claimable right now.
__device__ bool claim_item(const PersistArgs &p, int &g_out, uint32_t &idx_out) {
    const int lane = threadIdx.x & 31;
    for (uint32_t base = 0; base < p.n_commits; base += 32) {
        const uint32_t c = base + lane;
        int cand = -1;
        if (c < p.n_commits) {
            const PCommit cm = p.commits[c];
            const uint32_t s = ld_volatile(p.cur + c);
            if (s < cm.n_steps) {
                const uint32_t g = cm.first + s;
                if (ld_volatile(p.claim + g) < p.steps[g].n_items) cand = (int)g;
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, cand >= 0);
        while (m) {
            const int leader = __ffs(m) - 1;
            m &= m - 1;
            const int g = __shfl_sync(0xffffffffu, cand, leader);
            uint32_t got = 0;
            if (lane == leader) got = atomicAdd(p.claim + g, 1u);
            got = __shfl_sync(0xffffffffu, got, leader);
            if (got < p.steps[g].n_items) {
                g_out = g;
                idx_out = got;
                return true;
            }
        }
    }
    return false;
}

// Each item kind runs in a function of its own (not inlined), so every body
// gets the registers it has as a standalone kernel instead of sharing one
// allocation across all of them.  The functions address the dynamic shared
// memory through this array, not through a pointer argument, so the compiler
// keeps the tables' addresses as 32-bit shared-window offsets.
extern __shared__ uint4 persist_smem[];
template <int A, int B, int C>
__device__ __noinline__ void pass8_item(const PStep *st, uint64_t b, uint64_t e) {
    char *base = reinterpret_cast<char *>(persist_smem);
    const TablePassArgs a = st->tp;
    uint4 *twb = reinterpret_cast<uint4 *>(base + kPass8Smem);
    uint64_t *win = reinterpret_cast<uint64_t *>(twb + kTw8Window * 7);
    pass8_body<A, B, C>(a, b, e, base, twb, win);
}

template <int O, int AB>
__device__ __noinline__ void pf_item(const PStep *st, uint64_t b, uint64_t e) {
    char *base = reinterpret_cast<char *>(persist_smem);
    const TablePassArgs a = st->tp;
    uint4 *twb = reinterpret_cast<uint4 *>(base + pf_smem(O, AB));
    uint64_t *win = reinterpret_cast<uint64_t *>(twb + kTwWindow * 3);
    table_pass2_pf_body<O, AB>(a, b, e, reinterpret_cast<uint4 *>(base), twb, win);
}

template <int LAYERS>
__device__ __noinline__ void tp_item(const PStep *st, uint64_t b, uint64_t e) {
    char *base = reinterpret_cast<char *>(persist_smem);
    const TablePassArgs a = st->tp;
    uint4 *twb = reinterpret_cast<uint4 *>(base + table_smem(LAYERS));
    uint64_t *win = reinterpret_cast<uint64_t *>(twb + kTwWindow * (LAYERS == 2 ? 3 : 1));
    int *tz = reinterpret_cast<int *>(win + 2);
    table_pass_body<LAYERS>(a, b, e, reinterpret_cast<uint4 *>(base), twb, win, tz);
}

template <int D>
__device__ __noinline__ void deep_item(const PStep *st, uint64_t b, uint64_t e) {
    const DeepArgs a = st->dp;
    deep_pass_body<D, 0>(a, b + threadIdx.x, e, blockDim.x);
}

__device__ __noinline__ void generic_item(const PStep *st, uint64_t b, uint64_t e) {
    const DeepArgs a = st->dp;
    generic_layer_body(a.src, a.dst, a.tw, a.ell, st->layer, a.log_lanes, a.src_pos_bits,
                       b + threadIdx.x, e, blockDim.x);
}

__device__ __noinline__ void leaves_item(const PStep *st, uint64_t b, uint64_t e) {
    char *base = reinterpret_cast<char *>(persist_smem);
    const uint4 *cw = st->cw;
    uint32_t *leaves = st->leaves;
    if (st->kind == PK_B3_CHUNKED) {
        const uint64_t count = st->count, chunk0 = st->chunk0;
        const int log_c = st->log_c;
        uint32_t(*cvs)[9] = reinterpret_cast<uint32_t(*)[9]>(base);
        for (uint64_t u = b; u < e; ++u) {
            b3_leaves_chunked_body(cw, count, leaves, log_c, chunk0, u * blockDim.x, cvs);
            __syncthreads();  // the next group overwrites cvs
        }
    } else if (st->kind == PK_B3_SMALL) {
        b3_leaves_small_body(cw, st->log_lanes, e, leaves, b + threadIdx.x, blockDim.x);
    } else {
        sha_leaves_body(cw, st->log_lanes, e, leaves, b + threadIdx.x, blockDim.x);
    }
}

__device__ __noinline__ void levels_item(const PStep *st, uint64_t b, uint64_t e) {
    char *base = reinterpret_cast<char *>(persist_smem);
    const LevelsArgs a = st->lv;
    uint32_t(*nodes)[9] = reinterpret_cast<uint32_t(*)[9]>(base);
    for (uint64_t u = b; u < e; ++u) {
        merkle_levels_body(a, u, nodes);
        __syncthreads();
    }
}

__device__ __forceinline__ void run_item(const PStep *st, uint32_t idx) {
    const uint64_t units = st->units, n = st->n_items;
    const uint64_t b = units * idx / n, e = units * (idx + 1) / n;
    const int v = st->variant;
    switch (st->kind) {
        case PK_PASS8:
            switch (v) {
#define BZ_P8(A, B, C) \
    case A * 100 + B * 10 + C: pass8_item<A, B, C>(st, b, e); break;
                BZ_P8(4, 4, 4) BZ_P8(4, 4, 2) BZ_P8(4, 4, 1) BZ_P8(4, 2, 2) BZ_P8(4, 2, 1)
                BZ_P8(4, 1, 1) BZ_P8(2, 2, 2) BZ_P8(2, 2, 1) BZ_P8(2, 1, 1) BZ_P8(1, 1, 1)
#undef BZ_P8
                default: break;
            }
            break;
        case PK_PF:
            switch (v) {
#define BZ_PF(O, AB) \
    case O * 10 + AB: pf_item<O, AB>(st, b, e); break;
                BZ_PF(4, 4) BZ_PF(4, 2) BZ_PF(4, 1) BZ_PF(2, 2) BZ_PF(2, 1) BZ_PF(1, 1)
#undef BZ_PF
                default: break;
            }
            break;
        case PK_TP:
            if (v == 2) tp_item<2>(st, b, e);
            else tp_item<1>(st, b, e);
            break;
        case PK_DEEP:
            if (v == 1) deep_item<1>(st, b, e);
            else if (v == 2) deep_item<2>(st, b, e);
            else if (v == 3) deep_item<3>(st, b, e);
            else deep_item<4>(st, b, e);
            break;
        case PK_GENERIC: generic_item(st, b, e); break;
        case PK_B3_CHUNKED:
        case PK_B3_SMALL:
        case PK_SHA: leaves_item(st, b, e); break;
        case PK_LEVELS: levels_item(st, b, e); break;
        default: break;
    }
}

// Thread 0, after the CTA's barrier behind the item: count it; the step's
// last item copies the commit's root when it is the last step and advances
// the commit.
__device__ void finish_item(const PersistArgs &p, int g) {
    const PStep &st = p.steps[g];
    __threadfence();  // the CTA's writes (ordered before by the barrier)
    const uint32_t prev = atomicAdd(p.done + g, 1u);
    if (prev + 1 != st.n_items) return;
    __threadfence();  // every item of the step is visible from here
    if (st.root_dst) {
#pragma unroll
        for (int i = 0; i < 8; ++i) st.root_dst[i] = __ldcg(st.root_src + i);
        __threadfence();
    }
    atomicAdd(p.cur + st.commit, 1u);
    atomicAdd(p.steps_done, 1u);
}

__global__ void __launch_bounds__(512, 1) persistent_batch_kernel(PersistArgs p) {
    __shared__ int s_g;
    __shared__ uint32_t s_idx;
    for (;;) {
        if (threadIdx.x < 32) {
            int g = -1;
            uint32_t idx = 0;
            uint64_t t0 = 0;
            for (;;) {
                if (claim_item(p, g, idx)) break;
                g = -1;
                // nothing claimable: all done, failed, or waiting on running items
                if (ld_volatile(p.steps_done) >= p.total_steps || ld_volatile(p.err)) break;
                const uint64_t now = global_ns();
                if (t0 == 0) {
                    t0 = now;
                } else if (now - t0 > p.limit_ns) {
                    if (threadIdx.x == 0) atomicOr(p.err, 1u);
                    break;
                }
                __nanosleep(256);
            }
            if (threadIdx.x == 0) {
                s_g = g;
                s_idx = idx;
            }
            __threadfence();  // the open step's inputs before the barrier below
        }
        __syncthreads();
        const int g = s_g;
        const uint32_t idx = s_idx;
        if (g < 0) return;
        run_item(p.steps + g, idx);
        __syncthreads();
        if (threadIdx.x == 0) finish_item(p, g);
    }
}

// ---- host: the steps of one commit -----------------------------------------
struct StepBuilder {
    const Shape &s;
    uint32_t slot;
    int num_sms;
    std::vector<PStep> &out;

    // Items per step: a table pass's chunks in one item per SM at most (as
    // the standalone kernel's CTAs; twice as many items measured 3 % slower
    // on a 64-commit batch), other steps in up to four per SM; every item
    // large enough to amortise its table builds and claim.
    uint32_t items(uint64_t units, uint64_t min_units, uint64_t cap) const {
        const uint64_t n = std::max<uint64_t>(1, units / std::max<uint64_t>(1, min_units));
        return (uint32_t)std::min<uint64_t>({n, cap, units ? units : 1});
    }
    PStep base(int kind, int variant, uint64_t units, uint32_t n_items) const {
        PStep st;
        st.kind = kind;
        st.variant = variant;
        st.commit = slot;
        st.units = units;
        st.n_items = n_items;
        return st;
    }
    void table_step(int kind, int variant, const TablePassArgs &a) {
        const uint64_t chunks = a.n_tasks / 512;
        PStep st = base(kind, variant, chunks, items(chunks, 4, (uint64_t)num_sms));
        st.tp = a;
        out.push_back(st);
    }
};

// The NTT of one commit as steps, following the context's schedule for the
// shape (launch_ntt's choices with 512-thread CTAs: no fused tail, no
// two-stream pipeline, the deep pass's ALU multiply).
int ntt_steps(StepBuilder &sb, uint32_t schedule, const uint4 *msg, uint4 *cw, const uint4 *tw,
              std::string &why) {
    const Shape &s = sb.s;
    const int ell = s.k_code(), r = s.log_inv_rate, L = s.log_lanes, b = s.log_dim();
    const uint64_t P = (uint64_t)1 << ell;
    if (b == 0) {
        why = "persistent batch: single-column messages (no NTT layer) are not supported";
        return BZ_ERR_SHAPE;
    }
    const uint4 *src = msg;
    int src_bits = b;
    auto advance = [&]() {
        src = cw;
        src_bits = 62;
    };
    auto table_args = [&](int layer, int layers) {
        TablePassArgs a;
        a.src = src;
        a.dst = cw;
        a.tw = tw;
        a.ell = ell;
        a.layer = layer;
        a.log_lanes = L;
        a.src_pos_bits = src_bits;
        a.task_base = 0;
        a.n_tasks = (((uint64_t)1 << layer) << (ell - layer - layers)) << L;
        return a;
    };
    auto generic = [&](int layer) {
        const uint64_t tasks = (P / 2) << L;
        PStep st = sb.base(PK_GENERIC, 0, tasks, sb.items(tasks, 4096, 4 * (uint64_t)sb.num_sms));
        st.dp.src = src;
        st.dp.dst = cw;
        st.dp.tw = tw;
        st.dp.ell = ell;
        st.dp.log_lanes = L;
        st.dp.src_pos_bits = src_bits;
        st.layer = layer;
        sb.out.push_back(st);
        advance();
    };
    // one radix-4 / radix-2 table pass as launch_table_pass picks it
    auto table_pass = [&](int layer, int layers, uint32_t sched) {
        const TablePassArgs a = table_args(layer, layers);
        const bool narrow = (sched & SCHED_NARROW) && layers == 2 &&
                            narrow_class(twiddle_bits(ell, layer + 1)) <= 2;
        if (narrow) {
            const int wo = narrow_class(twiddle_bits(ell, layer));
            const int wab = narrow_class(twiddle_bits(ell, layer + 1));
            sb.table_step(PK_PF, wo * 10 + wab, a);
        } else if ((sched & SCHED_PREFETCH) && layers == 2) {
            sb.table_step(PK_PF, 44, a);
        } else {
            sb.table_step(PK_TP, layers, a);
        }
        advance();
    };
    if (!(schedule & SCHED_GENERIC) && !small_ntt_ok(s) && (schedule & SCHED_RADIX8) && L >= 9 &&
        ell - r >= 3) {
        const int rest = (ell - r) % 3;
        const uint32_t pass_sched = SCHED_PREFETCH | SCHED_NARROW;
        int layer = r;
        if ((schedule & SCHED_R8_HEAD) && rest) {
            table_pass(layer, rest, pass_sched);
            layer += rest;
        }
        while (ell - layer >= 3) {
            const int w2 = narrow_class(twiddle_bits(ell, layer + 2));
            const int w1 = std::max(narrow_class(twiddle_bits(ell, layer + 1)), w2);
            const int w0 = std::max(narrow_class(twiddle_bits(ell, layer)), w1);
            TablePassArgs a = table_args(layer, 3);
            sb.table_step(PK_PASS8, w0 * 100 + w1 * 10 + w2, a);
            advance();
            layer += 3;
        }
        if (layer < ell) table_pass(layer, ell - layer, pass_sched);
        return BZ_OK;
    }
    if ((schedule & SCHED_GENERIC) || small_ntt_ok(s)) {
        for (int layer = r; layer < ell; ++layer) generic(layer);
        return BZ_OK;
    }
    int deep = std::min<int>((int)(schedule & SCHED_DEEP_MASK), std::min(b, 4));
    const bool radix2 = (schedule & SCHED_RADIX2) != 0;
    const int table_end = ell - deep;
    int layer = r;
    while (layer < table_end) {
        const int layers = (!radix2 && layer + 1 < table_end) ? 2 : 1;
        if (!table_pass_ok(ell, layer, layers, L, 9)) {
            generic(layer);
            layer += 1;
            continue;
        }
        table_pass(layer, layers, schedule);
        layer += layers;
    }
    if (deep > 0) {
        const uint64_t tasks = (P >> deep) << L;
        PStep st = sb.base(PK_DEEP, deep, tasks, sb.items(tasks, 4096, 4 * (uint64_t)sb.num_sms));
        st.dp.src = src;
        st.dp.dst = cw;
        st.dp.tw = tw;
        st.dp.ell = ell;
        st.dp.log_lanes = L;
        st.dp.src_pos_bits = src_bits;
        st.dp.n_tasks = tasks;
        st.dp.task_base = 0;
        sb.out.push_back(st);
        advance();
    }
    return BZ_OK;
}

// Leaf hashes and tree levels (launch_merkle's kernels), the last step
// copying the root to root_dst.
int merkle_steps(StepBuilder &sb, const uint4 *cw, uint8_t *d_tree, uint32_t *root_dst,
                 std::string &why) {
    const Shape &s = sb.s;
    uint32_t *tree = reinterpret_cast<uint32_t *>(d_tree);
    const uint64_t n_leaves = s.n_leaves();
    const uint64_t cap = 4 * (uint64_t)sb.num_sms;
    if (s.hash_kind == 1 && s.log_lanes > 14) {
        why = "persistent batch: BLAKE3 leaves of more than 256 chunks are not supported";
        return BZ_ERR_SHAPE;
    }
    if (s.hash_kind == 1 && s.log_lanes >= 6) {
        const int log_c = s.log_lanes - 6;
        const uint64_t n_chunks = n_leaves << log_c;
        const uint64_t groups = (n_chunks + 511) / 512;
        PStep st = sb.base(PK_B3_CHUNKED, 0, groups, sb.items(groups, 1, cap));
        st.cw = cw;
        st.leaves = tree;
        st.count = n_chunks;
        st.log_c = log_c;
        st.chunk0 = s.chunk0;
        sb.out.push_back(st);
    } else {
        PStep st = sb.base(s.hash_kind == 1 ? PK_B3_SMALL : PK_SHA, 0, n_leaves,
                           sb.items(n_leaves, 512, cap));
        st.cw = cw;
        st.leaves = tree;
        st.log_lanes = s.log_lanes;
        sb.out.push_back(st);
    }
    // parent levels, nine per step (as launch_levels)
    uint64_t in_off = 0, n_in = n_leaves;
    while (n_in > 1) {
        int k = 0;
        for (uint64_t n = n_in; n > 1 && k < 9; n >>= 1) ++k;
        LevelsArgs a;
        a.in = tree + in_off * 8;
        a.n_in = n_in;
        a.k = k;
        a.kind = s.hash_kind;
        uint64_t off = in_off + n_in, cnt = n_in >> 1;
        for (int j = 0; j < k; ++j) {
            a.out[j] = tree + off * 8;
            off += cnt;
            cnt >>= 1;
        }
        const uint64_t groups = (n_in + 511) / 512;
        PStep st = sb.base(PK_LEVELS, 0, groups, sb.items(groups, 1, cap));
        st.lv = a;
        sb.out.push_back(st);
        uint64_t o = in_off + n_in, c = n_in >> 1;
        for (int j = 0; j < k - 1; ++j) {
            o += c;
            c >>= 1;
        }
        in_off = o;
        n_in = c;
    }
    PStep &last = sb.out.back();
    if (last.n_items != 1) {
        why = "persistent batch: the root step must be one item";
        return BZ_ERR_SHAPE;
    }
    last.root_src = tree + (s.tree_nodes() - 1) * 8;
    last.root_dst = root_dst;
    return BZ_OK;
}

}  // namespace
}  // namespace bz

using namespace bz;

extern "C" int bz_batch_plan_create_persistent(bz_ctx *ctx, size_t count,
                                               const uint64_t *const *d_msgs,
                                               const bz_params *params, bz_batch_plan **out) {
    if (!ctx || !d_msgs || !params || !out || count == 0) return BZ_ERR_ARG;
    *out = nullptr;
    bz_batch_plan *p = new bz_batch_plan();
    p->ctx = ctx;
    p->use_graph = 1;
    p->shapes.resize(count);
    int rc = BZ_OK;
    std::string why;
    for (size_t i = 0; i < count && rc == BZ_OK; ++i) {
        if (!d_msgs[i]) rc = set_msg(ctx, BZ_ERR_ARG, "null message");
        if (rc == BZ_OK) {
            rc = shape_from_params(&params[i], p->shapes[i], (size_t)1 << params[i].log_msg_len,
                                   why);
            if (rc) set_msg(ctx, rc, why);
        }
        if (rc == BZ_OK) {
            p->msgs.push_back((const uint4 *)d_msgs[i]);
            p->schedules.push_back(schedule_for(ctx, p->shapes[i]));
            bz_commitment *c = nullptr;
            rc = alloc_commitment(ctx, p->shapes[i], &c);
            p->commits.push_back(c);
        }
    }
    if (rc == BZ_OK) rc = dev_alloc(ctx, count * 32, (void **)&p->d_roots, false);
    // steps, commits in decreasing size (the scheduler's priority order)
    std::vector<PStep> steps;
    std::vector<PCommit> table;
    if (rc == BZ_OK) {
        std::vector<size_t> order(count);
        std::iota(order.begin(), order.end(), (size_t)0);
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return p->shapes[a].cw_words() > p->shapes[b].cw_words();
        });
        for (size_t slot = 0; slot < count && rc == BZ_OK; ++slot) {
            const size_t i = order[slot];
            const Shape &s = p->shapes[i];
            const uint4 *tw = nullptr;
            rc = get_twiddles(ctx, s.k_code(), &tw);
            if (rc) break;
            StepBuilder sb{s, (uint32_t)slot, ctx->num_sms, steps};
            const size_t first = steps.size();
            rc = ntt_steps(sb, p->schedules[i], p->msgs[i], p->commits[i]->d_cw, tw, why);
            if (rc == BZ_OK)
                rc = merkle_steps(sb, p->commits[i]->d_cw, p->commits[i]->d_tree,
                                  reinterpret_cast<uint32_t *>(p->d_roots + 32 * i), why);
            if (rc) {
                set_msg(ctx, rc, why);
                break;
            }
            table.push_back({(uint32_t)first, (uint32_t)(steps.size() - first)});
        }
    }
    // one device block: steps | commit table | state (steps_done, err, pad,
    // cur[count], claim[G], done[G]), the state zeroed by every launch
    const size_t G = steps.size();
    const size_t steps_bytes = (G * sizeof(PStep) + 255) & ~(size_t)255;
    const size_t table_bytes = (count * sizeof(PCommit) + 255) & ~(size_t)255;
    const size_t state_words = 4 + count + 2 * G;
    const size_t state_bytes = state_words * 4;
    if (rc == BZ_OK)
        rc = dev_alloc(ctx, steps_bytes + table_bytes + state_bytes, &p->d_persist, false);
    PersistArgs args{};
    if (rc == BZ_OK) {
        char *base = static_cast<char *>(p->d_persist);
        uint32_t *state = reinterpret_cast<uint32_t *>(base + steps_bytes + table_bytes);
        args.steps = reinterpret_cast<const PStep *>(base);
        args.commits = reinterpret_cast<const PCommit *>(base + steps_bytes);
        args.n_commits = (uint32_t)count;
        args.total_steps = (uint32_t)G;
        args.steps_done = state;
        args.err = state + 1;
        args.cur = state + 4;
        args.claim = state + 4 + count;
        args.done = state + 4 + count + G;
        args.limit_ns = kPersistWaitNs;
        p->d_persist_err = state + 1;
        cudaError_t e = cudaMemcpy(base, steps.data(), G * sizeof(PStep), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(base + steps_bytes, table.data(), count * sizeof(PCommit),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(persistent_batch_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPersistSmem);
        int per_sm = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_batch_kernel, 512,
                                                              kPersistSmem);
        if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "persistent plan setup", e);
        else if (per_sm < 1) rc = set_msg(ctx, BZ_ERR_CUDA, "persistent batch kernel does not fit an SM");
        if (rc == BZ_OK) {
            p->persist_args.assign(reinterpret_cast<const char *>(&args),
                                   reinterpret_cast<const char *>(&args) + sizeof args);
            p->persist_state_bytes = state_bytes;
            // one graph: reset the scheduler state, then the kernel
            e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                cudaMemsetAsync(state, 0, state_bytes, ctx->stream);
                persistent_batch_kernel<<<ctx->num_sms, 512, kPersistSmem, ctx->stream>>>(args);
                cudaError_t le = cudaGetLastError();
                e = cudaStreamEndCapture(ctx->stream, &p->graph);
                if (e == cudaSuccess) e = le;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
            if (e == cudaSuccess) e = cudaGraphUpload(p->exec, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "persistent plan graph", e);
        }
    }
    if (rc != BZ_OK) {
        cudaGetLastError();
        bz_batch_plan_destroy(p);
        return rc;
    }
    *out = p;
    return BZ_OK;
}

// Test hook: one direct launch of the plan's kernel that expects one step more
// than the plan has, with a wait limit of limit_ms.  Every CTA runs the real
// items, then finds nothing ready and gives up after the limit; the error word
// is read back and the state reset.  BZ_ERR_TIMEOUT when the kernel reported
// the expired wait.
extern "C" int bz_batch_plan_stall_check(bz_batch_plan *p, uint32_t limit_ms) {
    if (!p || p->persist_args.size() != sizeof(PersistArgs) || limit_ms == 0) return BZ_ERR_ARG;
    bz_ctx *ctx = p->ctx;
    PersistArgs args;
    memcpy(&args, p->persist_args.data(), sizeof args);
    args.total_steps += 1;  // a step that no item completes
    args.limit_ns = (uint64_t)limit_ms * 1000000ull;
    uint32_t *state = args.steps_done;
    uint32_t err = 0;
    cudaError_t e = cudaMemsetAsync(state, 0, p->persist_state_bytes, ctx->stream);
    if (e == cudaSuccess) {
        persistent_batch_kernel<<<ctx->num_sms, 512, kPersistSmem, ctx->stream>>>(args);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&err, args.err, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(state, 0, p->persist_state_bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return set_err(ctx, BZ_ERR_CUDA, "persistent stall check", e);
    return err ? set_msg(ctx, BZ_ERR_TIMEOUT, "persistent batch: bounded wait ran out")
               : BZ_OK;
}
