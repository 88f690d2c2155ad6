// Batched commits captured into one CUDA graph, the NTT schedule autotuner
// and the host-side ChaCha20 input generator.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "runtime.h"

using namespace bz;

namespace {

// RFC 8439 block function (host).
inline uint32_t rotl32(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }
void chacha_block(uint32_t k0, uint32_t k1, uint32_t counter, uint32_t out[16]) {
    uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, k0, k1, 0, 0,
                       0, 0, 0, 0, counter, 0, 0, 0};
    uint32_t x[16];
    memcpy(x, st, sizeof x);
    auto qr = [&](int a, int b, int c, int d) {
        x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16);
        x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12);
        x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);
        x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
    };
    for (int i = 0; i < 10; ++i) {
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15);
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14);
    }
    for (int i = 0; i < 16; ++i) out[i] = x[i] + st[i];
}

void chacha_range(uint64_t seed, uint64_t first_word, uint64_t *out, size_t lo, size_t hi) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    uint32_t blk[16];
    uint64_t cached = ~0ull;
    for (size_t i = lo; i < hi; ++i) {
        const uint64_t w = first_word + i, b = w >> 2;
        if (b != cached) {
            chacha_block(k0, k1, (uint32_t)b, blk);
            cached = b;
        }
        const uint32_t *p = blk + 4 * (w & 3);
        out[2 * i] = (uint64_t)p[0] | ((uint64_t)p[1] << 32);
        out[2 * i + 1] = (uint64_t)p[2] | ((uint64_t)p[3] << 32);
    }
}

}  // namespace

extern "C" {

int bz_chacha_fill_host(uint64_t seed, uint64_t first_word, uint64_t *out, size_t n_words,
                        int n_threads) {
    if (n_words && !out) return BZ_ERR_ARG;
    if (n_threads < 1) n_threads = 1;
    if (n_threads == 1 || n_words < (1u << 16)) {
        chacha_range(seed, first_word, out, 0, n_words);
        return BZ_OK;
    }
    std::vector<std::thread> th;
    const size_t per = ((n_words + n_threads - 1) / n_threads + 3) & ~(size_t)3;
    for (int t = 0; t < n_threads; ++t) {
        const size_t lo = (size_t)t * per, hi = std::min(n_words, lo + per);
        if (lo >= hi) break;
        th.emplace_back(chacha_range, seed, first_word, out, lo, hi);
    }
    for (auto &t : th) t.join();
    return BZ_OK;
}

// ---- batched commit -------------------------------------------------------
int bz_commit_batch_device(bz_ctx *ctx, size_t count, const uint64_t *const *d_msgs,
                           const bz_params *params, bz_commitment **outs, uint8_t *roots,
                           int use_graph) {
    if (!ctx || !d_msgs || !params || !outs) return BZ_ERR_ARG;
    std::vector<Shape> shapes(count);
    for (size_t i = 0; i < count; ++i) {
        outs[i] = nullptr;
        std::string why;
        if (!d_msgs[i]) return set_msg(ctx, BZ_ERR_ARG, "null message");
        int rc = shape_from_params(&params[i], shapes[i],
                                   (size_t)1 << params[i].log_msg_len, why);
        if (rc) return set_msg(ctx, rc, why);
    }
    // Resident buffers, twiddles and scratch are set up before any capture.
    size_t scratch = 0;
    for (size_t i = 0; i < count; ++i) {
        const uint4 *tw = nullptr;
        int rc = get_twiddles(ctx, shapes[i].k_code(), &tw);
        if (rc) return rc;
        scratch = std::max(scratch, merkle_scratch_bytes(shapes[i]));
        rc = alloc_commitment(ctx, shapes[i], &outs[i]);
        if (rc) {
            for (size_t j = 0; j < i; ++j) {
                bz_commitment_free(outs[j]);
                outs[j] = nullptr;
            }
            return rc;
        }
    }
    if (scratch) {
        int rc = ensure_scratch(ctx, scratch);
        if (rc) return rc;
    }
    if (!get_aux(ctx, ctx->stream)) return set_msg(ctx, BZ_ERR_CUDA, "aux stream");
    void *d_roots = nullptr;
    int rc = dev_alloc(ctx, count * 32, &d_roots, false);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return set_err(ctx, BZ_ERR_CUDA, "begin capture", e);
    }
    for (size_t i = 0; i < count && rc == BZ_OK; ++i) {
        rc = enqueue_commit(ctx, shapes[i], (const uint4 *)d_msgs[i], outs[i], st,
                            schedule_for(ctx, shapes[i]));
        if (rc == BZ_OK) {
            const uint8_t *src = outs[i]->d_tree + (shapes[i].tree_nodes() - 1) * 32;
            cudaMemcpyAsync((uint8_t *)d_roots + 32 * i, src, 32, cudaMemcpyDeviceToDevice, st);
        }
    }
    if (use_graph) {
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (rc == BZ_OK && e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "end capture", e);
        if (rc == BZ_OK) {
            e = cudaGraphInstantiate(&exec, graph, 0);
            if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "instantiate", e);
        }
        if (rc == BZ_OK) {
            e = cudaGraphLaunch(exec, st);
            if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "graph launch", e);
        }
    }
    if (rc == BZ_OK && roots) {
        cudaMemcpyAsync(roots, d_roots, count * 32, cudaMemcpyDeviceToHost, st);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == BZ_OK && e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "batch sync", e);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    dev_free(ctx, d_roots, 0, false);
    if (rc == BZ_OK && roots) {
        for (size_t i = 0; i < count; ++i) {
            memcpy(outs[i]->root, roots + 32 * i, 32);
            outs[i]->root_ready = true;
        }
    }
    if (rc != BZ_OK) {
        for (size_t i = 0; i < count; ++i) {
            if (outs[i]) bz_commitment_free(outs[i]);
            outs[i] = nullptr;
        }
    }
    return rc;
}

// ---- schedules ------------------------------------------------------------
int bz_schedule_get(bz_ctx *ctx, const bz_params *params, uint32_t *schedule) {
    if (!ctx || !params || !schedule) return BZ_ERR_ARG;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, (size_t)1 << params->log_msg_len, why);
    if (rc) return set_msg(ctx, rc, why);
    *schedule = schedule_for(ctx, s);
    return BZ_OK;
}

int bz_schedule_set(bz_ctx *ctx, const bz_params *params, uint32_t schedule) {
    if (!ctx || !params) return BZ_ERR_ARG;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, (size_t)1 << params->log_msg_len, why);
    if (rc) return set_msg(ctx, rc, why);
    std::lock_guard<std::mutex> g(ctx->sched_mu);
    ctx->schedules[shape_key(s)] = schedule;
    return BZ_OK;
}

int bz_autotune(bz_ctx *ctx, const bz_params *params, int reps, uint32_t *chosen) {
    if (!ctx || !params) return BZ_ERR_ARG;
    Shape s;
    std::string why;
    int rc = shape_from_params(params, s, (size_t)1 << params->log_msg_len, why);
    if (rc) return set_msg(ctx, rc, why);
    if (reps < 1) reps = 1;
    void *d_msg = nullptr;
    rc = dev_alloc(ctx, s.msg_words() * 16, &d_msg, false);
    if (rc) return rc;
    bz_chacha_fill_device(ctx, 12345, 0, (uint64_t *)d_msg, s.msg_words());
    bz_commitment *c = nullptr;
    rc = alloc_commitment(ctx, s, &c);
    if (rc) {
        dev_free(ctx, d_msg, 0, false);
        return rc;
    }
    std::vector<uint32_t> cands;
    const int b = s.log_dim();
    if (s.log_lanes >= 9 && s.k_code() - s.log_inv_rate >= 3) {
        // radix-8 passes, the leftover layers last or first
        cands.push_back(SCHED_RADIX8);
        if ((s.k_code() - s.log_inv_rate) % 3) cands.push_back(SCHED_RADIX8 | SCHED_R8_HEAD);
    }
    for (int d = 0; d <= std::min(4, b); ++d) {
        for (uint32_t r2 : {0u, (uint32_t)SCHED_RADIX2}) {
            if (d == 0) {
                // byte tables for every layer: plain, prefetching, 256-thread and
                // register-capped CTAs, each also as a two-stream pipeline whose
                // leaf hashing can share SMs with the capped table passes
                for (uint32_t extra : {0u, (uint32_t)SCHED_PREFETCH,
                                       (uint32_t)(SCHED_PREFETCH | SCHED_NARROW),
                                       (uint32_t)(SCHED_PREFETCH | SCHED_SMALL_CTA),
                                       (uint32_t)SCHED_SMALL_CTA,
                                       (uint32_t)(SCHED_PREFETCH | SCHED_SMALL_CTA | SCHED_LEAN)})
                    for (uint32_t pipe = 0; pipe < 4; ++pipe)
                        cands.push_back(r2 | extra | (pipe << SCHED_PIPE_SHIFT));
                continue;
            }
            for (uint32_t mode = 0; mode < 3; ++mode) {
                cands.push_back((uint32_t)d | r2 | (mode << SCHED_MODE_SHIFT));
                if (s.log_lanes >= 9 && d <= 3)
                    cands.push_back((uint32_t)d | r2 | SCHED_FUSED_TAIL |
                                    (mode << SCHED_MODE_SHIFT));
            }
            cands.push_back((uint32_t)d | r2 | SCHED_PREFETCH);
            cands.push_back((uint32_t)d | r2 | SCHED_PREFETCH | SCHED_NARROW);
            cands.push_back((uint32_t)d | r2 | SCHED_PREFETCH | SCHED_SMALL_CTA);
            for (uint32_t small : {0u, (uint32_t)SCHED_SMALL_CTA})
                for (uint32_t pipe = 0; pipe < 4; ++pipe)
                    if (small || pipe)
                        cands.push_back((uint32_t)d | r2 | small | (pipe << SCHED_PIPE_SHIFT));
        }
    }
    float best = 1e30f;
    uint32_t best_s = default_schedule(s);
    for (uint32_t cand : cands) {
        // warm-up, then timed reps
        rc = enqueue_commit(ctx, s, (const uint4 *)d_msg, c, ctx->stream, cand);
        if (rc) break;
        cudaEventRecord(ctx->ev0, ctx->stream);
        for (int r = 0; r < reps && rc == BZ_OK; ++r)
            rc = enqueue_commit(ctx, s, (const uint4 *)d_msg, c, ctx->stream, cand);
        cudaEventRecord(ctx->ev1, ctx->stream);
        if (cudaEventSynchronize(ctx->ev1) != cudaSuccess) {
            rc = set_msg(ctx, BZ_ERR_CUDA, "autotune sync");
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        if (ms < best) {
            best = ms;
            best_s = cand;
        }
    }
    bz_commitment_free(c);
    dev_free(ctx, d_msg, 0, false);
    cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> g(ctx->sched_mu);
        ctx->schedules[shape_key(s)] = best_s;
    }
    if (chosen) *chosen = best_s;
    return BZ_OK;
}

}  // extern "C"

// ===========================================================================
// Reusable batch plans.
// ===========================================================================
namespace {

// Enqueue every commit of the plan: polynomials are dealt to the branch
// streams largest first (longest-processing-time), forked from and joined back
// into the context stream.
int plan_enqueue(bz_batch_plan *p) {
    bz_ctx *ctx = p->ctx;
    cudaStream_t main = ctx->stream;
    const int nb = p->n_branches;
    cudaEventRecord(p->fork_join[0], main);
    for (int b = 0; b < nb; ++b) cudaStreamWaitEvent(p->branches[b], p->fork_join[0], 0);
    std::vector<size_t> order(p->shapes.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return p->shapes[a].cw_words() > p->shapes[b].cw_words();
    });
    std::vector<double> load(nb, 0.0);
    int rc = BZ_OK;
    for (size_t i : order) {
        const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[b] += (double)p->shapes[i].cw_words();
        cudaStream_t st = p->branches[b];
        rc = enqueue_commit(ctx, p->shapes[i], p->msgs[i], p->commits[i], st, p->schedules[i]);
        if (rc) break;
        const uint8_t *src = p->commits[i]->d_tree + (p->shapes[i].tree_nodes() - 1) * 32;
        cudaMemcpyAsync(p->d_roots + 32 * i, src, 32, cudaMemcpyDeviceToDevice, st);
    }
    for (int b = 0; b < nb; ++b) {
        cudaEventRecord(p->fork_join[1 + b], p->branches[b]);
        cudaStreamWaitEvent(main, p->fork_join[1 + b], 0);
    }
    return rc;
}

}  // namespace

extern "C" {

int bz_batch_plan_destroy(bz_batch_plan *p) {
    if (!p) return BZ_ERR_ARG;
    bz_ctx *ctx = p->ctx;
    cudaStreamSynchronize(ctx->stream);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    for (auto *c : p->commits)
        if (c) bz_commitment_free(c);
    if (p->d_roots) dev_free(ctx, p->d_roots, 0, false);
    if (p->d_persist) dev_free(ctx, p->d_persist, 0, false);
    for (auto s : p->branches) cudaStreamDestroy(s);
    for (auto e : p->fork_join) cudaEventDestroy(e);
    cudaStreamSynchronize(ctx->stream);
    delete p;
    return BZ_OK;
}

int bz_batch_plan_create(bz_ctx *ctx, size_t count, const uint64_t *const *d_msgs,
                         const bz_params *params, int use_graph, int n_branches,
                         bz_batch_plan **out) {
    if (!ctx || !d_msgs || !params || !out || count == 0) return BZ_ERR_ARG;
    *out = nullptr;
    bz_batch_plan *p = new bz_batch_plan();
    p->ctx = ctx;
    p->use_graph = use_graph;
    p->n_branches = std::max(1, std::min(n_branches, 16));
    p->shapes.resize(count);
    int rc = BZ_OK;
    size_t scratch = 0;
    for (size_t i = 0; i < count && rc == BZ_OK; ++i) {
        std::string why;
        if (!d_msgs[i]) rc = set_msg(ctx, BZ_ERR_ARG, "null message");
        if (rc == BZ_OK) {
            rc = shape_from_params(&params[i], p->shapes[i], (size_t)1 << params[i].log_msg_len,
                                   why);
            if (rc) set_msg(ctx, rc, why);
        }
        if (rc == BZ_OK && merkle_scratch_bytes(p->shapes[i]) > 0 && p->n_branches > 1)
            rc = set_msg(ctx, BZ_ERR_SHAPE,
                         "leaves above 256 chunks need the shared scratch: use one branch");
        if (rc == BZ_OK) {
            const uint4 *tw = nullptr;
            rc = get_twiddles(ctx, p->shapes[i].k_code(), &tw);
        }
        if (rc == BZ_OK) {
            scratch = std::max(scratch, merkle_scratch_bytes(p->shapes[i]));
            p->msgs.push_back((const uint4 *)d_msgs[i]);
            p->schedules.push_back(schedule_for(ctx, p->shapes[i]));
            bz_commitment *c = nullptr;
            rc = alloc_commitment(ctx, p->shapes[i], &c);
            p->commits.push_back(c);
        }
    }
    if (rc == BZ_OK && scratch) rc = ensure_scratch(ctx, scratch);
    if (rc == BZ_OK) rc = dev_alloc(ctx, count * 32, (void **)&p->d_roots, false);
    if (rc == BZ_OK) {
        p->branches.resize(p->n_branches);
        p->fork_join.resize(p->n_branches + 1);
        for (auto &s : p->branches) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        for (auto &e : p->fork_join) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        cudaStreamSynchronize(ctx->stream);
    }
    if (rc == BZ_OK) {
        // auxiliary streams of pipelined schedules exist before any capture
        for (auto st : p->branches)
            if (!get_aux(ctx, st)) rc = set_msg(ctx, BZ_ERR_CUDA, "aux stream");
    }
    if (rc == BZ_OK && use_graph) {
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "begin capture", e);
        if (rc == BZ_OK) {
            rc = plan_enqueue(p);
            e = cudaStreamEndCapture(ctx->stream, &p->graph);
            if (rc == BZ_OK && e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "end capture", e);
        }
        if (rc == BZ_OK) {
            e = cudaGraphInstantiate(&p->exec, p->graph, 0);
            if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "instantiate", e);
        }
        if (rc == BZ_OK) {
            e = cudaGraphUpload(p->exec, ctx->stream);
            if (e != cudaSuccess) rc = set_err(ctx, BZ_ERR_CUDA, "upload", e);
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

int bz_batch_plan_launch(bz_batch_plan *p) {
    if (!p) return BZ_ERR_ARG;
    bz_ctx *ctx = p->ctx;
    if (p->use_graph) {
        cudaError_t e = cudaGraphLaunch(p->exec, ctx->stream);
        if (e != cudaSuccess) return set_err(ctx, BZ_ERR_CUDA, "graph launch", e);
        // a graph of per-commit kernels was counted at capture time; a
        // persistent plan's graph holds one kernel
        if (p->d_persist) ctx->launches += 1;
        return BZ_OK;
    }
    return plan_enqueue(p);
}

int bz_batch_plan_roots(bz_batch_plan *p, uint8_t *roots) {
    if (!p || !roots) return BZ_ERR_ARG;
    bz_ctx *ctx = p->ctx;
    const size_t n = p->commits.size();
    cudaError_t e = cudaMemcpyAsync(roots, p->d_roots, n * 32, cudaMemcpyDeviceToHost, ctx->stream);
    uint32_t perr = 0;
    if (e == cudaSuccess && p->d_persist_err)
        e = cudaMemcpyAsync(&perr, p->d_persist_err, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return set_err(ctx, BZ_ERR_CUDA, "plan roots", e);
    if (perr)
        return set_msg(ctx, BZ_ERR_TIMEOUT,
                       "persistent batch: a CTA found no ready work item within its limit");
    for (size_t i = 0; i < n; ++i) {
        memcpy(p->commits[i]->root, roots + 32 * i, 32);
        p->commits[i]->root_ready = true;
    }
    return BZ_OK;
}

bz_commitment *bz_batch_plan_commitment(bz_batch_plan *p, size_t i) {
    if (!p || i >= p->commits.size()) return nullptr;
    return p->commits[i];
}

}  // extern "C"
