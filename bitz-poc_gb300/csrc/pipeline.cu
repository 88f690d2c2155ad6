// Two-stream software pipeline of one commit.
//
// The table passes are bound by the shared-memory pipe (byte-table lookups)
// while the deep layers and the BLAKE3 leaf hashes are bound by the ALU pipe.
// After the first table pass the codeword splits into independent position
// chunks (blocks of the next layer), so chunk k's remaining table passes run
// on the main stream while chunk k-1's deep layers and leaf hashes run on the
// auxiliary stream.  With 256-thread table-pass CTAs (schedule bit
// SCHED_SMALL_CTA) the two kinds of CTAs fit on one SM together and their
// pipes overlap.  The parent levels of the tree run once all chunks joined.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "bz_internal.h"

namespace bz {

int launch_commit_pipelined(const Shape &s, uint32_t schedule, const uint4 *d_msg, uint4 *d_cw,
                            uint8_t *d_tree, const uint4 *d_tw, cudaStream_t st,
                            cudaStream_t aux, cudaEvent_t *ev, int num_sms, LaunchLog *log) {
    const int pipe_log = (int)((schedule >> SCHED_PIPE_SHIFT) & 3);
    if (pipe_log == 0 || !aux || !ev) return -1;
    if (schedule & (SCHED_GENERIC | SCHED_FUSED_TAIL)) return -1;
    if (!leaves_range_supported(s)) return -1;
    const int ell = s.k_code(), r = s.log_inv_rate, L = s.log_lanes, b = s.log_dim();
    if (b < 2) return -1;
    int deep = (int)(schedule & SCHED_DEEP_MASK);
    deep = std::min(std::min(deep, b), 4);
    const bool radix2 = (schedule & SCHED_RADIX2) != 0;
    const int mode = (int)((schedule >> SCHED_MODE_SHIFT) & 3);
    const int threads = (schedule & SCHED_SMALL_CTA) ? 256 : 512;
    const int log_threads = threads == 256 ? 8 : 9;
    const int table_end = ell - deep;
    if (table_end <= r) return -1;
    const int first = (!radix2 && table_end - r >= 2) ? 2 : 1;
    const int chunks = 1 << pipe_log;
    if (r + first < pipe_log) return -1;  // not enough independent blocks
    // every table pass must be a table pass (not the generic fallback)
    for (int layer = r; layer < table_end;) {
        const int layers = (layer == r) ? first : ((!radix2 && layer + 1 < table_end) ? 2 : 1);
        if (ell - layer - layers + L < log_threads) return -1;
        layer += layers;
    }
    const uint64_t P = (uint64_t)1 << ell;
    int launches =
        launch_table_pass(s, r, first, d_msg, b, d_cw, d_tw, 0, P, threads, st, num_sms, schedule);
    if (log)
        log->mark((std::string(first == 2 ? "ntt_table_pass2_first" : "ntt_table_pass1_first") +
                   "@" + std::to_string(r))
                      .c_str());
    for (int k = 0; k < chunks; ++k) {
        const uint64_t p0 = P / chunks * k, p1 = P / chunks * (k + 1);
        for (int layer = r + first; layer < table_end;) {
            const int layers = (!radix2 && layer + 1 < table_end) ? 2 : 1;
            launches += launch_table_pass(s, layer, layers, d_cw, 62, d_cw, d_tw, p0, p1, threads,
                                          st, num_sms, schedule);
            layer += layers;
        }
        cudaEventRecord(ev[k], st);
        cudaStreamWaitEvent(aux, ev[k], 0);
        if (deep > 0)
            launches += launch_deep_range(s, deep, mode, d_cw, 62, d_cw, d_tw, p0, p1, aux,
                                          num_sms);
        launches += launch_leaves_range(s, d_cw, d_tree, p0, p1, aux, num_sms);
    }
    cudaEventRecord(ev[chunks], aux);
    cudaStreamWaitEvent(st, ev[chunks], 0);
    if (log) log->mark("pipelined_passes_and_leaves");
    launches += launch_merkle_levels(s, d_tree, st, log);
    return launches;
}

}  // namespace bz
