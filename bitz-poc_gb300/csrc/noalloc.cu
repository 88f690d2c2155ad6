// Allocation-free variant of the sumcheck fold + next-round message
// (bz_fold_and_msg_lsb).
//
// Who needs it: callers that must not allocate device memory themselves or
// through this library -- for example a prover host whose runtime reserved
// the GPU's memory up front for its own pool (a cudaMalloc from here would
// fail, or would break that pool's accounting), or a latency-critical fold
// loop that cannot pay for cudaMalloc's implicit synchronisation.  They pass
// their own input and output buffers; the only scratch the fold needs (one
// 256-bit partial sum pair per thread block) lives in the fixed device array
// below.  Every GPU that loads the library holds that array (64 KiB) until the
// process exits.
//
// The array's name is a host-side stand-in in host code, not a device
// address, so the entry point resolves the real address once per device with
// cudaGetSymbolAddress (on the first call made while that device is current)
// and passes it to the kernels.  Make that first call on each device before
// any stream capture.  The address and the kernels' shared-memory opt-in are
// kept for the life of the process, so a cudaDeviceReset after the first
// call on a device is not supported.  A launch error already pending on the
// calling thread is reported (BZ_ERR_CUDA) before anything is launched and
// left in place for its owner.  All calls share the array and it keeps the previous
// call's contents: nothing in it has to start at zero (every block overwrites
// its own slot and the final kernel reads only the slots of the current
// launch), but calls that overlap on the GPU -- two streams, two threads --
// race on it and give wrong results.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bitz_gpu.h"
#include "bz_internal.h"

namespace {

constexpr int kMaxBlocks = 1024;   // the fold launch never uses more blocks
constexpr int kMaxDevices = 64;
constexpr size_t kMaxWords = (size_t)1 << 40;

static __device__ __align__(256) uint64_t g_fold_partials[kMaxBlocks * 8];

std::mutex g_mu;
uint64_t *g_partials_addr[kMaxDevices] = {nullptr};
int g_num_sms[kMaxDevices] = {0};

bool pow2(size_t n) { return n && !(n & (n - 1)); }

}  // namespace

extern "C" int bz_fold_and_msg_lsb_static(const uint64_t *d_f, const uint64_t *d_b, size_t n,
                                          const uint64_t r[2], uint64_t *d_nf, uint64_t *d_nb,
                                          uint64_t *d_msg, void *stream) {
    if (!d_f || !d_b || !r || !d_nf || !d_nb || !d_msg) return BZ_ERR_ARG;
    if (!pow2(n) || n < 2) return BZ_ERR_SHAPE;  // n must be a power of two >= 2
    if (n > kMaxWords) return BZ_ERR_SHAPE;      // beyond 2^40 elements
    // an error some earlier launch left pending belongs to its owner: report
    // it without clearing it, so this call's own status cannot be mistaken
    if (cudaPeekAtLastError() != cudaSuccess) return BZ_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return BZ_ERR_CUDA;
    }
    uint64_t *partials = nullptr;
    int num_sms = 0;
    {
        std::lock_guard<std::mutex> g(g_mu);
        if (!g_partials_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_fold_partials) != cudaSuccess) {
                cudaGetLastError();
                return BZ_ERR_CUDA;
            }
            int sms = 0;
            if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
                cudaGetLastError();
                return BZ_ERR_CUDA;
            }
            // the fold kernel keeps the challenge's byte tables in 66 KB of
            // dynamic shared memory; opt in for this device (no allocation)
            bz::init_fold_kernels();
            // nothing was pending before (checked above), so this error is
            // the attribute call's own
            if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
            g_partials_addr[dev] = (uint64_t *)p;
            g_num_sms[dev] = sms;
        }
        partials = g_partials_addr[dev];
        num_sms = g_num_sms[dev];
    }
    const uint4 rr = make_uint4((uint32_t)r[0], (uint32_t)(r[0] >> 32), (uint32_t)r[1],
                                (uint32_t)(r[1] >> 32));
    bz::launch_fold_and_msg((const uint4 *)d_f, (const uint4 *)d_b, n, rr, (uint4 *)d_nf,
                            (uint4 *)d_nb, partials, d_msg, (cudaStream_t)stream, num_sms);
    // read right after this call's own launches (no error was pending before)
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
