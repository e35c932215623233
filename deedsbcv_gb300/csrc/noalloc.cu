// Allocation-free entry point: the inverse-consistency stage with its scratch
// in a fixed device array instead of context-owned memory.
//
// Some callers of this library cannot allocate device memory while they run:
// code embedded in a host framework whose memory pool owns the whole device
// (an allocation outside the pool fails or evicts its cache), real-time or
// serving loops that size everything at start-up and treat an allocation in
// steady state as a fault, and callers that must not block, because
// cudaMalloc / cudaFree may synchronise the device.  For them
// deeds_consistent_noalloc_dev() runs the same kernels as deeds_consistent_dev()
// with its scratch in g_consistent_scratch below.
//
// The array is a file-scope __device__ array: every GPU that loads the library
// holds its 12 x DEEDS_NOALLOC_MAX_NODES floats (6 MiB) until the process exits.
// Host code cannot use the symbol itself as a device address (in host code it
// is a host-side stand-in), so the first call on each device, with that device
// current, resolves the address with cudaGetSymbolAddress and keeps it; make
// that first call before any stream capture.  All calls share the array and it
// keeps the last call's contents; the kernels write every scratch element they
// read, so nothing needs clearing, but calls that overlap on the GPU race.
#include <atomic>

#include "../../include/deeds_gpu.h"
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr size_t kScratchFloats = (size_t)12 * DEEDS_NOALLOC_MAX_NODES;
__device__ __align__(256) float g_consistent_scratch[kScratchFloats];

constexpr int kMaxDevices = 64;
std::atomic<float*> g_scratch_addr[kMaxDevices];  // per device ordinal, resolved once

}  // namespace

extern "C" deeds_status deeds_consistent_noalloc_dev(float* d_u, float* d_v, float* d_w, float* d_u2, float* d_v2,
                                                     float* d_w2, int m, int n, int o, int g, void* stream) {
    if (!d_u || !d_v || !d_w || !d_u2 || !d_v2 || !d_w2 || m < 1 || n < 1 || o < 1 || g < 1) return DEEDS_ERR_INVALID;
    if ((long long)m * n * o > DEEDS_NOALLOC_MAX_NODES) return DEEDS_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DEEDS_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return DEEDS_ERR_INVALID;
    float* scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!scratch) {
        void* addr = nullptr;
        if (cudaGetSymbolAddress(&addr, g_consistent_scratch) != cudaSuccess || !addr) {
            cudaGetLastError();
            return DEEDS_ERR_CUDA;
        }
        scratch = static_cast<float*>(addr);
        g_scratch_addr[dev].store(scratch, std::memory_order_release);
    }
    if (deeds::launch_consistent(d_u, d_v, d_w, d_u2, d_v2, d_w2, m, n, o, g, scratch, (cudaStream_t)stream) !=
        cudaSuccess)
        return DEEDS_ERR_CUDA;
    return DEEDS_OK;
}
