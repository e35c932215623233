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
// The array is a file-scope __device__ array of 12 x DEEDS_NOALLOC_MAX_NODES
// floats (6 MiB).  With lazy module loading (the CUDA default) it is reserved
// when this file's module is loaded into a context, which happens at the first
// call on a device, not when the library is loaded; from then on the device
// holds it until the context ends (process exit or cudaDeviceReset).  That first
// call can therefore fail with DEEDS_ERR_CUDA if a memory pool already holds the
// whole device: make it at start-up, before a framework reserves the device and
// before any stream capture.
//
// Host code cannot use the symbol itself as a device address (in host code it
// is a host-side stand-in), so the address is resolved with cudaGetSymbolAddress
// with the device current and kept per device together with the identity of
// the context it belongs to (cuCtxGetId: unique for the process lifetime).  A
// call in a different context of that device (after cudaDeviceReset, or under
// a non-primary context) resolves the address again, which reloads the module
// there; the stale address of a destroyed context is never used.
//
// All calls share the array and it keeps the last call's contents; the kernels
// write every scratch element before they read it, so nothing needs clearing,
// but calls that overlap on the GPU race.
#include <cuda.h>

#include <cstdint>
#include <mutex>

#include "../../include/deeds_gpu.h"
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr size_t kScratchFloats = (size_t)12 * DEEDS_NOALLOC_MAX_NODES;
__device__ __align__(256) float g_consistent_scratch[kScratchFloats];

constexpr int kMaxDevices = 64;
// Grid limits of the stage's kernels: gridDim.y = n and gridDim.z = o.
constexpr int kMaxGridYZ = 65535;

struct ScratchSlot {
    unsigned long long ctx_id = 0;  // context the address belongs to (0: none yet)
    float* addr = nullptr;
};
ScratchSlot g_slots[kMaxDevices];
std::mutex g_slots_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// The current context's process-unique id; 0 when no context is current yet (the
// runtime creates the primary context on its first call that needs one) or the
// driver cannot tell.
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

extern "C" deeds_status deeds_consistent_noalloc_dev(float* d_u, float* d_v, float* d_w, float* d_u2, float* d_v2,
                                                     float* d_w2, int m, int n, int o, int g, void* stream) {
    if (!d_u || !d_v || !d_w || !d_u2 || !d_v2 || !d_w2 || m < 1 || n < 1 || o < 1 || g < 1) return DEEDS_ERR_INVALID;
    if ((long long)m * n * o > DEEDS_NOALLOC_MAX_NODES) return DEEDS_ERR_INVALID;
    if (n > kMaxGridYZ || o > kMaxGridYZ) return DEEDS_ERR_INVALID;  // checked before any launch: fields untouched
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DEEDS_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return DEEDS_ERR_INVALID;
    float* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_slots_mu);
        ScratchSlot& slot = g_slots[dev];
        const unsigned long long id = current_ctx_id();
        if (id != 0 && slot.ctx_id == id) {
            scratch = slot.addr;
        } else {
            void* addr = nullptr;
            if (cudaGetSymbolAddress(&addr, g_consistent_scratch) != cudaSuccess || !addr) {
                cudaGetLastError();
                return DEEDS_ERR_CUDA;
            }
            scratch = static_cast<float*>(addr);
            // the runtime has made its context current by now; an id of 0 (driver
            // without cuCtxGetId) keeps nothing, so every call resolves afresh
            slot.ctx_id = current_ctx_id();
            slot.addr = slot.ctx_id ? scratch : nullptr;
        }
    }
    if (deeds::launch_consistent(d_u, d_v, d_w, d_u2, d_v2, d_w2, m, n, o, g, scratch, (cudaStream_t)stream) !=
        cudaSuccess)
        return DEEDS_ERR_CUDA;
    return DEEDS_OK;
}
