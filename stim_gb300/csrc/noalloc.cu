// Fixed device scratch for gfs_sample_detections_device_noalloc (include/stim_gb300.h).
//
// The detection path needs scratch between the frame kernel and the transpose: one uint4 per
// (128-shot block, detector or observable).  The ordinary entry points cudaMalloc it on demand.  This
// file instead holds a file-scope __device__ array of kNoAllocScratchBytes that the allocation-free
// entry point reuses for every call.  Every device that loads this module holds the array until the
// process exits.
//
// Host code must not use `g_noalloc_scratch` itself as a pointer: on the host the name is a stand-in
// symbol, not a device address.  The device address is obtained once per device, with that device
// current, through cudaGetSymbolAddress, and cached here.
#include <cuda_runtime.h>

#include <mutex>

#include "noalloc.h"

namespace gfs {

static __device__ __align__(256) uint4 g_noalloc_scratch[kNoAllocScratchBytes / sizeof(uint4)];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu[kMaxDevices];
std::mutex g_table_mu;
void *g_addr[kMaxDevices] = {};
}  // namespace

std::mutex &noalloc_device_lock(int device) {
    return g_mu[(device >= 0 && device < kMaxDevices) ? device : 0];
}

cudaError_t noalloc_scratch_address(int device, void **out) {
    if (device < 0 || device >= kMaxDevices) {
        return cudaErrorInvalidDevice;
    }
    std::lock_guard<std::mutex> lock(g_table_mu);
    if (!g_addr[device]) {
        int current = -1;
        cudaError_t e = cudaGetDevice(&current);
        if (e != cudaSuccess) {
            return e;
        }
        if (current != device) {
            return cudaErrorInvalidDevice;  // the caller must make `device` current first
        }
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            return e;
        }
        g_addr[device] = p;
    }
    *out = g_addr[device];
    return cudaSuccess;
}

}  // namespace gfs
