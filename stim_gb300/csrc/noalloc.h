// Fixed device scratch of the allocation-free detection entry point (noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

namespace gfs {

// Size of the file-scope device scratch array (per device, held until process exit).
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;

// Device address of the scratch array on `device`, which must be the current device.  The first call per
// device looks the address up with cudaGetSymbolAddress; later calls return the cached address.
cudaError_t noalloc_scratch_address(int device, void **out);

// Serializes users of one device's scratch array within this process.
std::mutex &noalloc_device_lock(int device);

}  // namespace gfs
