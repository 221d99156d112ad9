// Static device scratch of rtmc_forward_noalloc.
//
// A file-scope __device__ array of RTMC_STATIC_SCRATCH_BYTES.  Every GPU on which the
// library's module is loaded holds it until the process exits.  In host code the name
// g_static_scratch is only a host-side stand-in, not a device address; the device
// address is obtained once per device with cudaGetSymbolAddress (the device must be
// current) and handed to the kernels as a plain pointer.
#include "rtmc_internal.h"

#include <cuda_runtime.h>

#include <mutex>

namespace rtmc {
namespace {

__device__ __align__(256) unsigned char g_static_scratch[RTMC_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

} // namespace

int static_scratch(int device, unsigned char **ptr, size_t *bytes)
{
    if (device < 0 || device >= kMaxDevices) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return (int)e;
        g_addr[device] = p;
    }
    *ptr = static_cast<unsigned char *>(g_addr[device]);
    *bytes = (size_t)RTMC_STATIC_SCRATCH_BYTES;
    return 0;
}

} // namespace rtmc
