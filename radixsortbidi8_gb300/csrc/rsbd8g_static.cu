// rsbd8g_static.cu - rsbd8g_radixsortcopy_static: the plain-key copy sort with its scratch (look-back
// state, histograms, control block) and its ping-pong buffer carved out of one file-scope device
// array, so the call allocates no device memory at all.
//
// Who needs it: code that is not allowed to call cudaMalloc -- a plugin whose host framework owns
// every byte of device memory through its own allocator or a fixed budget, a latency-critical path
// that cannot afford cudaMalloc's implicit device-wide synchronisation, or a caller that is only
// handed an input and an output buffer.
//
// The array below exists once per GPU that loads this library and stays allocated until the
// process exits.  In host code its name is only a host-side stand-in; the real device address is
// looked up with cudaGetSymbolAddress, once per device, by the first call made on that device.
#include <cuda_runtime.h>

#include <mutex>

#include "rsbd8g.h"
#include "rsbd8g_internal.h"

namespace rsbd8g {
namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;   // 64 MiB per device

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

struct StaticScratchAddress {
    std::once_flag once;
    void *ptr = nullptr;
    cudaError_t err = cudaSuccess;
};
StaticScratchAddress g_static_address[64];

}  // namespace
}  // namespace rsbd8g

using namespace rsbd8g;

extern "C" RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy_static(const rsbd8g_desc *desc, size_t count,
                                                                 const void *input, void *output,
                                                                 rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_DIRECT) return RSBD8G_ERR_BAD_ARG;
    if (count == 0) return RSBD8G_OK;
    if (!input || !output || input == output) return RSBD8G_ERR_BAD_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count == 1) {
        return cudaMemcpyAsync(output, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? RSBD8G_OK : RSBD8G_ERR_CUDA;
    }
    // scratch first, then the ping-pong buffer; both must fit the array
    if (count > (kStaticScratchBytes / r.elem_bytes)) return RSBD8G_ERR_TOO_LARGE;
    const Layout L = layout_for(r, count);
    const size_t buffer_bytes = (size_t(count) * r.elem_bytes + 255) & ~size_t(255);
    if (L.total + buffer_bytes > kStaticScratchBytes) return RSBD8G_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RSBD8G_ERR_CUDA;
    StaticScratchAddress &a = g_static_address[dev];
    std::call_once(a.once, [&a] { a.err = cudaGetSymbolAddress(&a.ptr, g_static_scratch); });
    if (a.err != cudaSuccess || !a.ptr) return RSBD8G_ERR_CUDA;
    unsigned char *scratch = static_cast<unsigned char *>(a.ptr);
    return enqueue_sort(r, count, scratch, L.total, input, output, scratch + L.total, false, false, s);
}
