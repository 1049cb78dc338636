// rsbd8g_static.cu - rsbd8g_radixsortcopy_static: the plain-key copy sort with its scratch (look-back
// state, histograms, control block) and its ping-pong buffer carved out of one file-scope device
// array, so the call allocates no device memory at all; rsbd8g_static_status reads the device-side
// status word that the sort leaves in that array.
//
// Who needs it: code that is not allowed to call cudaMalloc -- a plugin whose host framework owns
// every byte of device memory through its own allocator or a fixed budget, a latency-critical path
// that cannot afford cudaMalloc's implicit device-wide synchronisation, or a caller that is only
// handed an input and an output buffer.
//
// The array below exists once per GPU that loads this library and stays allocated until the
// process exits.  In host code its name is only a host-side stand-in; the real device address is
// looked up with cudaGetSymbolAddress, once per device, by the first call made on that device (a
// failed lookup is not remembered: the next call tries again).
#include <cuda_runtime.h>

#include <mutex>

#include "rsbd8g.h"
#include "rsbd8g_internal.h"

namespace rsbd8g {
namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;   // 64 MiB per device

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void *g_static_ptr[64];   // device address of g_static_scratch per device; null until looked up

// the array's device address on the current device (looked up on first use, with that device
// current); RSBD8G_ERR_CUDA when the lookup fails
rsbd8g_status static_scratch(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        (void)cudaGetLastError();
        return RSBD8G_ERR_CUDA;
    }
    std::lock_guard<std::mutex> g(g_static_mu);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) {
            (void)cudaGetLastError();
            return RSBD8G_ERR_CUDA;
        }
        g_static_ptr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_static_ptr[dev]);
    return RSBD8G_OK;
}

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
    // scratch first, then the ping-pong buffer; both must fit the array
    if (count > (kStaticScratchBytes / r.elem_bytes)) return RSBD8G_ERR_TOO_LARGE;
    const Layout L = layout_for(r, count);
    const size_t buffer_bytes = (size_t(count) * r.elem_bytes + 255) & ~size_t(255);
    if (L.total + buffer_bytes > kStaticScratchBytes) return RSBD8G_ERR_TOO_LARGE;
    if (count == 1) {
        return cudaMemcpyAsync(output, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? RSBD8G_OK : RSBD8G_ERR_CUDA;
    }
    unsigned char *scratch = nullptr;
    if ((st = static_scratch(&scratch)) != RSBD8G_OK) return st;
    return enqueue_sort(r, count, scratch, L.total, input, output, scratch + L.total, false, false, s);
}

extern "C" RSBD8G_API rsbd8g_status rsbd8g_static_status(rsbd8g_stream stream) {
    unsigned char *scratch = nullptr;
    rsbd8g_status st = static_scratch(&scratch);
    if (st != RSBD8G_OK) return st;
    return read_device_status(scratch, reinterpret_cast<cudaStream_t>(stream), true);
}
