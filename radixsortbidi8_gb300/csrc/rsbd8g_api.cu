// rsbd8g_api.cu - host side of the C ABI declared in include/rsbd8g.h.
//
// Mode resolution restates helper::isabsvalue / issignmode / isfltpmode / isdescsort /
// isrevorderwithindirection / isrevorderwithoutindirection (Radixsortbidi8.hpp:59778-59904);
// the call sequence per sort is
//   memset(control, histograms, look-back state) -> histogram (or gather+histogram)
//   -> plan (scan + pass-skip + ping-pong) -> one onesweep pass per digit -> copy step,
// all on the caller's stream, with no host synchronisation in between (a skipped pass
// returns at once on the device), so the sequence can be captured in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "rsbd8g.h"
#include "rsbd8g_internal.h"
#include "rsbd8g_device.cuh"

namespace rsbd8g {

namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }
constexpr uint64_t kMaxCount = uint64_t(1) << 40;
constexpr uint64_t kNarrowStatusLimit = uint64_t(1) << 30;  // 30-bit look-back counts below this

}  // namespace

int device_sms(int dev) {
    static int cache[64] = {0};
    if (dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 152;
    }
    return cache[dev];
}

// ---- launch profiling -----------------------------------------------------------------------

namespace {
struct ProfRec {
    rsbd8g_launch_record r;
    cudaEvent_t a, b;
};
struct ProfState {
    std::mutex mu;
    bool on = false;
    std::vector<ProfRec> recs;
    std::vector<cudaEvent_t> pool;
};
ProfState &prof() {
    static ProfState p;
    return p;
}
cudaEvent_t prof_event() {
    ProfState &p = prof();
    if (!p.pool.empty()) {
        cudaEvent_t e = p.pool.back();
        p.pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

LaunchTimer::LaunchTimer(cudaStream_t s, uint32_t kernel, uint32_t key_bytes, uint32_t pass, uint64_t n)
    : s_(s), a_(nullptr), b_(nullptr) {
    ProfState &p = prof();
    bool on;
    {
        std::lock_guard<std::mutex> g(p.mu);
        on = p.on;
    }
    if (!on) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (cs != cudaStreamCaptureStatusNone) return;
    {
        std::lock_guard<std::mutex> g(p.mu);
        a_ = prof_event();
        b_ = prof_event();
    }
    rec_ = rsbd8g_launch_record{};
    rec_.kernel = kernel;
    rec_.key_bytes = key_bytes;
    rec_.pass = pass;
    rec_.count = n;
    cudaEventRecord(a_, s);
}

LaunchTimer::~LaunchTimer() {
    if (!a_) return;
    cudaEventRecord(b_, s_);
    ProfState &p = prof();
    std::lock_guard<std::mutex> g(p.mu);
    ProfRec pr{};
    pr.r = rec_;
    pr.a = a_;
    pr.b = b_;
    p.recs.push_back(pr);
}

rsbd8g_status profile_enable(int enable) {
    std::lock_guard<std::mutex> g(prof().mu);
    prof().on = enable != 0;
    return RSBD8G_OK;
}

rsbd8g_status profile_collect(rsbd8g_launch_record *out, size_t cap, size_t *count) {
    ProfState &p = prof();
    std::lock_guard<std::mutex> g(p.mu);
    if (count) *count = p.recs.size();
    rsbd8g_status st = RSBD8G_OK;
    for (size_t i = 0; i < p.recs.size(); ++i) {
        ProfRec &pr = p.recs[i];
        float ms = 0.f;
        if (cudaEventSynchronize(pr.b) != cudaSuccess || cudaEventElapsedTime(&ms, pr.a, pr.b) != cudaSuccess)
            st = RSBD8G_ERR_CUDA;
        pr.r.ms = ms;
        if (out && i < cap) out[i] = pr.r;
        p.pool.push_back(pr.a);
        p.pool.push_back(pr.b);
    }
    p.recs.clear();
    return st;
}

rsbd8g_status resolve(const rsbd8g_desc *d, Resolved *r) {
    if (!d || !r) return RSBD8G_ERR_BAD_ARG;
    const uint32_t kb = d->key_bytes;
    if (kb != 1 && kb != 2 && kb != 4 && kb != 8 && kb != 16) return RSBD8G_ERR_BAD_ARG;
    if (d->key_kind > RSBD8G_KIND_X87) return RSBD8G_ERR_BAD_ARG;
    if (d->key_kind == RSBD8G_KIND_FLOAT && kb < 4) return RSBD8G_ERR_BAD_ARG;
    if (d->key_kind == RSBD8G_KIND_X87 && kb != 16) return RSBD8G_ERR_BAD_ARG;
    const uint32_t mode = d->mode, dir = d->direction;
    if (!(mode < 8u || (mode >= 64u && mode <= 66u))) return RSBD8G_ERR_BAD_ARG;
    if (dir > 3u) return RSBD8G_ERR_BAD_ARG;
    if (d->indirection > RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    const bool is_float = d->key_kind == RSBD8G_KIND_FLOAT || d->key_kind == RSBD8G_KIND_X87;
    const bool is_signed = d->key_kind == RSBD8G_KIND_SIGNED || is_float;
    Filter f;
    f.absv = (mode >= 65u && is_signed) || (mode < 64u && (mode & 1u));
    f.sign = (mode >= 64u && mode <= 65u && is_signed) || (mode < 64u && (mode & 2u));
    f.fltp = (mode >= 64u && is_float) || (mode < 64u && (mode & 4u));
    f.desc = dir & 1u;
    r->f = f;
    r->indirect = d->indirection;
    r->rev = d->indirection ? ((dir >> 1) & 1u)
                            : (((dir >> 1) & 1u) && ((f.absv && f.sign) || (!f.absv && f.sign && f.fltp)));
    r->key_bytes = d->key_bytes;
    r->x87 = d->key_kind == RSBD8G_KIND_X87;
    r->digits = r->x87 ? 10u : d->key_bytes;
    r->elem_bytes = d->indirection ? 8u : d->key_bytes;
    r->off1 = d->offset1;
    r->off2 = d->offset2;
    r->flags = d->flags;
    r->prefetch = 0;
    r->keys = nullptr;
    return RSBD8G_OK;
}

Layout layout_for(const Resolved &r, uint64_t n) {
    Layout L{};
    L.wide_status = n >= kNarrowStatusLimit;
    L.large_tiles = !r.indirect && r.key_bytes <= 4 && n >= kLargeTileMinKeys && !L.wide_status;
    L.small_tiles = !r.indirect && r.key_bytes <= 4 && n < kSmallTileMaxKeys;
    const SweepGeometry g = L.large_tiles   ? sweep_geometry_large(int(r.key_bytes))
                            : L.small_tiles ? sweep_geometry_small(int(r.key_bytes))
                                            : sweep_geometry(int(r.key_bytes), r.indirect != 0);
    const int tile = g.threads * g.items;
    L.num_tiles = uint32_t((n + tile - 1) / tile);
    const size_t sw = L.wide_status ? 8 : 4;
    const uint32_t passes = r.digits;
    L.ctrl = 0;
    L.ghist = align_up(sizeof(Control));
    L.bstart = L.ghist + align_up(size_t(kMaxPasses) * kBuckets * 8);
    L.status = L.bstart + align_up(size_t(kMaxPasses) * kBuckets * 8);
    L.status_pass_bytes = align_up(size_t(L.num_tiles) * kBuckets * sw);
    L.zero_bytes = L.status + size_t(passes) * L.status_pass_bytes;
    L.keys_a = L.zero_bytes;
    const size_t kb = r.indirect ? align_up(size_t(n) * r.key_bytes) : 0;
    L.keys_b = L.keys_a + kb;
    L.total = L.keys_b + kb;
    return L;
}

int filter_class(const rsbd8g_desc *d) {
    Resolved r;
    if (resolve(d, &r) != RSBD8G_OK) return -1;
    return int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2) | (r.x87 << 3));
}

bool device_memory(const void *p) {
    if (!p) return true;                  // an absent array takes no part
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();         // not a pointer CUDA accepts: reset the (non-sticky) error
        return false;
    }
    return at.type == cudaMemoryTypeDevice;
}

rsbd8g_status enqueue_sort(const Resolved &rin, uint64_t n, void *scratch, size_t scratch_bytes, const void *in,
                           void *out, void *buf, bool inplace, bool to_buffer, cudaStream_t s) {
    // the scatter passes prefetch tiles into L2 with bulk copies only from device memory
    // (cudaMalloc, memory pools); managed and host memory is read with plain loads alone
    Resolved r = rin;
    r.prefetch = (r.flags & RSBD8G_FLAG_DEVICE_ARRAYS) ||
                 (device_memory(in) && device_memory(out) && device_memory(buf) &&
                  (!r.indirect || device_memory(scratch)));
    if (n > kMaxCount) return RSBD8G_ERR_TOO_LARGE;
    const Layout L = layout_for(r, n);
    if (!scratch || scratch_bytes < L.total) return RSBD8G_ERR_BAD_ARG;
    if ((reinterpret_cast<uintptr_t>(scratch) & (kAlign - 1)) != 0) return RSBD8G_ERR_BAD_ARG;
    unsigned char *sc = static_cast<unsigned char *>(scratch);
    if (r.key_bytes == 16 && !r.indirect) {   // 16-byte keys move as aligned 16-byte words
        auto mis = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; };
        if (mis(in) || (out && mis(out)) || (buf && mis(buf))) return RSBD8G_ERR_BAD_ARG;
    }
    cudaError_t e;
    switch (r.key_bytes) {
        case 1: e = launch_sort_k1(r, n, L, sc, in, out, buf, inplace, to_buffer, s); break;
        case 2: e = launch_sort_k2(r, n, L, sc, in, out, buf, inplace, to_buffer, s); break;
        case 4: e = launch_sort_k4(r, n, L, sc, in, out, buf, inplace, to_buffer, s); break;
        case 8: e = launch_sort_k8(r, n, L, sc, in, out, buf, inplace, to_buffer, s); break;
        default:
            e = r.x87 ? launch_sort_x87(r, n, L, sc, in, out, buf, inplace, to_buffer, s)
                      : launch_sort_k16(r, n, L, sc, in, out, buf, inplace, to_buffer, s);
            break;
    }
    return e == cudaSuccess ? RSBD8G_OK : RSBD8G_ERR_CUDA;
}

rsbd8g_status read_device_status(void *scratch, cudaStream_t s, bool clear) {
    if (!scratch) return RSBD8G_ERR_BAD_ARG;
    uint32_t err = 0;
    Control *ctrl = static_cast<Control *>(scratch);
    if (cudaMemcpyAsync(&err, &ctrl->error, sizeof err, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return RSBD8G_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RSBD8G_ERR_CUDA;
    if (clear && err) {
        if (cudaMemsetAsync(&ctrl->error, 0, sizeof err, s) != cudaSuccess) return RSBD8G_ERR_CUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return RSBD8G_ERR_CUDA;
    }
    if (err & kDevTimeout) return RSBD8G_ERR_TIMEOUT;
    if (err & kDevFault) return RSBD8G_ERR_DEVICE_FAULT;
    return RSBD8G_OK;
}

}  // namespace rsbd8g

// an empty kernel of this library's module: its attributes give the architecture the module was
// compiled for (cudaFuncAttributes::binaryVersion)
static __global__ void k_binary_probe() {}

// ---- the C ABI --------------------------------------------------------------------------------

using namespace rsbd8g;

extern "C" {

RSBD8G_API int rsbd8g_version(void) { return 200; }

RSBD8G_API rsbd8g_status rsbd8g_binary_version(int *version) {
    if (!version) return RSBD8G_ERR_BAD_ARG;
    cudaFuncAttributes at{};
    if (cudaFuncGetAttributes(&at, k_binary_probe) != cudaSuccess) {
        (void)cudaGetLastError();
        return RSBD8G_ERR_CUDA;
    }
    *version = at.binaryVersion;
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_prepare(const rsbd8g_desc *desc) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    cudaError_t e;
    switch (r.key_bytes) {
        case 1: e = launch_sort_k1_prepare(r); break;
        case 2: e = launch_sort_k2_prepare(r); break;
        case 4: e = launch_sort_k4_prepare(r); break;
        case 8: e = launch_sort_k8_prepare(r); break;
        default: e = r.x87 ? launch_sort_x87_prepare(r) : launch_sort_k16_prepare(r); break;
    }
    if (e == cudaSuccess && r.indirect == RSBD8G_DIRECT && !r.x87) e = prepare_segmented(r);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return RSBD8G_ERR_CUDA;
    }
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_profile_enable(int enable) { return profile_enable(enable); }

RSBD8G_API rsbd8g_status rsbd8g_profile_collect(rsbd8g_launch_record *records, size_t capacity, size_t *count) {
    return profile_collect(records, capacity, count);
}

RSBD8G_API const char *rsbd8g_status_string(rsbd8g_status st) {
    switch (st) {
        case RSBD8G_OK: return "ok";
        case RSBD8G_ERR_BAD_ARG: return "bad argument";
        case RSBD8G_ERR_NO_MEMORY: return "device allocation failed";
        case RSBD8G_ERR_CUDA: return "CUDA runtime error";
        case RSBD8G_ERR_TIMEOUT: return "device-side wait timed out";
        case RSBD8G_ERR_DEVICE_FAULT: return "device-side fault flag";
        case RSBD8G_ERR_TOO_LARGE: return "count too large";
        case RSBD8G_ERR_BUSY: return "admission refused: memory budget exhausted";
    }
    return "unknown status";
}

RSBD8G_API rsbd8g_status rsbd8g_scratch_bytes(const rsbd8g_desc *desc, size_t count, size_t *bytes) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (!bytes) return RSBD8G_ERR_BAD_ARG;
    if (count > kMaxCount) return RSBD8G_ERR_TOO_LARGE;
    *bytes = layout_for(r, count).total;
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortcopynoalloc(const rsbd8g_desc *desc, size_t count, void *scratch,
                                                     size_t scratch_bytes, const void *input, void *output,
                                                     void *buffer, rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect == RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    if (count == 0) return RSBD8G_OK;
    if (!input || !output) return RSBD8G_ERR_BAD_ARG;
    if (input == output) return RSBD8G_ERR_BAD_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count == 1) {
        return cudaMemcpyAsync(output, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? RSBD8G_OK : RSBD8G_ERR_CUDA;
    }
    if (!buffer || buffer == input || buffer == output) return RSBD8G_ERR_BAD_ARG;
    return enqueue_sort(r, count, scratch, scratch_bytes, input, output, buffer, false, false, s);
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortnoalloc(const rsbd8g_desc *desc, size_t count, void *scratch,
                                                 size_t scratch_bytes, void *input, void *buffer, int movetobuffer,
                                                 rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect == RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    if (count == 0) return RSBD8G_OK;
    if (!input) return RSBD8G_ERR_BAD_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count == 1) {
        if (!movetobuffer) return RSBD8G_OK;
        if (!buffer) return RSBD8G_ERR_BAD_ARG;
        return cudaMemcpyAsync(buffer, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? RSBD8G_OK : RSBD8G_ERR_CUDA;
    }
    if (!buffer || buffer == input) return RSBD8G_ERR_BAD_ARG;
    return enqueue_sort(r, count, scratch, scratch_bytes, input, nullptr, buffer, true, movetobuffer != 0, s);
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortcopynoalloc_keyed(const rsbd8g_desc *desc, size_t count, const void *keys,
                                                           void *scratch, size_t scratch_bytes, const void *input,
                                                           void *output, void *buffer, rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    r.keys = keys;
    if (count == 0) return RSBD8G_OK;
    if (!input || !output || input == output) return RSBD8G_ERR_BAD_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count == 1) {
        return cudaMemcpyAsync(output, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? RSBD8G_OK : RSBD8G_ERR_CUDA;
    }
    if (!keys || !buffer || buffer == input || buffer == output) return RSBD8G_ERR_BAD_ARG;
    return enqueue_sort(r, count, scratch, scratch_bytes, input, output, buffer, false, false, s);
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortnoalloc_keyed(const rsbd8g_desc *desc, size_t count, const void *keys,
                                                       void *scratch, size_t scratch_bytes, void *input, void *buffer,
                                                       int movetobuffer, rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    r.keys = keys;
    if (count == 0) return RSBD8G_OK;
    if (!input) return RSBD8G_ERR_BAD_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count == 1) {
        if (!movetobuffer) return RSBD8G_OK;
        if (!buffer) return RSBD8G_ERR_BAD_ARG;
        return cudaMemcpyAsync(buffer, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? RSBD8G_OK : RSBD8G_ERR_CUDA;
    }
    if (!keys || !buffer || buffer == input) return RSBD8G_ERR_BAD_ARG;
    return enqueue_sort(r, count, scratch, scratch_bytes, input, nullptr, buffer, true, movetobuffer != 0, s);
}

RSBD8G_API rsbd8g_status rsbd8g_scratch_status(void *scratch, rsbd8g_stream stream) {
    return read_device_status(scratch, reinterpret_cast<cudaStream_t>(stream), true);
}

// The allocating forms draw buffer + scratch from a library-owned stream-ordered pool per device
// that keeps up to kPoolKeepBytes of freed memory mapped, so back-to-back sorts do not map (and
// the CUDA driver does not unmap) hundreds of megabytes on every call; the process-wide default pool
// is left as the application configured it.
constexpr uint64_t kPoolKeepBytes = uint64_t(8) << 30;

static cudaMemPool_t sort_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    static std::once_flag once[64];
    static cudaMemPool_t pools[64];
    std::call_once(once[dev & 63], [&] {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) == cudaSuccess) {
            uint64_t keep = kPoolKeepBytes;
            cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
            pools[dev & 63] = p;
        } else {
            cudaGetLastError();
        }
    });
    return pools[dev & 63];
}

// allocating forms: one stream-ordered allocation of buffer + scratch, freed on the stream;
// the call waits for the sort, as the reference's functions return only when sorted
static rsbd8g_status sort_alloc(const rsbd8g_desc *desc, size_t count, const void *input, void *output, bool inplace,
                                rsbd8g_stream stream, const void *keys) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    r.keys = keys;
    if (count > kMaxCount) return RSBD8G_ERR_TOO_LARGE;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (count <= 1) {
        if (!inplace && count == 1) {
            if (!input || !output || input == output) return RSBD8G_ERR_BAD_ARG;
            if (cudaMemcpyAsync(output, input, r.elem_bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                return RSBD8G_ERR_CUDA;
            return cudaStreamSynchronize(s) == cudaSuccess ? RSBD8G_OK : RSBD8G_ERR_CUDA;
        }
        return RSBD8G_OK;
    }
    if (!input || (!inplace && (!output || input == output))) return RSBD8G_ERR_BAD_ARG;
    const Layout L = layout_for(r, count);
    const size_t buf_bytes = (size_t(count) * r.elem_bytes + 255) & ~size_t(255);
    void *mem = nullptr;
    if (r.flags & RSBD8G_FLAG_DIAG_NOMEM) return RSBD8G_ERR_NO_MEMORY;
    cudaMemPool_t pool = sort_pool();
    const cudaError_t ae = pool ? cudaMallocFromPoolAsync(&mem, L.total + buf_bytes, pool, s)
                                : cudaMallocAsync(&mem, L.total + buf_bytes, s);
    if (ae != cudaSuccess || !mem) {
        cudaGetLastError();
        return RSBD8G_ERR_NO_MEMORY;
    }
    unsigned char *scratch = static_cast<unsigned char *>(mem);
    void *buffer = scratch + L.total;
    st = enqueue_sort(r, count, scratch, L.total, input, inplace ? nullptr : output, buffer, inplace, false, s);
    rsbd8g_status dev = RSBD8G_OK;
    if (st == RSBD8G_OK) dev = read_device_status(scratch, s, false);
    cudaFreeAsync(mem, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && st == RSBD8G_OK) st = RSBD8G_ERR_CUDA;
    return st != RSBD8G_OK ? st : dev;
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy(const rsbd8g_desc *desc, size_t count, const void *input, void *output,
                                              rsbd8g_stream stream) {
    if (desc && desc->indirection == RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    return sort_alloc(desc, count, input, output, false, stream, nullptr);
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy_keyed(const rsbd8g_desc *desc, size_t count, const void *keys,
                                                    const void *input, void *output, rsbd8g_stream stream) {
    if (!desc || desc->indirection != RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    if (count > 1 && !keys) return RSBD8G_ERR_BAD_ARG;
    return sort_alloc(desc, count, input, output, false, stream, keys);
}

RSBD8G_API rsbd8g_status rsbd8g_radixsort(const rsbd8g_desc *desc, size_t count, void *input, rsbd8g_stream stream) {
    if (desc && desc->indirection == RSBD8G_KEYED) return RSBD8G_ERR_BAD_ARG;
    return sort_alloc(desc, count, input, nullptr, true, stream, nullptr);
}

}  // extern "C"
