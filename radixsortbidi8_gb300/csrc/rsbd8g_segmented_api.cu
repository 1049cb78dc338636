// rsbd8g_segmented_api.cu - C ABI of the batched (segmented) sort declared in include/rsbd8g.h.
#include <cuda_runtime.h>

#include <algorithm>

#include "rsbd8g.h"
#include "rsbd8g_internal.h"
#include "rsbd8g_segmented.cuh"

namespace rsbd8g {
namespace {

constexpr size_t kA = 256;
constexpr size_t up(size_t x) { return (x + kA - 1) & ~(kA - 1); }

rsbd8g_status seg_layout(const Resolved &r, uint64_t total, uint64_t nsegs, const rsbd8g_segtuning *t,
                         SegLayout *L) {
    *L = SegLayout{};
    const uint32_t variant = t ? t->small_variant : 1u;
    if (variant >= uint32_t(kSegSmallVariants)) return RSBD8G_ERR_BAD_ARG;
    const SegSmallShape sh = seg_small_shape(int(r.key_bytes), int(variant));
    const uint32_t cap = uint32_t(sh.threads * sh.items);
    const uint32_t cutoff = (t && t->small_cutoff) ? t->small_cutoff : cap;
    if (cutoff > cap) return RSBD8G_ERR_BAD_ARG;
    const uint32_t lvariant = t ? t->large_variant : 0u;
    if (lvariant >= uint32_t(kSegLargeVariants)) return RSBD8G_ERR_BAD_ARG;
    const SweepGeometry g = seg_sweep_geometry(int(r.key_bytes), int(lvariant));
    L->tile = uint32_t(g.threads * g.items);
    L->cutoff = cutoff;
    L->small_variant = variant;
    L->large_variant = lvariant;
    L->nlarge_max = std::max<uint64_t>(1, std::min<uint64_t>(nsegs, total / (uint64_t(cutoff) + 1)));
    L->tiles_max = total / L->tile + L->nlarge_max + 1;
    if (L->tiles_max >= (uint64_t(1) << 32) || nsegs >= (uint64_t(1) << 32)) return RSBD8G_ERR_TOO_LARGE;
    const uint64_t P = r.digits;
    L->ctrl = 0;
    L->seg_hist = up(sizeof(SegControl));
    L->zero_bytes = L->seg_hist + up(L->nlarge_max * P * kBuckets * 4);
    L->large_seg = L->zero_bytes;
    L->large_tbase = L->large_seg + up(L->nlarge_max * 4);
    L->small_seg = L->large_tbase + up((L->nlarge_max + 1) * 4);
    L->seg_mask = L->small_seg + up(nsegs * 4);
    L->tile_seg = L->seg_mask + up(L->nlarge_max * 4);
    L->status = L->tile_seg + up(L->tiles_max * 4);
    L->status_bytes = up(L->tiles_max * kBuckets * 4);
    L->total = L->status + L->status_bytes;
    return RSBD8G_OK;
}

}  // namespace

cudaError_t prepare_segmented(const Resolved &r) {
    switch (r.key_bytes) {
        case 1: return launch_segmented_k1_prepare(r);
        case 2: return launch_segmented_k2_prepare(r);
        case 4: return launch_segmented_k4_prepare(r);
        case 8: return launch_segmented_k8_prepare(r);
        default: return launch_segmented_k16_prepare(r);
    }
}
}  // namespace rsbd8g

using namespace rsbd8g;

extern "C" {

RSBD8G_API rsbd8g_status rsbd8g_segmented_scratch_bytes(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                        const rsbd8g_segtuning *tuning, size_t *bytes) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_DIRECT || !bytes || r.x87) return RSBD8G_ERR_BAD_ARG;
    SegLayout L;
    if ((st = seg_layout(r, total, nsegs, tuning, &L)) != RSBD8G_OK) return st;
    *bytes = L.total;
    return RSBD8G_OK;
}

static rsbd8g_status segmented_common(const rsbd8g_desc *desc, size_t total, size_t nsegs, const uint64_t *offsets,
                                      void *scratch, size_t scratch_bytes, const void *input, void *output,
                                      void *buffer, const uint64_t *in_ptrs, const uint64_t *out_ptrs,
                                      const uint64_t *buf_ptrs, const uint8_t *seg_dirs, const rsbd8g_segtuning *tuning,
                                      rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_DIRECT || r.x87) return RSBD8G_ERR_BAD_ARG;
    if (nsegs == 0 || total == 0) return RSBD8G_OK;
    if (!offsets || !scratch) return RSBD8G_ERR_BAD_ARG;
    if (!in_ptrs) {
        if (!input || !output || !buffer) return RSBD8G_ERR_BAD_ARG;
        if (input == output || input == buffer || output == buffer) return RSBD8G_ERR_BAD_ARG;
    } else if (!out_ptrs || !buf_ptrs) {
        return RSBD8G_ERR_BAD_ARG;
    }
    if ((reinterpret_cast<uintptr_t>(scratch) & (kA - 1)) != 0) return RSBD8G_ERR_BAD_ARG;
    if (r.key_bytes == 16 && !in_ptrs) {      // 16-byte keys move as aligned 16-byte words
        auto mis = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; };
        if (mis(input) || mis(output) || mis(buffer)) return RSBD8G_ERR_BAD_ARG;
    }
    SegLayout L;
    if ((st = seg_layout(r, total, nsegs, tuning, &L)) != RSBD8G_OK) return st;
    if (scratch_bytes < L.total) return RSBD8G_ERR_BAD_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned char *sc = static_cast<unsigned char *>(scratch);
    cudaError_t e;
    {
        LaunchTimer t(s, RSBD8G_KERNEL_MEMSET, r.key_bytes, 0, total);
        e = cudaMemsetAsync(sc, 0, L.zero_bytes, s);
    }
    if (e != cudaSuccess) return RSBD8G_ERR_CUDA;
    SegArgs a{};
    a.offsets = offsets;
    a.total = total;
    a.nsegs = uint32_t(nsegs);
    a.cutoff = L.cutoff;
    a.tile = L.tile;
    a.rev = r.rev;
    a.dmask = r.f.desc ? 0xFFu : 0u;
    a.nlarge_max = uint32_t(L.nlarge_max);
    a.ctrl = reinterpret_cast<SegControl *>(sc + L.ctrl);
    a.large_seg = reinterpret_cast<uint32_t *>(sc + L.large_seg);
    a.large_tbase = reinterpret_cast<uint32_t *>(sc + L.large_tbase);
    a.small_seg = reinterpret_cast<uint32_t *>(sc + L.small_seg);
    a.seg_hist = reinterpret_cast<uint32_t *>(sc + L.seg_hist);
    a.seg_mask = reinterpret_cast<uint32_t *>(sc + L.seg_mask);
    a.tile_seg = reinterpret_cast<uint32_t *>(sc + L.tile_seg);
    a.ptr_in = in_ptrs;
    a.ptr_out = out_ptrs;
    a.ptr_buf = buf_ptrs;
    a.spin_limit_ns = (r.flags & RSBD8G_FLAG_DIAG_STALL) ? 200000000ull : 1000000000ull;
    // tiles are prefetched into L2 only from device memory: the contiguous form checks its three
    // arrays, the pointer-table form relies on the caller's RSBD8G_FLAG_DEVICE_ARRAYS
    a.seg_dir = seg_dirs;
    // isrevorder is honoured by the regular absolute modes and regular floating point
    // (Radixsortbidi8.hpp:59877-59904), the same for every segment of the call
    a.rev_ok = (r.f.absv && r.f.sign) || (!r.f.absv && r.f.sign && r.f.fltp);
    a.prefetch = (r.flags & RSBD8G_FLAG_DEVICE_ARRAYS) ||
                 (!in_ptrs && device_memory(input) && device_memory(output) && device_memory(buffer));
    switch (r.key_bytes) {
        case 1: e = launch_segmented_k1(r, a, L, sc, input, output, buffer, s); break;
        case 2: e = launch_segmented_k2(r, a, L, sc, input, output, buffer, s); break;
        case 4: e = launch_segmented_k4(r, a, L, sc, input, output, buffer, s); break;
        case 8: e = launch_segmented_k8(r, a, L, sc, input, output, buffer, s); break;
        default: e = launch_segmented_k16(r, a, L, sc, input, output, buffer, s); break;
    }
    return e == cudaSuccess ? RSBD8G_OK : RSBD8G_ERR_CUDA;
}

RSBD8G_API rsbd8g_status rsbd8g_segmented_sortcopy(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                   const uint64_t *offsets, void *scratch, size_t scratch_bytes,
                                                   const void *input, void *output, void *buffer,
                                                   const rsbd8g_segtuning *tuning, rsbd8g_stream stream) {
    return segmented_common(desc, total, nsegs, offsets, scratch, scratch_bytes, input, output, buffer, nullptr,
                            nullptr, nullptr, nullptr, tuning, stream);
}

RSBD8G_API rsbd8g_status rsbd8g_segmented_sortcopy_ptrs(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                        const uint64_t *offsets, const uint64_t *input_ptrs,
                                                        const uint64_t *output_ptrs, const uint64_t *buffer_ptrs,
                                                        void *scratch, size_t scratch_bytes,
                                                        const rsbd8g_segtuning *tuning, rsbd8g_stream stream) {
    return segmented_common(desc, total, nsegs, offsets, scratch, scratch_bytes, nullptr, nullptr, nullptr,
                            input_ptrs, output_ptrs, buffer_ptrs, nullptr, tuning, stream);
}

RSBD8G_API rsbd8g_status rsbd8g_segmented_sortcopy_ptrs_dirs(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                             const uint64_t *offsets, const uint64_t *input_ptrs,
                                                             const uint64_t *output_ptrs, const uint64_t *buffer_ptrs,
                                                             const uint8_t *directions, void *scratch,
                                                             size_t scratch_bytes, const rsbd8g_segtuning *tuning,
                                                             rsbd8g_stream stream) {
    if (!directions && nsegs && total) return RSBD8G_ERR_BAD_ARG;
    return segmented_common(desc, total, nsegs, offsets, scratch, scratch_bytes, nullptr, nullptr, nullptr,
                            input_ptrs, output_ptrs, buffer_ptrs, directions, tuning, stream);
}

}  // extern "C"
