// rsbd8g_seglaunch.cuh - launch sequence of the batched (segmented) sort for one key size:
//   memset(control, histograms) -> classify -> small-segment block sort -> large-segment
//   histograms -> per-segment plan -> per pass: memset(look-back words) + segmented onesweep
//   -> copy of fully skipped large segments
// all stream-ordered without host synchronisation, so one CUDA graph can replay a whole batch.
#pragma once
#include <algorithm>
#include <mutex>

#include "rsbd8g_internal.h"
#include "rsbd8g_segmented.cuh"

namespace rsbd8g {

// one-time setup (which also loads the kernel) of the small-segment kernel on device `dev`: its
// resident CTAs per SM (see SweepKernels in rsbd8g_launch.cuh)
template <typename U, int MODE, int THREADS, int ITEMS>
int small_setup(int dev) {
    using SM = SmallSmem<U, THREADS, ITEMS>;
    static std::once_flag once[64];
    static int occ[64];
    std::call_once(once[dev & 63], [&] {
        auto kern = k_seg_small<U, MODE, THREADS, ITEMS>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SM::kBytes));
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, THREADS, SM::kBytes);
        occ[dev & 63] = b > 0 ? b : 1;
    });
    return occ[dev & 63];
}

template <typename U, int MODE, int THREADS, int ITEMS>
cudaError_t launch_small_t(const SegArgs &a, const U *in, U *out, cudaStream_t s) {
    using SM = SmallSmem<U, THREADS, ITEMS>;
    auto kern = k_seg_small<U, MODE, THREADS, ITEMS>;
    int dev = 0;
    cudaGetDevice(&dev);
    const int occ = small_setup<U, MODE, THREADS, ITEMS>(dev);
    const uint32_t grid = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(a.nsegs, uint64_t(occ) * device_sms(dev))));
    LaunchTimer t(s, RSBD8G_KERNEL_SEGMENTED, uint32_t(sizeof(U)), 100, a.nsegs);
    kern<<<grid, THREADS, SM::kBytes, s>>>(a, in, out);
    return cudaGetLastError();
}

// one-time setup of the segmented scatter kernels (see SweepKernels in rsbd8g_launch.cuh)
template <typename U, int MODE, int THREADS, int ITEMS>
struct SegSweepKernels {
    using SM = OnesweepSmem<U, false, THREADS, ITEMS>;
    using PM = PipeSmem<U, THREADS, ITEMS>;
    static void setup(int dev, int *occ_out, int *pocc_out) {
        static std::once_flag once[64];
        static int occ[64], pocc[64];
        std::call_once(once[dev & 63], [&] {
            auto kern = k_seg_sweep<U, MODE, THREADS, ITEMS>;
            auto pkern = k_seg_sweep_pipe<U, MODE, THREADS, ITEMS>;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SM::kBytes));
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            int b = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, THREADS, SM::kBytes);
            occ[dev & 63] = b > 0 ? b : 1;
            cudaFuncSetAttribute(pkern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(PM::kBytes));
            cudaFuncSetAttribute(pkern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            int pb = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pb, pkern, THREADS, PM::kBytes);
            pocc[dev & 63] = pb > 0 ? pb : 1;
        });
        if (occ_out) *occ_out = occ[dev & 63];
        if (pocc_out) *pocc_out = pocc[dev & 63];
    }
};

// one-time setup of the large-segment histogram kernel
template <typename U, int MODE>
void seg_hist_setup(int dev) {
    constexpr int P = KeyTraits<U>::kDigits;
    constexpr size_t smem = size_t(hist_lane_copies<P>()) * P * kBuckets * 4;
    static std::once_flag once[64];
    std::call_once(once[dev & 63], [&] {
        cudaFuncSetAttribute(k_seg_hist<U, MODE, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    });
}

template <typename U, int MODE, int THREADS, int ITEMS>
cudaError_t launch_seg_sweeps_t(const SegArgs &a, const SegLayout &L, unsigned char *scratch, const U *in, U *out,
                                U *buf, uint32_t stall_tile, cudaStream_t s) {
    // the pipelined pass when the batch has tiles enough to fill it (tiles_max bounds the large tiles)
    using K = SegSweepKernels<U, MODE, THREADS, ITEMS>;
    using SM = typename K::SM;
    using PM = typename K::PM;
    auto kern = k_seg_sweep<U, MODE, THREADS, ITEMS>;
    auto pkern = k_seg_sweep_pipe<U, MODE, THREADS, ITEMS>;
    int dev = 0;
    cudaGetDevice(&dev);
    int occ = 1, pocc = 1;
    K::setup(dev, &occ, &pocc);
    const uint64_t president = uint64_t(pocc) * device_sms(dev);
    const bool pipe = uint64_t(L.tiles_max) >= 2 * president;
    const uint64_t resident = pipe ? president : uint64_t(occ) * device_sms(dev);
    const uint32_t grid = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(L.tiles_max, resident)));
    uint32_t *status = reinterpret_cast<uint32_t *>(scratch + L.status);
    for (int p = 0; p < KeyTraits<U>::kDigits; ++p) {
        cudaError_t e;
        {
            LaunchTimer t(s, RSBD8G_KERNEL_MEMSET, uint32_t(sizeof(U)), uint32_t(p), L.tiles_max);
            e = cudaMemsetAsync(status, 0, L.status_bytes, s);
        }
        if (e != cudaSuccess) return e;
        LaunchTimer t(s, RSBD8G_KERNEL_SEGMENTED, uint32_t(sizeof(U)), uint32_t(p), L.tiles_max);
        if (pipe)
            pkern<<<grid, THREADS, PM::kBytes, s>>>(a, p, KeyTraits<U>::kDigits, in, out, buf, status, stall_tile);
        else
            kern<<<grid, THREADS, SM::kBytes, s>>>(a, p, KeyTraits<U>::kDigits, in, out, buf, status, stall_tile);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename U, int MODE>
cudaError_t launch_segmented_mode_t(const Resolved &r, const SegArgs &a, const SegLayout &L, unsigned char *scratch,
                                    const void *in_, void *out_, void *buf_, cudaStream_t s) {
    const U *in = static_cast<const U *>(in_);
    U *out = static_cast<U *>(out_);
    U *buf = static_cast<U *>(buf_);
    cudaError_t e;
    int dev = 0;
    cudaGetDevice(&dev);
    const int sms = device_sms(dev);
    {
        LaunchTimer t(s, RSBD8G_KERNEL_SEGMENTED, uint32_t(sizeof(U)), 200, a.nsegs);
        k_seg_classify<<<1, 1024, 0, s>>>(a);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    constexpr SegSmallShape sh0 = seg_small_shape(int(sizeof(U)), 0), sh1 = seg_small_shape(int(sizeof(U)), 1),
                            sh2 = seg_small_shape(int(sizeof(U)), 2);
    switch (L.small_variant) {
        case 0: e = launch_small_t<U, MODE, sh0.threads, sh0.items>(a, in, out, s); break;
        case 1: e = launch_small_t<U, MODE, sh1.threads, sh1.items>(a, in, out, s); break;
        default: e = launch_small_t<U, MODE, sh2.threads, sh2.items>(a, in, out, s); break;
    }
    if (e != cudaSuccess) return e;
    {
        LaunchTimer t(s, RSBD8G_KERNEL_HISTOGRAM, uint32_t(sizeof(U)), 0, a.nsegs);
        constexpr int P = KeyTraits<U>::kDigits;
        constexpr size_t smem = size_t(hist_lane_copies<P>()) * P * kBuckets * 4;
        auto kern = k_seg_hist<U, MODE, 1024>;
        seg_hist_setup<U, MODE>(dev);
        kern<<<uint32_t(sms), 1024, smem, s>>>(a, in);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    {
        LaunchTimer t(s, RSBD8G_KERNEL_PLAN, uint32_t(sizeof(U)), 0, a.nsegs);
        const uint32_t g = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(a.nlarge_max, uint64_t(sms) * 16)));
        k_seg_plan<<<g, 256, 0, s>>>(a, KeyTraits<U>::kDigits);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    constexpr SweepGeometry g0 = seg_sweep_geometry(int(sizeof(U)), 0), g1 = seg_sweep_geometry(int(sizeof(U)), 1);
    const uint32_t stall = (r.flags & RSBD8G_FLAG_DIAG_STALL) ? 1u : 0xFFFFFFFFu;
    if (L.large_variant == 1 && g1.items != g0.items)
        e = launch_seg_sweeps_t<U, MODE, g1.threads, g1.items>(a, L, scratch, in, out, buf, stall, s);
    else
        e = launch_seg_sweeps_t<U, MODE, g0.threads, g0.items>(a, L, scratch, in, out, buf, stall, s);
    if (e != cudaSuccess) return e;
    {
        LaunchTimer t(s, RSBD8G_KERNEL_COPY, uint32_t(sizeof(U)), 0, a.nsegs);
        k_seg_copy<U><<<uint32_t(sms) * 4, 256, 0, s>>>(a, in, out);
    }
    return cudaGetLastError();
}

template <typename U>
cudaError_t launch_segmented_t(const Resolved &r, const SegArgs &a, const SegLayout &L, unsigned char *scratch,
                               const void *in, void *out, void *buf, cudaStream_t s) {
    const int mode = int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2));
    cudaError_t e;
#define RSBD8G_SEG(M) e = launch_segmented_mode_t<U, M>(r, a, L, scratch, in, out, buf, s)
    RSBD8G_MODE_SWITCH(mode, RSBD8G_SEG)
#undef RSBD8G_SEG
    return e;
}

// load and set up every kernel a segmented sort with filter MODE can launch
template <typename U, int MODE>
cudaError_t prepare_segmented_mode_t(int dev) {
    constexpr SegSmallShape sh0 = seg_small_shape(int(sizeof(U)), 0), sh1 = seg_small_shape(int(sizeof(U)), 1),
                            sh2 = seg_small_shape(int(sizeof(U)), 2);
    constexpr SweepGeometry g0 = seg_sweep_geometry(int(sizeof(U)), 0), g1 = seg_sweep_geometry(int(sizeof(U)), 1);
    small_setup<U, MODE, sh0.threads, sh0.items>(dev);
    small_setup<U, MODE, sh1.threads, sh1.items>(dev);
    small_setup<U, MODE, sh2.threads, sh2.items>(dev);
    seg_hist_setup<U, MODE>(dev);
    SegSweepKernels<U, MODE, g0.threads, g0.items>::setup(dev, nullptr, nullptr);
    SegSweepKernels<U, MODE, g1.threads, g1.items>::setup(dev, nullptr, nullptr);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, k_seg_classify);
    cudaFuncGetAttributes(&fa, k_seg_plan);
    cudaFuncGetAttributes(&fa, k_seg_copy<U>);
    return cudaGetLastError();
}

template <typename U>
cudaError_t prepare_segmented_t(const Resolved &r) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int mode = int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2));
#define RSBD8G_PREP(M) e = prepare_segmented_mode_t<U, M>(dev)
    RSBD8G_MODE_SWITCH(mode, RSBD8G_PREP)
#undef RSBD8G_PREP
    return e;
}

}  // namespace rsbd8g

#define RSBD8G_DEFINE_SEG_LAUNCH(name, U)                                                                       \
    namespace rsbd8g {                                                                                          \
    cudaError_t name(const Resolved &r, const SegArgs &a, const SegLayout &L, unsigned char *scratch,          \
                     const void *in, void *out, void *buf, cudaStream_t s) {                                   \
        return launch_segmented_t<U>(r, a, L, scratch, in, out, buf, s);                                       \
    }                                                                                                           \
    cudaError_t name##_prepare(const Resolved &r) { return prepare_segmented_t<U>(r); }                        \
    }
