// rsbd8g_launch.cuh - host-side launch sequence of one sort, templated on the key size; each
// rsbd8g_sort_k*.cu instantiates it for one key size so the kernels compile in parallel.
//
//   memset(control, histograms, look-back state) -> histogram (or gather + histogram), whose last
//   CTA to finish writes the plan (scan + pass-skip + ping-pong) -> one onesweep pass per digit,
//   the last of which also runs the copy step of the copy forms -> copy step (in-place forms only)
// all on the caller's stream, with no host synchronisation in between (a skipped pass returns at
// once on the device), so the sequence can be captured in a CUDA graph: 2 + digits launches for
// the copy forms, 3 + digits for the in-place forms.
#pragma once
#include <algorithm>
#include <mutex>

#include "rsbd8g_internal.h"
#include "rsbd8g_kernels.cuh"

namespace rsbd8g {

constexpr int kHistThreads = 512;         // gather histogram (indirect keys)
constexpr int kHistDirectThreads = 1024;  // direct keys: one CTA per SM

// The one-time setup of a kernel pair on a device: shared-memory limits and carveout, and the
// resident CTAs per SM.  Setting an attribute also loads the kernel (the CUDA runtime loads each
// kernel at its first use), so running this ahead of the first sort (rsbd8g_prepare) keeps that
// cost, which can stall the calling thread for tens of milliseconds, out of the first call.
template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S>
struct SweepKernels {
    using SM = OnesweepSmem<U, HAS_VAL, THREADS, ITEMS>;
    using PM = PipeSmem<U, THREADS, ITEMS, HAS_VAL>;
    // resident CTAs per SM of k_onesweep (occ) and k_onesweep_pipe (pocc) on device `dev`
    static void setup(int dev, int *occ_out, int *pocc_out) {
        static std::once_flag once[64];
        static int occ[64], pocc[64];
        std::call_once(once[dev & 63], [&] {
            auto kern = k_onesweep<U, MODE, HAS_VAL, THREADS, ITEMS, S>;
            auto pkern = k_onesweep_pipe<U, MODE, HAS_VAL, THREADS, ITEMS, S>;
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

template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S>
cudaError_t launch_sweeps_t(uint32_t passes, uint64_t n, const Layout &L, unsigned char *scratch,
                            const SortArrays &arrs, uint32_t dmask, bool fold_copy, cudaStream_t s) {
    // the pipelined pass, unless there are too few tiles to fill its pipeline (a sort of about one
    // tile per CTA runs each tile's phases back to back in k_onesweep instead)
    using K = SweepKernels<U, MODE, HAS_VAL, THREADS, ITEMS, S>;
    using SM = typename K::SM;
    using PM = typename K::PM;
    auto kern = k_onesweep<U, MODE, HAS_VAL, THREADS, ITEMS, S>;
    auto pkern = k_onesweep_pipe<U, MODE, HAS_VAL, THREADS, ITEMS, S>;
    int dev = 0;
    cudaGetDevice(&dev);
    int occ = 1, pocc = 1;
    K::setup(dev, &occ, &pocc);
    const uint64_t resident = uint64_t(pocc) * device_sms(dev);
    const bool pipe = uint64_t(L.num_tiles) >= 2 * resident;
    const uint32_t grid = uint32_t(std::min<uint64_t>(L.num_tiles, pipe ? resident : uint64_t(occ) * device_sms(dev)));
    Control *ctrl = reinterpret_cast<Control *>(scratch + L.ctrl);
    const unsigned long long *bstart = reinterpret_cast<const unsigned long long *>(scratch + L.bstart);
    for (uint32_t p = 0; p < passes; ++p) {
        S *status = reinterpret_cast<S *>(scratch + L.status + size_t(p) * L.status_pass_bytes);
        LaunchTimer t(s, RSBD8G_KERNEL_ONESWEEP, uint32_t(sizeof(U)), p, n);
        const uint32_t fc = (fold_copy && p + 1 == passes) ? 1u : 0u;   // the copy forms' copy, in the last pass
        if (pipe)
            pkern<<<grid, THREADS, PM::kBytes, s>>>(ctrl, arrs, bstart, status, int(p), n, L.num_tiles, dmask, fc);
        else
            kern<<<grid, THREADS, SM::kBytes, s>>>(ctrl, arrs, bstart, status, int(p), n, L.num_tiles, dmask, fc);
    }
    return cudaGetLastError();
}

// the direct-key histogram kernel's one-time setup on device `dev` (see SweepKernels)
template <typename U, int MODE>
void histogram_setup(int dev) {
    constexpr int P = KeyTraits<U>::kDigits;
    constexpr size_t smem = size_t(hist_lane_copies<P>()) * P * kBuckets * 4;
    static std::once_flag once[64];
    std::call_once(once[dev & 63], [&] {
        cudaFuncSetAttribute(k_histogram<U, MODE, kHistDirectThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem));
    });
}

template <typename U, int MODE>
cudaError_t launch_histogram_t(const Resolved &r, uint64_t n, const void *in, const Layout &L,
                               unsigned char *scratch, uint32_t dmask, const PlanArgs &pa, cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t per_cta = uint64_t(kHistThreads) * 64;   // keys per CTA sweep, to size the grid
    const uint32_t grid = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>((n + per_cta - 1) / per_cta,
                                                                            uint64_t(device_sms(dev)) * 4)));
    unsigned long long *ghist = reinterpret_cast<unsigned long long *>(scratch + L.ghist);
    Control *ctrl = reinterpret_cast<Control *>(scratch + L.ctrl);
    unsigned long long *bstart = reinterpret_cast<unsigned long long *>(scratch + L.bstart);
    LaunchTimer t(s, RSBD8G_KERNEL_HISTOGRAM, uint32_t(sizeof(U)), 0, n);
    if (r.indirect) {
        k_gather_histogram<U, MODE, kHistThreads><<<grid, kHistThreads, 0, s>>>(
            static_cast<const uint64_t *>(in), n, dmask, r.off1, r.off2, int(r.indirect),
            static_cast<const U *>(r.keys), reinterpret_cast<U *>(scratch + L.keys_a), ghist, ctrl, bstart, pa);
    } else {
        constexpr int P = KeyTraits<U>::kDigits;
        constexpr size_t smem = size_t(hist_lane_copies<P>()) * P * kBuckets * 4;
        auto kern = k_histogram<U, MODE, kHistDirectThreads>;
        histogram_setup<U, MODE>(dev);
        const uint64_t per = uint64_t(kHistDirectThreads) * 16;   // at least 16 keys a thread
        const uint32_t g = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>((n + per - 1) / per, device_sms(dev))));
        kern<<<g, kHistDirectThreads, smem, s>>>(static_cast<const U *>(in), n, dmask, ghist, ctrl, bstart, pa);
    }
    return cudaGetLastError();
}

template <typename U>
cudaError_t launch_sort_t(const Resolved &r, uint64_t n, const Layout &L, unsigned char *scratch, const void *in,
                          void *out, void *buf, bool inplace, bool to_buffer, cudaStream_t s) {
    constexpr SweepGeometry gd = sweep_geometry(int(sizeof(U)), false);
    constexpr SweepGeometry gl = sweep_geometry_large(int(sizeof(U)));
    constexpr SweepGeometry gs = sweep_geometry_small(int(sizeof(U)));
    constexpr SweepGeometry gi = sweep_geometry(int(sizeof(U)), true);
    cudaError_t e;
    {
        LaunchTimer t(s, RSBD8G_KERNEL_MEMSET, uint32_t(sizeof(U)), 0, n);
        e = cudaMemsetAsync(scratch, 0, L.zero_bytes, s);
    }
    if (e != cudaSuccess) return e;
    const int mode = int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2));
    const uint32_t dmask = r.f.desc ? 0xFFu : 0u;
    SortArrays arrs{};
    arrs.p[kArrIn] = in;
    arrs.p[kArrOut] = out;
    arrs.p[kArrBuf] = buf;
    arrs.p[kArrKeysA] = r.indirect ? scratch + L.keys_a : nullptr;
    arrs.p[kArrKeysB] = r.indirect ? scratch + L.keys_b : nullptr;
    PlanArgs a{};
    a.inplace = inplace;
    a.to_buffer = to_buffer;
    a.rev = r.rev;
    a.indirect = r.indirect != 0;
    a.passes = uint32_t(KeyTraits<U>::kDigits);
    a.prefetch = r.prefetch;
    a.hot_ok = 1u;
    const bool stall = (r.flags & RSBD8G_FLAG_DIAG_STALL) != 0;
    a.stall_tile = stall ? 1u : 0xFFFFFFFFu;
    a.spin_limit_ns = stall ? 200000000ull : 1000000000ull;
    // the histograms; the CTA that finishes them last writes the plan
#define RSBD8G_HIST(M) e = launch_histogram_t<U, M>(r, n, in, L, scratch, dmask, a, s)
    RSBD8G_MODE_SWITCH(mode, RSBD8G_HIST)
#undef RSBD8G_HIST
    if (e != cudaSuccess) return e;
    const uint32_t P = uint32_t(KeyTraits<U>::kDigits);
    if (r.indirect) {
        e = L.wide_status
                ? launch_sweeps_t<U, 0, true, gi.threads, gi.items, uint64_t>(P, n, L, scratch, arrs, 0u, !inplace, s)
                : launch_sweeps_t<U, 0, true, gi.threads, gi.items, uint32_t>(P, n, L, scratch, arrs, 0u, !inplace, s);
    } else if (L.wide_status) {
#define RSBD8G_SWEEP(M) e = launch_sweeps_t<U, M, false, gd.threads, gd.items, uint64_t>(P, n, L, scratch, arrs, dmask, !inplace, s)
        RSBD8G_MODE_SWITCH(mode, RSBD8G_SWEEP)
#undef RSBD8G_SWEEP
    } else if (L.large_tiles) {
#define RSBD8G_SWEEP(M) e = launch_sweeps_t<U, M, false, gl.threads, gl.items, uint32_t>(P, n, L, scratch, arrs, dmask, !inplace, s)
        RSBD8G_MODE_SWITCH(mode, RSBD8G_SWEEP)
#undef RSBD8G_SWEEP
    } else if (L.small_tiles) {
#define RSBD8G_SWEEP(M) e = launch_sweeps_t<U, M, false, gs.threads, gs.items, uint32_t>(P, n, L, scratch, arrs, dmask, !inplace, s)
        RSBD8G_MODE_SWITCH(mode, RSBD8G_SWEEP)
#undef RSBD8G_SWEEP
    } else {
#define RSBD8G_SWEEP(M) e = launch_sweeps_t<U, M, false, gd.threads, gd.items, uint32_t>(P, n, L, scratch, arrs, dmask, !inplace, s)
        RSBD8G_MODE_SWITCH(mode, RSBD8G_SWEEP)
#undef RSBD8G_SWEEP
    }
    if (e != cudaSuccess) return e;
    if (!inplace) return cudaSuccess;   // the copy forms' copy step ran in the last pass's launch
    int dev = 0;
    cudaGetDevice(&dev);
    const uint32_t cgrid = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, uint64_t(device_sms(dev)) * 8)));
    {
        LaunchTimer t(s, RSBD8G_KERNEL_COPY, uint32_t(sizeof(U)), 0, n);
        k_copy<<<cgrid, 256, 0, s>>>(reinterpret_cast<Control *>(scratch + L.ctrl), arrs, n, uint32_t(r.elem_bytes));
    }
    return cudaGetLastError();
}

// load and set up every kernel a sort with filter MODE can launch, at any count
template <typename U, int MODE>
cudaError_t prepare_mode_t(bool indirect, int dev) {
    constexpr SweepGeometry gd = sweep_geometry(int(sizeof(U)), false);
    constexpr SweepGeometry gl = sweep_geometry_large(int(sizeof(U)));
    constexpr SweepGeometry gs = sweep_geometry_small(int(sizeof(U)));
    constexpr SweepGeometry gi = sweep_geometry(int(sizeof(U)), true);
    cudaFuncAttributes fa{};
    if (indirect) {
        cudaFuncGetAttributes(&fa, k_gather_histogram<U, MODE, kHistThreads>);
        SweepKernels<U, 0, true, gi.threads, gi.items, uint32_t>::setup(dev, nullptr, nullptr);
        SweepKernels<U, 0, true, gi.threads, gi.items, uint64_t>::setup(dev, nullptr, nullptr);
    } else {
        histogram_setup<U, MODE>(dev);
        SweepKernels<U, MODE, false, gd.threads, gd.items, uint32_t>::setup(dev, nullptr, nullptr);
        SweepKernels<U, MODE, false, gd.threads, gd.items, uint64_t>::setup(dev, nullptr, nullptr);
        SweepKernels<U, MODE, false, gl.threads, gl.items, uint32_t>::setup(dev, nullptr, nullptr);
        SweepKernels<U, MODE, false, gs.threads, gs.items, uint32_t>::setup(dev, nullptr, nullptr);
    }
    cudaFuncGetAttributes(&fa, k_copy);
    return cudaGetLastError();
}

template <typename U>
cudaError_t prepare_sort_t(const Resolved &r) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int mode = int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2));
#define RSBD8G_PREP(M) e = prepare_mode_t<U, M>(r.indirect != 0, dev)
    RSBD8G_MODE_SWITCH(mode, RSBD8G_PREP)
#undef RSBD8G_PREP
    return e;
}

}  // namespace rsbd8g

#define RSBD8G_DEFINE_LAUNCH(name, U)                                                                          \
    namespace rsbd8g {                                                                                         \
    cudaError_t name(const Resolved &r, uint64_t n, const Layout &L, unsigned char *scratch, const void *in,   \
                     void *out, void *buf, bool inplace, bool to_buffer, cudaStream_t s) {                    \
        return launch_sort_t<U>(r, n, L, scratch, in, out, buf, inplace, to_buffer, s);                       \
    }                                                                                                          \
    cudaError_t name##_prepare(const Resolved &r) { return prepare_sort_t<U>(r); }                             \
    }
