// rsbd8g_internal.h - shared host-side declarations of the GB300 radix sort library.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "rsbd8g.h"
#include "rsbd8g_device.cuh"

namespace rsbd8g {

// a descriptor after the reference's compile-time mode resolution
struct Resolved {
    Filter f;
    uint32_t rev;         // effective isrevorder
    uint32_t key_bytes;   // 1, 2, 4, 8, 16
    uint32_t x87;         // 16-byte x87 extended precision keys (10 digits)
    uint32_t digits;      // 8-bit digit passes of the key
    uint32_t elem_bytes;  // bytes per array element (key bytes, or 8 for object pointers)
    uint32_t indirect;    // RSBD8G_DIRECT / RSBD8G_MEMBER / RSBD8G_MEMBER2
    uint32_t flags;
    uint32_t prefetch;    // every array of the call is device memory (tiles may be prefetched into L2)
    int64_t off1, off2;
    const void *keys;     // RSBD8G_KEYED: the caller's key array
};

// byte offsets of the parts of a scratch area
struct Layout {
    size_t ctrl, ghist, bstart, status, status_pass_bytes, zero_bytes, keys_a, keys_b, total;
    uint32_t num_tiles;
    bool wide_status;
    bool large_tiles;     // sweep_geometry_large applies
    bool small_tiles;     // sweep_geometry_small applies
};

// brackets one kernel launch with CUDA events on its stream while launch profiling is on
class LaunchTimer {
public:
    LaunchTimer(cudaStream_t s, uint32_t kernel, uint32_t key_bytes, uint32_t pass, uint64_t n);
    ~LaunchTimer();
    LaunchTimer(const LaunchTimer &) = delete;
    LaunchTimer &operator=(const LaunchTimer &) = delete;

private:
    cudaStream_t s_;
    cudaEvent_t a_, b_;
    rsbd8g_launch_record rec_{};
};

int device_sms(int dev);

// the launch sequence of one sort, per key size (rsbd8g_sort_k{1,2,4,8}.cu)
#define RSBD8G_DECLARE_LAUNCH(name)                                                                          \
    cudaError_t name(const Resolved &r, uint64_t n, const Layout &L, unsigned char *scratch, const void *in, \
                     void *out, void *buf, bool inplace, bool to_buffer, cudaStream_t s);                   \
    cudaError_t name##_prepare(const Resolved &r);   /* load every kernel this sort can launch */
RSBD8G_DECLARE_LAUNCH(launch_sort_k1)
RSBD8G_DECLARE_LAUNCH(launch_sort_k2)
RSBD8G_DECLARE_LAUNCH(launch_sort_k4)
RSBD8G_DECLARE_LAUNCH(launch_sort_k8)
RSBD8G_DECLARE_LAUNCH(launch_sort_k16)
RSBD8G_DECLARE_LAUNCH(launch_sort_x87)

// tile geometry of the onesweep passes, per key size (keys per tile = threads * items)
struct SweepGeometry {
    int threads, items;
};
constexpr SweepGeometry sweep_geometry(int key_bytes, bool indirect) {
    if (indirect) return SweepGeometry{512, key_bytes == 16 ? 6 : 8};
    return SweepGeometry{512, key_bytes == 16 ? 6 : (key_bytes == 8 ? 16 : 24)};
}
// Direct keys of up to 4 bytes take three tile sizes by the count of the sort (narrow look-back
// words only, under 2^30 keys): 512 x 32 from kLargeTileMinKeys keys on -- fewer tiles mean fewer
// per-tile phases and shorter look-back chains (uint32 2^28: -5 % against 512 x 24) -- 512 x 24 in
// between, and 512 x 16 below kSmallTileMaxKeys, where more tiles keep every SM busy and fill the
// pipelined pass sooner (uint32 2^20 / 2^21 / 2^22: -10 / -10 / -5 %).  The choice depends on the
// count alone, so a scratch size computed once fits every call of that count.
constexpr uint64_t kLargeTileMinKeys = uint64_t(1) << 25;
constexpr uint64_t kSmallTileMaxKeys = uint64_t(1) << 23;
constexpr SweepGeometry sweep_geometry_large(int key_bytes) {
    return key_bytes <= 4 ? SweepGeometry{512, 32} : sweep_geometry(key_bytes, false);
}
constexpr SweepGeometry sweep_geometry_small(int key_bytes) {
    return key_bytes <= 4 ? SweepGeometry{512, 16} : sweep_geometry(key_bytes, false);
}
// the segmented sort's large segments, two tile sizes per key size, picked per batch shape by the
// autotuner (rsbd8g_segtuning::large_variant).  Variant 0: 512 x 28 for keys up to 4 bytes (measured
// against 24 and 32 on the 2^28-key batch of uint32 arrays) and 512 x 12 for 8-byte keys, smaller
// than the plain sort's tiles because a segment's last tile is partly empty.  Variant 1: 512 x 20
// and 512 x 16, for batches of shorter or longer large segments.  16-byte keys: 512 x 6 in both.
constexpr int kSegLargeVariants = 2;
constexpr SweepGeometry seg_sweep_geometry(int key_bytes, int variant) {
    return SweepGeometry{512, key_bytes == 16 ? 6
                              : key_bytes == 8 ? (variant == 1 ? 16 : 12)
                                               : (variant == 1 ? 20 : 28)};
}

#define RSBD8G_MODE_SWITCH(mode, CALL) \
    switch (mode) {                    \
        case 0: CALL(0); break;        \
        case 1: CALL(1); break;        \
        case 2: CALL(2); break;        \
        case 3: CALL(3); break;        \
        case 4: CALL(4); break;        \
        case 5: CALL(5); break;        \
        case 6: CALL(6); break;        \
        default: CALL(7); break;       \
    }

// shapes of the small-segment block sort (threads x items = the largest small segment)
struct SegSmallShape {
    int threads, items;
};
constexpr SegSmallShape seg_small_shape(int key_bytes, int variant) {
    return key_bytes == 16 ? (variant == 0 ? SegSmallShape{256, 4} : variant == 1 ? SegSmallShape{256, 6} : SegSmallShape{512, 4})
         : key_bytes == 8 ? (variant == 0 ? SegSmallShape{256, 8} : variant == 1 ? SegSmallShape{256, 12} : SegSmallShape{512, 12})
                          : (variant == 0 ? SegSmallShape{256, 8} : variant == 1 ? SegSmallShape{256, 16} : SegSmallShape{512, 16});
}
constexpr int kSegSmallVariants = 3;

// byte offsets of the parts of a segmented-sort scratch area
struct SegLayout {
    size_t ctrl, large_seg, large_tbase, small_seg, seg_hist, seg_mask, tile_seg, status, status_bytes, zero_bytes, total;
    uint64_t nlarge_max, tiles_max;
    uint32_t cutoff, small_variant, tile, large_variant;
};

struct SegArgs;
#define RSBD8G_DECLARE_SEG_LAUNCH(name)                                                                \
    cudaError_t name(const Resolved &r, const SegArgs &a, const SegLayout &L, unsigned char *scratch, \
                     const void *in, void *out, void *buf, cudaStream_t s);                           \
    cudaError_t name##_prepare(const Resolved &r);   /* load every kernel this sort can launch */
RSBD8G_DECLARE_SEG_LAUNCH(launch_segmented_k1)
RSBD8G_DECLARE_SEG_LAUNCH(launch_segmented_k2)
RSBD8G_DECLARE_SEG_LAUNCH(launch_segmented_k4)
RSBD8G_DECLARE_SEG_LAUNCH(launch_segmented_k8)
RSBD8G_DECLARE_SEG_LAUNCH(launch_segmented_k16)

rsbd8g_status resolve(const rsbd8g_desc *d, Resolved *r);
cudaError_t prepare_segmented(const Resolved &r);   // rsbd8g_segmented_api.cu: rsbd8g_prepare's segmented part
// p is device memory (cudaMalloc, a memory pool, a __device__ array); null counts as such
bool device_memory(const void *p);
// the resolved filter of a descriptor (isabsvalue | issignmode << 1 | isfltpmode << 2 | x87 << 3),
// -1 for a bad descriptor: descriptors of one key size and filter sort alike but for direction
int filter_class(const rsbd8g_desc *d);
Layout layout_for(const Resolved &r, uint64_t n);
rsbd8g_status enqueue_sort(const Resolved &r, uint64_t n, void *scratch, size_t scratch_bytes, const void *in,
                           void *out, void *buf, bool inplace, bool to_buffer, cudaStream_t s);
rsbd8g_status read_device_status(void *scratch, cudaStream_t s, bool clear);

}  // namespace rsbd8g
