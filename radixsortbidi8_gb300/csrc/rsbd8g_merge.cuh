// rsbd8g_merge.cuh - stable merge of sorted runs on the device (the reference's mergehalves* /
// mergethirds*, Radixsortbidi8.hpp:54437-56418).
//
// Two runs A and B, each sorted by the same descriptor, merge into one stably sorted array: an
// element of A goes before an element of B when its filtered key orders first, and on equal keys
// when A has precedence -- the earlier run in forward order, the later run under isrevorder (the
// reference walks its halves from the top and swaps their roles for isrevorder,
// Radixsortbidi8.hpp:54453-54456).  Three runs are merged as (A merge B) merge C through a buffer,
// which gives the same order as the reference's three-way walk (:55381-55386).
//
// k_merge2: persistent CTAs, each writing one contiguous range of the output (see the kernel).
// No scratch memory.
#pragma once
#include "rsbd8g_device.cuh"

namespace rsbd8g {

// the filtered key of raw bits in the order of the sort: complemented for descending sorts
template <int MODE, typename U>
__host__ __device__ __forceinline__ U order_key(U b, bool desc) {
    const U k = filter_key<MODE>(b);
    return desc ? key_not(k) : k;
}

template <typename U>
__host__ __device__ __forceinline__ bool key_less(U a, U b) { return a < b; }
template <int HB>
__host__ __device__ __forceinline__ bool key_less(KeyWide<HB> a, KeyWide<HB> b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// does a (from run A) go before b (from run B)?  a_first: A has precedence on equal keys
template <int MODE, typename U>
__host__ __device__ __forceinline__ bool a_before_b(U a, U b, bool desc, bool a_first) {
    const U ka = order_key<MODE>(a, desc), kb = order_key<MODE>(b, desc);
    return a_first ? !key_less(kb, ka) : key_less(ka, kb);
}

// elements of A among the first d elements of the merge of A[0, na) and B[0, nb), found by one
// warp (all 32 lanes call it with the same arguments): each round probes 32 points of the interval
// holding the answer and keeps the gap between the last true and the first false probe, so a
// search over n elements takes about log32(n) dependent loads instead of log2(n)
// (`at_a(i)` / `at_b(j)`: element i of A, element j of B -- global arrays or the circular windows)
template <int MODE, typename U, typename I, typename FA, typename FB>
__device__ __forceinline__ I merge_path_warp_by(FA at_a, I na, FB at_b, I nb, I d, bool desc, bool a_first) {
    I lo = d > nb ? d - nb : 0, hi = d < na ? d : na;             // the answer lies in [lo, hi]
    const uint32_t lane = threadIdx.x & 31u;
    while (hi - lo > 32) {
        const I p = lo + I(uint64_t(hi - lo) * (lane + 1) / 33);   // 32 increasing points of (lo, hi)
        const bool t = a_before_b<MODE>(at_a(p), at_b(d - 1 - p), desc, a_first);
        const int k = __popc(__ballot_sync(0xFFFFFFFFu, t));     // the true probes are a prefix
        const I below = __shfl_sync(0xFFFFFFFFu, p, k > 0 ? k - 1 : 0);
        const I above = __shfl_sync(0xFFFFFFFFu, p, k < 32 ? k : 31);
        if (k > 0) lo = below + 1;
        if (k < 32) hi = above;
    }
    const I p = lo + lane;
    const bool t = p < hi && a_before_b<MODE>(at_a(p), at_b(d - 1 - p), desc, a_first);
    return lo + I(__popc(__ballot_sync(0xFFFFFFFFu, t)));
}

template <int MODE, typename U>
__device__ __forceinline__ uint64_t merge_path_warp(const U *A, uint64_t na, const U *B, uint64_t nb, uint64_t d,
                                                    bool desc, bool a_first) {
    return merge_path_warp_by<MODE, U, uint64_t>([A](uint64_t i) { return A[i]; }, na,
                                                 [B](uint64_t j) { return B[j]; }, nb, d, desc, a_first);
}

// the same search on the circular shared-memory windows of the persistent merge: element x of the
// A window is wa[(a0 + x) % TILE], and the windows hold at least d elements of each run (or the run's rest)
template <int MODE, int TILE, typename U>
__device__ __forceinline__ uint32_t merge_path_window(const U *wa, uint32_t a0, uint32_t na, const U *wb, uint32_t b0,
                                                      uint32_t nb, uint32_t d, bool desc, bool a_first) {
    uint32_t lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a_before_b<MODE>(wa[(a0 + mid) & (TILE - 1)], wb[(b0 + d - 1 - mid) & (TILE - 1)], desc, a_first)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <typename U, int THREADS, int ITEMS>
struct MergeSmem {
    static constexpr int kTile = THREADS * ITEMS;
    static_assert((kTile & (kTile - 1)) == 0, "the windows are circular buffers of a power of two");
    // circular windows of A and B (kTile elements each), and the merged tile with one pad slot per 32
    static constexpr size_t kWin = size_t(kTile) * sizeof(U);
    static constexpr size_t kOut = size_t(kTile + kTile / 32) * sizeof(U);
    static constexpr size_t kBytes = 2 * kWin + kOut + 64;
    __device__ static uint32_t pad(uint32_t i) { return i + (i >> 5); }
};

// Persistent merge: CTA c writes the outputs [c * per, (c + 1) * per) tile by tile.  One warp finds
// where the range starts on the merge path; from there the CTA keeps a window of the next TILE
// elements of A and of B in circular shared-memory buffers.  Per tile: thread 0 finds how many of
// the tile's outputs come from A (a search in the windows); every thread starts the global loads of
// the elements that slide into the windows for the next tile (into registers), finds its own
// ITEMS-output diagonal and merges sequentially into the staging array; the tile is stored
// coalesced and the loaded elements replace the consumed ones.  Every element is read from global
// memory once.
template <typename U, int MODE, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS) k_merge2(const U *__restrict__ A, uint64_t na, const U *__restrict__ B,
                                                    uint64_t nb, U *__restrict__ out, uint32_t desc, uint32_t a_first,
                                                    uint64_t per) {
    using L = MergeSmem<U, THREADS, ITEMS>;
    constexpr int TILE = L::kTile;
    constexpr uint32_t M = TILE - 1;
    extern __shared__ __align__(16) unsigned char smem[];
    U *wa = reinterpret_cast<U *>(smem);
    U *wb = reinterpret_cast<U *>(smem + L::kWin);
    U *sout = reinterpret_cast<U *>(smem + 2 * L::kWin);
    uint64_t *misc = reinterpret_cast<uint64_t *>(smem + 2 * L::kWin + L::kOut);   // [0] range start split [1] tile split
    const uint64_t total = na + nb;
    uint64_t o = uint64_t(blockIdx.x) * per;
    if (o >= total) return;
    const uint64_t oend = o + per < total ? o + per : total;
    const bool dsc = desc != 0, af = a_first != 0;
    const int tid = threadIdx.x;
    if (tid < 32) {
        const uint64_t sp = merge_path_warp<MODE>(A, na, B, nb, o, dsc, af);
        if (tid == 0) misc[0] = sp;
    }
    __syncthreads();
    uint64_t ia = misc[0], ib = o - ia;
    // fill the windows: A[ia, ia + TILE) and B[ib, ib + TILE), cut at the runs' ends
    uint64_t aend = ia + TILE < na ? ia + TILE : na, bend = ib + TILE < nb ? ib + TILE : nb;
    for (uint64_t x = ia + tid; x < aend; x += THREADS) wa[x & M] = A[x];
    for (uint64_t x = ib + tid; x < bend; x += THREADS) wb[x & M] = B[x];
    __syncthreads();
    while (o < oend) {
        const uint32_t r = uint32_t(oend - o < uint64_t(TILE) ? oend - o : uint64_t(TILE));
        const uint32_t ca = uint32_t(aend - ia), cb = uint32_t(bend - ib);       // elements in the windows
        if (tid < 32) {      // the tile's share of A: one warp, 32 probes a round
            const uint32_t a0 = uint32_t(ia & M), b0 = uint32_t(ib & M);
            const uint32_t sp = merge_path_warp_by<MODE, U, uint32_t>([wa, a0](uint32_t i) { return wa[(a0 + i) & M]; }, ca,
                                                                    [wb, b0](uint32_t j) { return wb[(b0 + j) & M]; }, cb,
                                                                    r, dsc, af);
            if (tid == 0) misc[1] = sp;
        }
        __syncthreads();
        const uint32_t sa = uint32_t(misc[1]);
        const uint64_t ia2 = ia + sa, ib2 = ib + (r - sa);
        // the elements that slide into the windows for the next tile, loaded now (consumed slots are
        // only overwritten after the merge below has read them)
        const uint64_t aend2 = ia2 + TILE < na ? ia2 + TILE : na, bend2 = ib2 + TILE < nb ? ib2 + TILE : nb;
        const uint32_t na_new = uint32_t(aend2 - aend), nb_new = uint32_t(bend2 - bend);
        U va[ITEMS], vb[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t x = uint32_t(tid) + uint32_t(j) * THREADS;
            if (x < na_new) va[j] = A[aend + x];
            if (x < nb_new) vb[j] = B[bend + x];
        }
        // this thread's outputs [d0, d0 + ITEMS) of the tile
        const uint32_t d0 = uint32_t(tid) * ITEMS;
        if (d0 < r) {
            const uint32_t a0 = uint32_t(ia & M), b0 = uint32_t(ib & M);
            uint32_t xa = merge_path_window<MODE, TILE>(wa, a0, ca, wb, b0, cb, d0, dsc, af), xb = d0 - xa;
            const uint32_t cnt = r - d0 < uint32_t(ITEMS) ? r - d0 : uint32_t(ITEMS), nat = sa, nbt = r - sa;
            // the next element of each side and its ordering key stay in registers: one load and one
            // filter per output
            U ua = wa[(a0 + xa) & M], ub = wb[(b0 + xb) & M];
            U ka = order_key<MODE>(ua, dsc), kb = order_key<MODE>(ub, dsc);
#pragma unroll
            for (int q = 0; q < ITEMS; ++q) {
                if (uint32_t(q) < cnt) {
                    // A goes first unless its share of the tile is used up, B's is, or B orders first
                    const bool take_a = xa < nat && (xb >= nbt || (af ? !key_less(kb, ka) : key_less(ka, kb)));
                    sout[L::pad(d0 + q)] = take_a ? ua : ub;
                    if (take_a) {
                        ++xa;
                        ua = wa[(a0 + xa) & M];
                        ka = order_key<MODE>(ua, dsc);
                    } else {
                        ++xb;
                        ub = wb[(b0 + xb) & M];
                        kb = order_key<MODE>(ub, dsc);
                    }
                }
            }
        }
        __syncthreads();
        for (uint32_t x = uint32_t(tid); x < r; x += THREADS) out[o + x] = sout[L::pad(x)];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t x = uint32_t(tid) + uint32_t(j) * THREADS;
            if (x < na_new) wa[(aend + x) & M] = va[j];
            if (x < nb_new) wb[(bend + x) & M] = vb[j];
        }
        __syncthreads();
        o += r;
        ia = ia2;
        ib = ib2;
        aend = aend2;
        bend = bend2;
    }
}

}  // namespace rsbd8g
