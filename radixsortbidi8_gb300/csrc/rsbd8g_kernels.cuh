// rsbd8g_kernels.cuh - the sm_103a kernels of the stable LSD radix sort.
//
//   k_histogram / k_gather_histogram   all 256-bin digit histograms in one read of the keys, with
//                                      shared-memory atomics on per-lane-class counters (direct
//                                      keys) or warp-aggregated atomics on sub-histogram copies
//                                      (the gather form, which reads the key through each object
//                                      pointer and writes the filtered keys once); the CTA that
//                                      finishes last runs plan_body: the exclusive scan of every
//                                      digit histogram, the reference's pass-skip test and the
//                                      ping-pong plan of the passes
//   k_onesweep                         one stable scatter pass of a surviving digit: persistent
//                                      CTAs claim tiles in order, rank keys with a warp
//                                      multisplit (TileRank: shared-memory match words), resolve
//                                      the tile's global bucket offsets with a bounded decoupled
//                                      look-back, stage the tile in shared memory sorted by digit
//                                      and write it out coalesced
//   k_onesweep_pipe                    the same pass with the look-back of one tile overlapping the
//                                      load and ranking of the next, and the next tile prefetched
//                                      into L2 (the pass of every sort of two tiles per CTA or more)
//   k_copy                             the plain / reversed copy of the in-place forms when parity
//                                      or all-skipped passes need one (the copy forms need one only
//                                      when every pass was skipped, and the last pass's launch does it)
#pragma once
#include "rsbd8g_device.cuh"

namespace rsbd8g {

// ---- scan, pass-skip and plan -----------------------------------------------------------------

struct PlanArgs {
    uint64_t spin_limit_ns;
    uint32_t inplace;      // radixsort / radixsortnoalloc: sort `in` using `buf`
    uint32_t to_buffer;    // movetobuffer
    uint32_t rev;          // effective isrevorder
    uint32_t indirect;
    uint32_t stall_tile;
    uint32_t passes;       // digits of the key
    uint32_t prefetch;     // every array is device memory (Control::prefetch)
    uint32_t hot_ok;       // crowded digits may be ranked with ballots (PassPlan::hot)
};

// a digit is ranked with ballots (PassPlan::hot) when it holds more than 1/kHotShare of the keys: the
// ballots cost every key of the pass instructions (about 30 % more time on a pass of uniform digits
// with two hot digits), and they pay only where many lanes of a unit share the digit (float32 keys
// of N(0, 1e3) by absolute value, top digit: 56 % of the keys in one bucket, 28 % in the next; that
// pass 1.13 ms -> 1.05 ms at 2^28 keys with the fullest digit ranked by ballots, 1.13 ms with both)
constexpr unsigned long long kHotShare = 4;

// the plan's 256 threads (one per digit) meet at named barrier 1, so the rest of the block that runs
// the plan can leave
__device__ __forceinline__ void plan_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
__device__ __forceinline__ int plan_sync_or(int pred) {
    int r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.or.pred q, 1, 256, p;\n\t"
                 "selp.s32 %0, 1, 0, q;\n\t}" : "=r"(r) : "r"(pred) : "memory");
    return r;
}

// the largest value over the plan's 8 warps (threads 0..255 call it)
__device__ __forceinline__ unsigned long long plan_block_max(unsigned long long v, unsigned long long *wbuf) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = y > v ? y : v;
    }
    if (lane == 0) wbuf[w] = v;
    plan_sync();
    unsigned long long m = wbuf[0];
    for (int i = 1; i < kBuckets / 32; ++i) m = wbuf[i] > m ? wbuf[i] : m;
    plan_sync();
    return m;
}

// The plan of the sort from the complete digit histograms: bucket starts (exclusive scans), the
// pass-skip test, the crowded digit of each pass and the ping-pong schedule.  Run by the last
// histogram CTA to finish (so it needs no launch of its own): its threads 0..255, one per digit,
// call it; the block's other threads do not.
__device__ __forceinline__ void plan_body(Control *__restrict__ ctrl, const unsigned long long *__restrict__ ghist,
                                          unsigned long long *__restrict__ bstart, uint64_t n, const PlanArgs &a) {
    __shared__ unsigned long long wsum[kBuckets / 32];
    __shared__ int skip[kMaxPasses];
    __shared__ uint32_t hot[kMaxPasses];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int p = 0; p < int(a.passes); ++p) {
        // the other CTAs' counts arrive through L2 (their atomics were fenced before they finished)
        const unsigned long long h = __ldcg(ghist + p * kBuckets + t);
        // pass-skip: one bucket holds every key (Radixsortbidi8.hpp:12259, :12272, :2903)
        const int all_in_one = plan_sync_or(h == n);
        // the pass's fullest bucket, (count << 8) | digit: a crowded one is ranked with ballots
        const unsigned long long m0 = plan_block_max((h << 8) | uint32_t(t), wsum);
        if (t == 0) {
            const uint32_t h0 = (m0 >> 8) > n / kHotShare ? uint32_t(m0 & 0xFFu) : kNoHot;
            hot[p] = a.hot_ok ? ((kNoHot << 16) | h0) : kNoHotPair;
        }
        unsigned long long x = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        plan_sync();
        unsigned long long before = 0;
        for (int i = 0; i < w; ++i) before += wsum[i];
        bstart[p * kBuckets + t] = before + x - h;
        if (t == 0) skip[p] = all_in_one;
        plan_sync();
    }
    if (t != 0) return;
    int k = 0;
    for (int p = 0; p < int(a.passes); ++p) k += !skip[p];
    ctrl->active_passes = uint32_t(k);
    ctrl->spin_limit_ns = a.spin_limit_ns;
    ctrl->stall_tile = a.stall_tile;
    ctrl->prefetch = a.prefetch;
    ctrl->copy_mode = kCopyNone;
    uint32_t cur = kArrIn;                // where the data (values for indirection) is
    uint32_t curk = kArrKeysA;            // indirection: where the filtered keys are
    int i = 0;
    for (int p = 0; p < int(a.passes); ++p) {
        PassPlan &pp = ctrl->plan[p];
        pp.active = !skip[p];
        pp.hot = hot[p];
        if (skip[p]) continue;
        ++i;
        uint32_t dst;
        if (a.inplace) dst = (cur == kArrIn) ? kArrBuf : kArrIn;
        else dst = ((k - i) % 2 == 0) ? kArrOut : kArrBuf;
        pp.reverse = (i == 1) && a.rev;
        if (a.indirect) {
            pp.src_vals = cur;
            pp.dst_vals = dst;
            pp.src_keys = curk;
            const uint32_t dk = (curk == kArrKeysA) ? kArrKeysB : kArrKeysA;
            pp.dst_keys = (i == k) ? kArrNone : dk;
            curk = dk;
        } else {
            pp.src_keys = cur;
            pp.dst_keys = dst;
            pp.src_vals = kArrNone;
            pp.dst_vals = kArrNone;
        }
        cur = dst;
    }
    if (!a.inplace) {
        if (k == 0) {
            ctrl->copy_mode = a.rev ? kCopyReversed : kCopyPlain;
            ctrl->copy_src = kArrIn;
            ctrl->copy_dst = kArrOut;
        }
    } else {
        const uint32_t target = a.to_buffer ? kArrBuf : kArrIn;
        if (k == 0 && a.rev) {
            ctrl->copy_mode = a.to_buffer ? kCopyReversed : kReverseInPlace;
            ctrl->copy_src = kArrIn;
            ctrl->copy_dst = target;
        } else if (cur != target) {
            ctrl->copy_mode = kCopyPlain;
            ctrl->copy_src = cur;
            ctrl->copy_dst = target;
        }
    }
}

// ---- up-front histograms --------------------------------------------------------------------

// Gather-histogram counting: each CTA keeps kHistCopies sub-histograms (P digits x 256 bins, u32)
// in shared memory and its warps spread over them, so warps rarely collide on a bin.  A warp whose
// lanes all share the digit (a skewed digit, e.g. the zero top bytes of small keys) adds 32 with
// one atomic instead of 32 conflicting ones.
constexpr int kHistCopies = 4;

__device__ __forceinline__ void hist_add(uint32_t *h, uint32_t d, bool valid) {
    const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, 0);
    const bool v0 = __shfl_sync(0xFFFFFFFFu, valid, 0);
    if (__all_sync(0xFFFFFFFFu, valid && d == d0)) {
        if ((threadIdx.x & 31u) == 0 && v0) atomicAdd(h + d0, 32u);
    } else if (valid) {
        atomicAdd(h + d, 1u);
    }
}

template <typename U>
__device__ __forceinline__ void count_key(uint32_t *sh, U k, bool valid, uint32_t dmask) {
#pragma unroll
    for (int p = 0; p < KeyTraits<U>::kDigits; ++p) hist_add(sh + p * kBuckets, digit_of(k, p) ^ dmask, valid);
}

// copies of the gather histogram: fewer for the 16 digits of 128-bit keys (static shared memory)
template <int P>
constexpr int gather_hist_copies() { return P > 8 ? 2 : kHistCopies; }

template <int THREADS, int P>
__device__ __forceinline__ void zero_hist(uint32_t *sh) {
    for (int i = threadIdx.x; i < gather_hist_copies<P>() * P * kBuckets; i += THREADS) sh[i] = 0;
    __syncthreads();
}

template <int THREADS, int P>
__device__ __forceinline__ void flush_hist(const uint32_t *sh, unsigned long long *ghist) {
    __syncthreads();
    for (int i = threadIdx.x; i < P * kBuckets; i += THREADS) {
        uint32_t v = 0;
#pragma unroll
        for (int c = 0; c < gather_hist_copies<P>(); ++c) v += sh[c * P * kBuckets + i];
        if (v) atomicAdd(ghist + i, (unsigned long long)v);
    }
}

// The CTA that finishes its share of the histograms last computes the plan (plan_body): each CTA
// fences its global-histogram atomics before it counts itself done.  Every thread calls this.
template <int THREADS>
__device__ __forceinline__ void plan_if_last(Control *__restrict__ ctrl, const unsigned long long *__restrict__ ghist,
                                             unsigned long long *__restrict__ bstart, uint64_t n, const PlanArgs &a) {
    static_assert(THREADS >= kBuckets && THREADS % 32 == 0, "the plan needs a thread per digit");
    __shared__ uint32_t last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&ctrl->hist_done, 1u) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (!last || threadIdx.x >= kBuckets) return;
    __threadfence();
    plan_body(ctrl, ghist, bstart, n, a);
}

// Direct keys: all P digit histograms in one read.  Every (digit position, bin) has C shared-memory
// counters, one per lane class (lane % C), laid out so that lane l always uses bank l % 32: the 32
// lanes of a warp never meet in a bank (C = 32, keys up to 4 bytes) or at most pairwise (C = 16,
// 8-byte keys, 128 KB either way).  One 1024-thread CTA per SM reads 16-byte vectors grid-strided;
// at the end each CTA folds its C copies (rotated reads, conflict-free) into the global histogram.
template <int P>
constexpr int hist_lane_copies() { return P <= 4 ? 32 : (P <= 8 ? 16 : 8); }

template <typename U, int MODE, int THREADS>
__global__ void __launch_bounds__(THREADS) k_histogram(const U *__restrict__ keys, uint64_t n, uint32_t dmask,
                                                       unsigned long long *__restrict__ ghist, Control *__restrict__ ctrl,
                                                       unsigned long long *__restrict__ bstart, PlanArgs pa) {
    constexpr int P = KeyTraits<U>::kDigits;
    constexpr int C = hist_lane_copies<P>();
    constexpr int V = 16 / int(sizeof(U));
    extern __shared__ __align__(16) uint32_t shl[];
    for (int i = threadIdx.x; i < C * P * kBuckets; i += THREADS) shl[i] = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t *sh = shl + (lane & uint32_t(C - 1));
    auto count = [&](U k, bool ok) {
        if (!ok) return;
#pragma unroll
        for (int p = 0; p < P; ++p) atomicAdd(sh + (p * kBuckets + (digit_of(k, p) ^ dmask)) * C, 1u);
    };
    const uint64_t mis = (reinterpret_cast<uintptr_t>(keys) & 15u) / sizeof(U);
    const uint64_t head = mis ? (uint64_t(V) - mis < n ? uint64_t(V) - mis : n) : 0;
    const uint64_t nvec = (n - head) / V;
    const uint64_t tail0 = head + nvec * V;
    const uint64_t gthread = uint64_t(blockIdx.x) * THREADS + threadIdx.x;
    const uint64_t nthreads = uint64_t(gridDim.x) * THREADS;
    if (gthread < 32) {
        for (uint64_t i = gthread; i < head; i += 32) count(filter_key<MODE>(keys[i]), true);
        for (uint64_t i = tail0 + gthread; i < n; i += 32) count(filter_key<MODE>(keys[i]), true);
    }
    const uint4 *kv = reinterpret_cast<const uint4 *>(keys + head);
    constexpr int UNR = 4;
    for (uint64_t b = gthread; b < nvec; b += nthreads * UNR) {
        uint4 v[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const uint64_t i = b + uint64_t(u) * nthreads;
            v[u] = i < nvec ? __ldg(kv + i) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const bool ok = b + uint64_t(u) * nthreads < nvec;
            U k[V];
            memcpy(k, &v[u], 16);
#pragma unroll
            for (int j = 0; j < V; ++j) count(filter_key<MODE>(k[j]), ok);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < P * kBuckets; i += THREADS) {
        uint32_t t = 0;
#pragma unroll 8
        for (int c = 0; c < C; ++c) t += shl[i * C + ((c + i) & (C - 1))];
        if (t) atomicAdd(ghist + i, (unsigned long long)t);
    }
    plan_if_last<THREADS>(ctrl, ghist, bstart, n, pa);
}

// indirect form: gather the key through each object pointer (level 1: at off1; level 2: behind the
// pointer held at off1, at off2; level 3: keys_in[i], supplied by the caller), write the filtered key
template <typename U, int MODE, int THREADS>
__global__ void __launch_bounds__(THREADS) k_gather_histogram(const uint64_t *__restrict__ ptrs, uint64_t n,
                                                              uint32_t dmask, int64_t off1, int64_t off2, int level,
                                                              const U *__restrict__ keys_in,
                                                              U *__restrict__ keys_out,
                                                              unsigned long long *__restrict__ ghist,
                                                              Control *__restrict__ ctrl,
                                                              unsigned long long *__restrict__ bstart, PlanArgs pa) {
    constexpr int P = KeyTraits<U>::kDigits;
    __shared__ uint32_t shall[gather_hist_copies<P>() * P * kBuckets];
    zero_hist<THREADS, P>(shall);
    uint32_t *sh = shall + ((threadIdx.x >> 5) % gather_hist_copies<P>()) * P * kBuckets;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t gwarp = (uint64_t(blockIdx.x) * THREADS + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * THREADS) >> 5;
    constexpr int UNR = 4;
    for (uint64_t b = gwarp * 32 * UNR; b < n; b += nwarps * 32 * UNR) {
        U raw[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const uint64_t i = b + u * 32 + lane;
            raw[u] = U{};
            if (i < n) {
                if (level == 3) {
                    raw[u] = keys_in[i];
                } else {
                    const unsigned char *obj = reinterpret_cast<const unsigned char *>(ptrs[i]) + off1;
                    if (level == 2) obj = load_ptr(obj) + off2;
                    raw[u] = load_member<U>(obj);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const uint64_t i = b + u * 32 + lane;
            const bool ok = i < n;
            // the stored key is final: filtered, and complemented for descending sorts
            const U k = dmask ? key_not(filter_key<MODE>(raw[u])) : filter_key<MODE>(raw[u]);
            if (ok) keys_out[i] = k;
            count_key(sh, k, ok, 0u);
        }
    }
    flush_hist<THREADS, P>(shall, ghist);
    plan_if_last<THREADS>(ctrl, ghist, bstart, n, pa);
}

// ---- copy step --------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ void copy_elems(const Control &c, const T *src, T *dst, uint64_t n) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uint64_t i0 = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c.copy_mode == kCopyPlain) {
        for (uint64_t i = i0; i < n; i += stride) dst[i] = src[i];
    } else if (c.copy_mode == kCopyReversed) {
        for (uint64_t i = i0; i < n; i += stride) dst[i] = src[n - 1u - i];
    } else if (c.copy_mode == kReverseInPlace) {
        for (uint64_t i = i0; i < n / 2u; i += stride) {
            const T a = dst[i], b = dst[n - 1u - i];
            dst[i] = b;
            dst[n - 1u - i] = a;
        }
    }
}

// the copy step: plain or reversed copy (or reversal in place) of n elements of elem_bytes bytes,
// as the plan in the control block names it; every thread of the grid calls it.  elem_bytes and the
// arrays are kernel parameters, like everything that sizes or addresses an access.
__device__ __forceinline__ void copy_step(Control *__restrict__ ctrl, const SortArrays &arrs, uint64_t n,
                                          uint32_t elem_bytes) {
    const Control c = *ctrl;
    if (c.copy_mode == kCopyNone) return;
    bool bad = false;
    const void *src = sort_array(arrs, c.copy_src, kArrIn, &bad);
    void *dst = sort_array(arrs, c.copy_dst, kArrBuf, &bad);
    if (bad || !src || !dst) {      // a damaged control block
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&ctrl->error, kDevFault);
        return;
    }
    switch (elem_bytes) {
        case 1: copy_elems<uint8_t>(c, static_cast<const uint8_t *>(src), static_cast<uint8_t *>(dst), n); break;
        case 2: copy_elems<uint16_t>(c, static_cast<const uint16_t *>(src), static_cast<uint16_t *>(dst), n); break;
        case 4: copy_elems<uint32_t>(c, static_cast<const uint32_t *>(src), static_cast<uint32_t *>(dst), n); break;
        case 8: copy_elems<uint64_t>(c, static_cast<const uint64_t *>(src), static_cast<uint64_t *>(dst), n); break;
        default:                   // 16-byte elements
            copy_elems<uint4>(c, static_cast<const uint4 *>(src), static_cast<uint4 *>(dst), n);
            break;
    }
}

// the copy step of the in-place forms, after the last pass
static __global__ void __launch_bounds__(256) k_copy(Control *__restrict__ ctrl, const SortArrays arrs, uint64_t n,
                                                     uint32_t elem_bytes) {
    copy_step(ctrl, arrs, n, elem_bytes);
}

// ---- the onesweep scatter pass ----------------------------------------------------------------

// Tile geometry: THREADS threads (a multiple of 256 is not required, but at least 256: thread d
// owns digit d in the per-digit phases), ITEMS keys per thread, TILE = THREADS * ITEMS keys.
template <typename U, bool HAS_VAL, int THREADS, int ITEMS>
struct OnesweepSmem {
    static constexpr int kTile = THREADS * ITEMS;
    static constexpr int kWarps = THREADS / 32;
    static constexpr size_t kStageK = size_t(kTile) * sizeof(U);
    static constexpr size_t kStageV = HAS_VAL ? size_t(kTile) * 8 : 0;
    static constexpr size_t kOffV = (kStageK + 15) & ~size_t(15);
    static constexpr size_t kOffWofs = kOffV + kStageV;                       // u32: the TileRank table
    static constexpr size_t kOffGofs = kOffWofs + size_t(THREADS / 16) * kBuckets * 4; // i64 [256]
    static constexpr size_t kOffBstart = kOffGofs + kBuckets * 8;              // u64 [256]
    static constexpr size_t kOffMisc = kOffBstart + kBuckets * 8;              // u32 [16]
    static constexpr size_t kBytes = kOffMisc + 64;
};

// the digit of key k for this pass: filtered key (compile-time mode), byte `pass`, complemented
// for descending sorts (dmask = 0xFF) -- the descending order is the ascending order of ~K
template <int MODE, typename U>
__device__ __forceinline__ uint32_t pass_digit(U k, int pass, uint32_t dmask) {
    return digit_of(filter_key<MODE>(k), pass) ^ dmask;
}

// ---- ranking a tile: the warp multisplit ----------------------------------------------------------
// A tile is ranked in units of LANES lanes (a half-warp or a warp): unit u = threadIdx.x / LANES owns
// the contiguous slots [u * LANES * ITEMS, (u + 1) * LANES * ITEMS), and its item i covers the slots
// u * LANES * ITEMS + LANES * i + (threadIdx.x mod LANES), so ranking in unit, item and lane order
// ranks in slot order (the sort is stable).  The lanes of a unit holding digit d in an item OR their
// bit into a mask word for d (a commutative update: the mask is exact whatever order the lanes run
// in) and read it back; a lane's rank is the unit's count of d before the item plus its peers in
// lower lanes, and the lowest peer advances the count and clears the mask for the next item.
//   Half-warp units (LANES 16) keep mask and count in one word per (unit, digit): bits 0..15 the
// mask, bits 16..31 the count.  The word read back carries the count too, and the leader's single
// add of (group size << 16) - mask advances the count and clears the mask: three shared-memory
// operations per key and no shuffle.
//   Warp units (LANES 32) keep a count word per (warp, digit) and a mask word per (warp, digit); the
// leader advances the count with one returning atomic, clears the mask and hands the old count to
// its peers with a shuffle: four operations and a shuffle per key, but half as many units to scan
// per tile, which pays for small tiles.
// Both tables take (THREADS / 16) * 256 words.  A unit holds at most LANES * ITEMS keys, so counts
// stay below 2^16.  Large tiles keep their ranks packed in registers and recompute the digit when the
// key is staged (registers are what limits them); small tiles keep (rank << 8) | digit per key.
//   Crowded passes (HOT > 0): up to two digits that hold a large share of the pass's keys (found in
// the pass's histogram) never touch the table while ranking -- many lanes of a unit holding the same
// digit would serialise on one word.  For those digits a ballot gives the unit's peers, each unit
// keeps the digit's running count in a register (the same value in all its lanes), and the unit's
// first lane stores the count into the table word afterwards, where the scan finds it: the ranks
// are the ones the table would have given.

template <int MODE, typename U>
__device__ __forceinline__ uint32_t slot_digit(const U &k, uint32_t slot, uint32_t tvalid, int pass, uint32_t dmask) {
    return slot < tvalid ? pass_digit<MODE>(k, pass, dmask) : uint32_t(kBuckets - 1);   // padding ranks last
}

// the unit size that measured faster for a tile of THREADS * ITEMS keys
template <int ITEMS>
constexpr int rank_lanes() { return ITEMS >= 16 ? 16 : 32; }

// DENSE packs the ranks of large tiles as tightly as the unit size allows and advances a half-warp
// unit's count with a plain store (the same word the add would leave: no other lane writes it before
// the next item).  It pays only where registers are scarcest: the segmented pass over 8-byte keys
// (batch of 20,000 arrays: -3.2 %, spills 36 -> 20 bytes); on the plain sorts it measured within
// +-0.6 % of the default, a net loss on the mixed workload.
template <int THREADS, int ITEMS, int LANES = rank_lanes<ITEMS>(), bool DENSE = false>
struct TileRank {
    static_assert(LANES == 16 || LANES == 32, "half-warp or warp units");
    static constexpr int kLanes = LANES;
    static constexpr int kUnits = THREADS / LANES;
    static constexpr int kShift = LANES == 16 ? 16 : 0;     // where a table word keeps the count
    static constexpr int kWords = (THREADS / 16) * kBuckets;
    static constexpr bool kPacked = ITEMS >= 12;
    // a rank within its unit is below LANES * ITEMS: dense packing takes fields of 8 bits (units of
    // up to 256 keys, four to a register) or 10 bits (up to 1024, three), the default 16 bits (two)
    static constexpr int kRankBits = !DENSE ? 16 : (LANES * ITEMS <= 256 ? 8 : (LANES * ITEMS <= 1024 ? 10 : 16));
    static constexpr int kPerReg = 32 / kRankBits;
    static constexpr int kRankRegs = kPacked ? (ITEMS + kPerReg - 1) / kPerReg : ITEMS;

    __device__ static uint32_t slot0() { return (threadIdx.x / LANES) * LANES * ITEMS + threadIdx.x % LANES; }
    // the unit's count (later offset) words
    __device__ static uint32_t *row(uint32_t *tab) { return tab + (threadIdx.x / LANES) * kBuckets; }

    // rank this lane's ITEMS keys within its unit (the unit's masks clear, its counts zero); with
    // HOT > 0 the digits in `hot` ((digit1 << 16) | digit0, kNoHot for none) are ranked by ballots
    template <int MODE, int HOT = 0, typename U>
    __device__ static void rank(const U (&keys)[ITEMS], uint32_t (&rk)[kRankRegs], uint32_t *tab, uint32_t slot0,
                                uint32_t tvalid, int pass, uint32_t dmask, uint32_t hot = kNoHotPair) {
        uint32_t *crow = row(tab);
        const uint32_t bit = 1u << (threadIdx.x % LANES), below = bit - 1u;
        // this unit's lanes within a warp ballot
        const uint32_t ushift = LANES == 16 ? (threadIdx.x & 16u) : 0u;
        const uint32_t umask = LANES == 16 ? 0xFFFFu : 0xFFFFFFFFu;
        const uint32_t h0 = hot & 0xFFFFu, h1 = hot >> 16;
        uint32_t hc0 = 0, hc1 = 0;          // the unit's running counts of the hot digits
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t d = slot_digit<MODE>(keys[i], slot0 + uint32_t(LANES) * i, tvalid, pass, dmask);
            bool is_hot = false;
            uint32_t rh = 0;
            if constexpr (HOT > 0) {
                const uint32_t b0 = (__ballot_sync(0xFFFFFFFFu, d == h0) >> ushift) & umask;
                if (d == h0) {
                    rh = hc0 + uint32_t(__popc(b0 & below));
                    is_hot = true;
                }
                hc0 += uint32_t(__popc(b0));
                if constexpr (HOT > 1) {
                    const uint32_t b1 = (__ballot_sync(0xFFFFFFFFu, d == h1) >> ushift) & umask;
                    if (d == h1) {
                        rh = hc1 + uint32_t(__popc(b1 & below));
                        is_hot = true;
                    }
                    hc1 += uint32_t(__popc(b1));
                }
            }
            uint32_t r;
            if constexpr (LANES == 16) {
                if (!is_hot) atomicOr(crow + d, bit);
                __syncwarp();
                const uint32_t w = is_hot ? 0u : crow[d];
                __syncwarp();
                const uint32_t peers = w & 0xFFFFu;
                const uint32_t lower = uint32_t(__popc(peers & below));
                if (!is_hot && lower == 0) {
                    if constexpr (DENSE) crow[d] = ((w >> 16) + uint32_t(__popc(peers))) << 16;
                    else atomicAdd(crow + d, (uint32_t(__popc(peers)) << 16) - peers);
                }
                __syncwarp();      // the cleared mask is visible to the next item's updates
                r = is_hot ? rh : (w >> 16) + lower;
            } else {
                uint32_t *mrow = tab + (THREADS / 32) * kBuckets + (threadIdx.x / 32) * kBuckets;
                if (!is_hot) atomicOr(mrow + d, bit);
                __syncwarp();
                const uint32_t peers = is_hot ? 0u : mrow[d];
                __syncwarp();
                const uint32_t lower = uint32_t(__popc(peers & below));
                uint32_t before = 0;
                if (!is_hot && lower == 0) {
                    before = atomicAdd(crow + d, uint32_t(__popc(peers)));
                    mrow[d] = 0u;
                }
                __syncwarp();
                const uint32_t src = peers ? uint32_t(__ffs(peers) - 1) : 0u;
                const uint32_t b = __shfl_sync(0xFFFFFFFFu, before, src);
                r = is_hot ? rh : b + lower;
            }
            if constexpr (!kPacked) rk[i] = (r << 8) | d;
            else if (i % kPerReg != 0) rk[i / kPerReg] |= r << (kRankBits * (i % kPerReg));
            else rk[i / kPerReg] = r;
        }
        if constexpr (HOT > 0) {
            // the hot digits' unit counts go where the table keeps counts (their words are zero)
            if (threadIdx.x % LANES == 0) {
                if (h0 < kBuckets) crow[h0] = hc0 << kShift;
                if (HOT > 1 && h1 < kBuckets) crow[h1] = hc1 << kShift;
            }
        }
    }

    __device__ static uint32_t rank_of(const uint32_t (&rk)[kRankRegs], int i) {
        if constexpr (!kPacked) return rk[i] >> 8;
        else return (rk[i / kPerReg] >> (kRankBits * (i % kPerReg))) & ((1u << kRankBits) - 1u);
    }

    // the digit item i was ranked under (slot = its slot in the tile)
    template <int MODE, typename U>
    __device__ static uint32_t digit_of_item(const uint32_t (&rk)[kRankRegs], int i, const U &k, uint32_t slot,
                                             uint32_t tvalid, int pass, uint32_t dmask) {
        if constexpr (!kPacked) return rk[i] & 0xFFu;
        else return slot_digit<MODE>(k, slot, tvalid, pass, dmask);
    }

    // digit d's count in the tile: the sum over the units
    __device__ static uint32_t total(const uint32_t *tab, int d) {
        uint32_t run = 0;
#pragma unroll
        for (int u = 0; u < kUnits; ++u) run += tab[u * kBuckets + d] >> kShift;
        return run;
    }

    // digit d's count over the units [U0, U1)
    template <int U0, int U1>
    __device__ static uint32_t total_of(const uint32_t *tab, int d) {
        uint32_t run = 0;
#pragma unroll
        for (int u = U0; u < U1; ++u) run += tab[u * kBuckets + d] >> kShift;
        return run;
    }

    // replace digit d's unit counts by the units' staging offsets, the first one at the tile start ts
    __device__ static void offsets(uint32_t *tab, int d, uint32_t ts) { offsets_of<0, kUnits>(tab, d, ts); }

    // the same for the units [U0, U1), the first of them starting at ts
    template <int U0, int U1>
    __device__ static void offsets_of(uint32_t *tab, int d, uint32_t ts) {
#pragma unroll
        for (int u = U0; u < U1; ++u) {
            const uint32_t c = tab[u * kBuckets + d] >> kShift;
            tab[u * kBuckets + d] = ts;
            ts += c;
        }
    }

    // a warp zeroes its units' offset words once its keys are staged, ready for the next tile
    // (the masks are clear already)
    __device__ static void clear_own(uint32_t *tab) {
        uint32_t *rows = tab + (threadIdx.x / 32) * (32 / LANES) * kBuckets;
        __syncwarp();
#pragma unroll
        for (int i = threadIdx.x % 32; i < (32 / LANES) * kBuckets; i += 32) rows[i] = 0u;
    }
};

// ---- tile loads --------------------------------------------------------------------------------
// This lane's ITEMS elements of a tile of `tile` slots: item i is slot slot0 + LANES * i, the
// element tbase + slot of the array, or element n - 1 - (tbase + slot) when the pass reads back to
// front; slots past tvalid (the array's end) get `fill`.  A full tile loads without checks, in
// either direction.
template <int ITEMS, int LANES, typename T>
__device__ __forceinline__ void load_items(T (&v)[ITEMS], const T *src, uint64_t n, uint64_t tbase, uint32_t slot0,
                                           uint32_t tvalid, uint32_t tile, bool reverse, T fill) {
    if (tvalid == tile) {
        if (!reverse) {
            const T *p = src + tbase + slot0;
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) v[i] = p[size_t(i) * LANES];
        } else {
            const T *p = src + (n - 1u - tbase - slot0);
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) v[i] = *(p - size_t(i) * LANES);
        }
    } else {
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t slot = slot0 + uint32_t(i) * LANES;
            const uint64_t gi = tbase + slot;
            v[i] = slot < tvalid ? src[reverse ? (n - 1u - gi) : gi] : fill;
        }
    }
}

// ---- tile prefetch ---------------------------------------------------------------------------------
// Ask the L2 for elements [0, count) of p ahead of their loads: one bulk prefetch (the copy engine
// fetches it while the SM works on the tile before), trimmed inward to 16-byte boundaries so it
// never touches bytes outside the array.  count * sizeof(T) is one tile: far below 2^32.
template <typename T>
__device__ __forceinline__ void prefetch_l2(const T *p, uint64_t count) {
    uint64_t a = reinterpret_cast<uint64_t>(p), b = a + count * sizeof(T);
    a = (a + 15u) & ~uint64_t(15);
    b &= ~uint64_t(15);
    if (b > a) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(uint32_t(b - a)) : "memory");
}

// the elements of tile `tile` (TILE slots) of an n-element array, read forwards or back to front
template <int TILE, typename T>
__device__ __forceinline__ void prefetch_tile(const T *src, uint64_t n, uint32_t tile, bool reverse) {
    const uint64_t first = uint64_t(tile) * TILE;
    if (first >= n) return;
    const uint64_t cnt = (n - first) < uint64_t(TILE) ? (n - first) : uint64_t(TILE);
    prefetch_l2(reverse ? src + (n - first - cnt) : src + first, cnt);
}

// ---- decoupled look-back -------------------------------------------------------------------------
// load the status words of digit d for tiles j, j-1, ..., j-W+1 (none below tile 0)
template <int W, typename S>
__device__ __forceinline__ void lookback_load(const S *status, int64_t j, int d, S (&w)[W]) {
#pragma unroll
    for (int q = 0; q < W; ++q) w[q] = (j - q >= 0) ? ld_relaxed(status + size_t(j - q) * kBuckets + d) : S(0);
}

// Walk back from tile `tile` - 1 for digit d, starting from the window `w` already loaded for the
// tiles tile-1 ... tile-W: add the predecessors' aggregates to `excl` until an inclusive prefix;
// an unpublished predecessor is re-read (a bounded wait: past spin_limit ns, or once another CTA
// has aborted, the pass is flagged and the walk gives up).  A window may have been loaded early:
// a published word only ever changes from aggregate to inclusive, and either adds up to the same
// prefix.  Returns false if the walk gave up.
template <int W, typename S>
__device__ __forceinline__ bool lookback_walk(const S *status, uint32_t tile, int d, S (&w)[W], uint64_t &excl,
                                              uint32_t *err_word, uint32_t *abort_word, uint64_t spin_limit) {
    int64_t j = int64_t(tile) - 1;
    uint32_t spins = 0;
    uint64_t t0 = 0;
    while (j >= 0) {
        int q = 0;
        for (; q < W && j - q >= 0; ++q) {
            const uint32_t st = StatusWord<S>::state(w[q]);
            if (st == kStInvalid) break;
            excl += StatusWord<S>::value(w[q]);
            if (st == kStInclusive) return true;
        }
        if (q == W) {           // a window of aggregates: keep walking back
            j -= W;
        } else {                // wait on the first unpublished predecessor
            j -= q;
            if (++spins > 16u) {
                if (*reinterpret_cast<volatile uint32_t *>(abort_word)) return false;
                const uint64_t now = globaltimer_ns();
                if (t0 == 0) t0 = now;
                else if (now - t0 > spin_limit) {
                    atomicOr(err_word, kDevTimeout);
                    atomicExch(abort_word, 1u);
                    return false;
                }
                __nanosleep(32);
            }
        }
        lookback_load(status, j, d, w);
    }
    return true;
}

// the signed offset from a staged slot to its output position: 32-bit while every count fits the
// 30-bit look-back words (sorts of fewer than 2^30 keys), 64-bit beyond
template <typename S>
using TileOffset = std::conditional_t<std::is_same_v<S, uint32_t>, int32_t, long long>;

template <typename U, bool HAS_VAL, int THREADS>
constexpr int onesweep_min_blocks() {
    return THREADS >= 512 ? 2 : (HAS_VAL ? 3 : (sizeof(U) <= 4 ? 4 : 3));
}

// one tile of one scatter pass, relative to the array (or segment) it belongs to
template <typename U, typename S>
struct SweepTile {
    const U *src_k;
    U *dst_k;                 // null: keys are dropped (last pass of an indirect sort)
    const uint64_t *src_v;
    uint64_t *dst_v;
    S *status;                // look-back words of tile 0 of this array / segment
    uint64_t n;               // elements of the array / segment
    uint32_t tile;            // tile index within the array / segment
    bool reverse;             // read the source back to front
};

// Process one tile: load, rank (half-warp multisplit), publish and resolve the look-back, stage sorted
// by digit in shared memory, write out.  `bstart` (shared) holds the bucket starts of this pass for
// the array / segment.  Called by all threads; ends with a barrier.
template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S, int HOT = 0>
__device__ __forceinline__ void sweep_tile(unsigned char *smem, const SweepTile<U, S> &t,
                                           const unsigned long long *bstart, int pass, uint32_t dmask,
                                           uint32_t *err_word, uint32_t *abort_word, uint64_t spin_limit,
                                           uint32_t stall_tile, uint32_t hot = kNoHotPair) {
    using L = OnesweepSmem<U, HAS_VAL, THREADS, ITEMS>;
    constexpr int TILE = L::kTile;
    using R = TileRank<THREADS, ITEMS>;
    U *stage_k = reinterpret_cast<U *>(smem);
    uint64_t *stage_v = reinterpret_cast<uint64_t *>(smem + L::kOffV);
    uint32_t *wofs = reinterpret_cast<uint32_t *>(smem + L::kOffWofs);
    using G = TileOffset<S>;
    G *gofs = reinterpret_cast<G *>(smem + L::kOffGofs);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);  // [1] bad [2..9] scan
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t *urow = R::row(wofs);
    const uint32_t tile = t.tile;
    const uint64_t n = t.n;
    const uint64_t tbase = uint64_t(tile) * TILE;
    const uint32_t tvalid = uint32_t((n - tbase) < uint64_t(TILE) ? (n - tbase) : uint64_t(TILE));

    // load ITEMS keys per thread: item i of this lane is slot R::slot0() + R::kLanes * i (see TileRank).
    // Slots past the end get digit 255: they rank after every real key of the tile.
    U keys[ITEMS];
    uint64_t vals[HAS_VAL ? ITEMS : 1];
    uint32_t rk[R::kRankRegs];
    const uint32_t slot0 = R::slot0();
    load_items<ITEMS, R::kLanes>(keys, t.src_k, n, tbase, slot0, tvalid, TILE, t.reverse, KeyTraits<U>::fill());
    if constexpr (HAS_VAL) load_items<ITEMS, R::kLanes>(vals, t.src_v, n, tbase, slot0, tvalid, TILE, t.reverse, uint64_t(0));
    R::template rank<MODE, HOT>(keys, rk, wofs, slot0, tvalid, pass, dmask, hot);
    __syncthreads();

    // per digit: the tile count; publish the aggregate
    uint32_t count = 0, x = 0, run = 0;
    if (tid < kBuckets) {
        run = R::total(wofs, tid);
        count = run;
        if (tid == kBuckets - 1) count -= uint32_t(TILE) - tvalid;   // the padding slots
        if (tile != stall_tile)
            st_relaxed(t.status + size_t(tile) * kBuckets + tid,
                       StatusWord<S>::make(tile == 0 ? kStInclusive : kStAggregate, count));
        x = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) misc[2 + warp] = x;
    }
    __syncthreads();
    if (tid < kBuckets) {
        uint32_t before = 0;
        for (int i = 0; i < warp; ++i) before += misc[2 + i];
        const uint32_t ts = before + x - run;          // tile start of digit tid
        R::offsets(wofs, tid, ts);
        // decoupled look-back for digit tid: read predecessors kWin at a time (bounded wait)
        uint64_t excl = 0;
        bool bad = false;
        if (tile > 0) {
            constexpr int kWin = sizeof(U) <= 4 ? 4 : 8;   // measured best per key size
            S w[kWin];
            lookback_load(t.status, int64_t(tile) - 1, tid, w);
            bad = !lookback_walk(t.status, tile, tid, w, excl, err_word, abort_word, spin_limit);
            if (tile != stall_tile)
                st_relaxed(t.status + size_t(tile) * kBuckets + tid,
                           StatusWord<S>::make(kStInclusive, excl + count));
        }
        if (bad) misc[1] = 1u;
        gofs[tid] = G((long long)(bstart[tid] + excl) - (long long)ts);
    }
    __syncthreads();
    const bool tile_bad = misc[1] != 0 || tile == stall_tile;

    // stage the tile in shared memory, sorted by digit (padding slots land past tvalid)
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const uint32_t d = R::template digit_of_item<MODE>(rk, i, keys[i], slot0 + uint32_t(R::kLanes) * i, tvalid, pass, dmask);
        const uint32_t pos = urow[d] + R::rank_of(rk, i);
        stage_k[pos] = keys[i];
        if constexpr (HAS_VAL) stage_v[pos] = vals[i];
    }
    R::clear_own(wofs);
    __syncthreads();
    // write out: consecutive threads take consecutive slots of a bucket run
    if (!tile_bad) {
        if (tvalid == TILE) {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t s = uint32_t(tid) + uint32_t(i) * THREADS;
                const U k = stage_k[s];
                const G g = gofs[pass_digit<MODE>(k, pass, dmask)] + G(s);
                if (uint64_t(g) < n) {
                    if (t.dst_k) t.dst_k[g] = k;
                    if constexpr (HAS_VAL) t.dst_v[g] = stage_v[s];
                } else {
                    atomicOr(err_word, kDevFault);      // an offset outside the array: flagged, not written
                }
            }
        } else {
            for (uint32_t s = tid; s < tvalid; s += THREADS) {
                const U k = stage_k[s];
                const G g = gofs[pass_digit<MODE>(k, pass, dmask)] + G(s);
                if (uint64_t(g) < n) {
                    if (t.dst_k) t.dst_k[g] = k;
                    if constexpr (HAS_VAL) t.dst_v[g] = stage_v[s];
                } else {
                    atomicOr(err_word, kDevFault);      // an offset outside the array: flagged, not written
                }
            }
        }
    }
    __syncthreads();
}

template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S>
__device__ __forceinline__ void sweep_init_smem(unsigned char *smem) {
    using L = OnesweepSmem<U, HAS_VAL, THREADS, ITEMS>;
    uint32_t *wofs = reinterpret_cast<uint32_t *>(smem + L::kOffWofs);
    for (int i = threadIdx.x; i < (THREADS / 16) * kBuckets; i += THREADS) wofs[i] = 0u;
}

template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S, int HOT>
__device__ __forceinline__ void onesweep_body(unsigned char *smem, Control *__restrict__ ctrl,
                                              const PassPlan &plan, const SortArrays &arrs,
                                              const unsigned long long *__restrict__ bstart_all,
                                              S *__restrict__ status, int pass, uint64_t n, uint32_t num_tiles,
                                              uint32_t dmask) {
    using L = OnesweepSmem<U, HAS_VAL, THREADS, ITEMS>;
    unsigned long long *bstart = reinterpret_cast<unsigned long long *>(smem + L::kOffBstart);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);
    SweepTile<U, S> t;
    bool bad = false;
    t.src_k = static_cast<const U *>(sort_array(arrs, plan.src_keys, HAS_VAL ? kArrKeysA : kArrIn, &bad));
    t.dst_k = static_cast<U *>(sort_array(arrs, plan.dst_keys, HAS_VAL ? kArrKeysB : kArrBuf, &bad));
    t.src_v = static_cast<const uint64_t *>(sort_array(arrs, plan.src_vals, kArrIn, &bad));
    t.dst_v = static_cast<uint64_t *>(sort_array(arrs, plan.dst_vals, kArrBuf, &bad));
    if (bad || !t.src_k || (HAS_VAL ? (!t.src_v || !t.dst_v) : !t.dst_k)) {   // a damaged control block
        if (threadIdx.x == 0) atomicOr(&ctrl->error, kDevFault);
        return;
    }
    t.status = status;
    t.n = n;
    t.reverse = plan.reverse != 0;
    const uint64_t spin_limit = ctrl->spin_limit_ns;
    const uint32_t stall_tile = ctrl->stall_tile;
    const bool prefetch = ctrl->prefetch != 0;
    for (int i = threadIdx.x; i < kBuckets; i += THREADS) bstart[i] = bstart_all[pass * kBuckets + i];
    sweep_init_smem<U, MODE, HAS_VAL, THREADS, ITEMS, S>(smem);
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t tile = atomicAdd(&ctrl->tile_counter[pass], 1u);
            misc[0] = tile;
            misc[1] = 0;
            // the tile one grid stride on is about the next one any CTA claims: its data go to L2 now
            const uint32_t ahead = tile + gridDim.x;
            if (prefetch && ahead < num_tiles) {
                constexpr int TILE = L::kTile;
                prefetch_tile<TILE>(t.src_k, n, ahead, t.reverse);
                if constexpr (HAS_VAL) prefetch_tile<TILE>(t.src_v, n, ahead, t.reverse);
            }
        }
        __syncthreads();
        const uint32_t tile = misc[0];
        if (tile >= num_tiles) break;
        t.tile = tile;
        sweep_tile<U, MODE, HAS_VAL, THREADS, ITEMS, S, HOT>(smem, t, bstart, pass, dmask, &ctrl->error,
                                                             &ctrl->abort, spin_limit, stall_tile, plan.hot);
    }
}

template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S>
__global__ void __launch_bounds__(THREADS, onesweep_min_blocks<U, HAS_VAL, THREADS>())
    k_onesweep(Control *__restrict__ ctrl, const SortArrays arrs, const unsigned long long *__restrict__ bstart_all,
               S *__restrict__ status, int pass, uint64_t n, uint32_t num_tiles, uint32_t dmask, uint32_t fold_copy) {
    using L = OnesweepSmem<U, HAS_VAL, THREADS, ITEMS>;
    static_assert(THREADS >= kBuckets && THREADS % 32 == 0, "one thread per digit");
    static_assert(L::kTile <= 65535, "tile ranks are 16-bit");
    extern __shared__ __align__(16) unsigned char smem[];
    const PassPlan plan = ctrl->plan[pass];
    if (!plan.active) {
        // the last pass of a copy form: when every pass was skipped, the copy the plan asks for
        if (fold_copy) copy_step(ctrl, arrs, n, HAS_VAL ? 8u : uint32_t(sizeof(U)));
        return;
    }
    // a crowded pass ranks its hot digits with ballots (the choice is uniform over the launch)
    if (plan.hot == kNoHotPair)
        onesweep_body<U, MODE, HAS_VAL, THREADS, ITEMS, S, 0>(smem, ctrl, plan, arrs, bstart_all, status, pass, n, num_tiles,
                                                              dmask);
    else
        onesweep_body<U, MODE, HAS_VAL, THREADS, ITEMS, S, 1>(smem, ctrl, plan, arrs, bstart_all, status, pass, n, num_tiles,
                                                              dmask);
}

// ---- the pipelined scatter pass -----------------------------------------------------------------
// Tile B is loaded and ranked while tile A, ranked one iteration earlier and staged in shared
// memory, waits for its look-back; A's look-back then runs in threads 256..511 while threads 0..255
// scan B's counts, and A is written out while B's offsets are finished.  The look-back wait of one
// tile overlaps the load and ranking of the next (four CTA barriers per tile instead of six).
// Stability and the output are those of k_onesweep: the same slots, ranks and stores, one tile
// later.  Progress: a CTA's pending tile A only waits on earlier tiles, and ranking B waits on
// nothing, so the lowest unresolved tile always resolves.  Tile B's unit words are scanned into
// offsets in (3a) and cleared by each warp once B is staged in (4), so one table serves every tile.

template <typename U, int THREADS, int ITEMS, bool HAS_VAL = false>
struct PipeSmem {
    static constexpr int kTile = THREADS * ITEMS;
    static constexpr int kWarps = THREADS / 32;
    static constexpr size_t kStageK = size_t(kTile) * sizeof(U);
    static constexpr size_t kOffV = (kStageK + 15) & ~size_t(15);     // u64 [TILE]: the staged pointers
    static constexpr size_t kOffUnits = kOffV + (HAS_VAL ? size_t(kTile) * 8 : 0);  // u32: the TileRank table
    static constexpr size_t kOffGofs = kOffUnits + size_t(THREADS / 16) * kBuckets * 4;   // i64 [256] of tile A
    static constexpr size_t kOffBstart = kOffGofs + kBuckets * 8;     // u64 [256]
    static constexpr size_t kOffTs = kOffBstart + kBuckets * 8;       // u32 [2][256] tile starts
    static constexpr size_t kOffCnt = kOffTs + 2 * kBuckets * 4;      // u32 [2][256] tile counts
    static constexpr size_t kOffMisc = kOffCnt + 2 * kBuckets * 4;    // u32 [32]
    static constexpr size_t kOffAux = kOffMisc + 128;                 // 128 B for the kernel's own use
    static constexpr size_t kOffHalf = kOffAux + 128;                 // u32 [2][256]: split offset scan
    static constexpr size_t kBytes = kOffHalf + 2 * kBuckets * 4;
};

template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S, int HOT>
__device__ __forceinline__ void onesweep_pipe_body(unsigned char *smem, Control *__restrict__ ctrl, const PassPlan &plan,
                                                   const SortArrays &arrs,
                                                   const unsigned long long *__restrict__ bstart_all,
                                                   S *__restrict__ status, int pass, uint64_t n, uint32_t num_tiles,
                                                   uint32_t dmask) {
    using L = PipeSmem<U, THREADS, ITEMS, HAS_VAL>;
    constexpr int TILE = L::kTile;
    using R = TileRank<THREADS, ITEMS>;
    const uint32_t hot = plan.hot;
    U *stage = reinterpret_cast<U *>(smem);
    uint64_t *stage_v = reinterpret_cast<uint64_t *>(smem + L::kOffV);
    uint32_t *utab = reinterpret_cast<uint32_t *>(smem + L::kOffUnits);
    using G = TileOffset<S>;
    G *gofs = reinterpret_cast<G *>(smem + L::kOffGofs);
    unsigned long long *bstart = reinterpret_cast<unsigned long long *>(smem + L::kOffBstart);
    uint32_t *tsall = reinterpret_cast<uint32_t *>(smem + L::kOffTs);
    uint32_t *cntall = reinterpret_cast<uint32_t *>(smem + L::kOffCnt);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);   // [0] next tile [1] bad [2..9] scan
    // with 32 ranking units, all 512 threads write B's unit offsets in (3a), 16 units each: thread d
    // the first half, thread d + 256 the second, from the digit's prefix and first-half count here
    constexpr bool kSplit = R::kUnits == 32;
    uint32_t *half = reinterpret_cast<uint32_t *>(smem + L::kOffHalf);

    bool bad_plan = false;
    const U *src = static_cast<const U *>(sort_array(arrs, plan.src_keys, HAS_VAL ? kArrKeysA : kArrIn, &bad_plan));
    U *dst = static_cast<U *>(sort_array(arrs, plan.dst_keys, HAS_VAL ? kArrKeysB : kArrBuf, &bad_plan));  // null: keys
                                                                       // are dropped (last pass of an indirect sort)
    const uint64_t *src_v = static_cast<const uint64_t *>(sort_array(arrs, plan.src_vals, kArrIn, &bad_plan));
    uint64_t *dst_v = static_cast<uint64_t *>(sort_array(arrs, plan.dst_vals, kArrBuf, &bad_plan));
    if (bad_plan || !src || (HAS_VAL ? (!src_v || !dst_v) : !dst)) {   // a damaged control block
        if (threadIdx.x == 0) atomicOr(&ctrl->error, kDevFault);
        return;
    }
    const bool reverse = plan.reverse != 0;
    const uint64_t spin_limit = ctrl->spin_limit_ns;
    const uint32_t stall_tile = ctrl->stall_tile;
    const bool prefetch = ctrl->prefetch != 0;
    uint32_t *err_word = &ctrl->error;
    uint32_t *abort_word = &ctrl->abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t *urow = R::row(utab);
    const uint32_t slot0 = R::slot0();

    for (int i = tid; i < kBuckets; i += THREADS) bstart[i] = bstart_all[pass * kBuckets + i];
    for (int i = tid; i < R::kWords; i += THREADS) utab[i] = 0u;
    if (tid == 0) {
        misc[0] = atomicAdd(&ctrl->tile_counter[pass], 1u);
        misc[1] = 0u;
    }
    __syncthreads();
    uint32_t tileB = misc[0];
    bool hasA = false;
    uint32_t tileA = 0, tvalidA = 0;
    int par = 0;                       // ts / count parity of tile B
    for (;;) {
        const bool hasB = tileB < num_tiles;
        if (!hasA && !hasB) break;
        uint32_t *tsB = tsall + par * kBuckets, *tsA = tsall + (par ^ 1) * kBuckets;
        uint32_t *cntB = cntall + par * kBuckets, *cntA = cntall + (par ^ 1) * kBuckets;
        uint32_t next = 0xFFFFFFFFu;
        if (hasB && tid == 0) {
            next = atomicAdd(&ctrl->tile_counter[pass], 1u);   // the tile after B: its keys go to L2 now
            if (prefetch && next < num_tiles) {
                prefetch_tile<TILE>(src, n, next, reverse);
                if constexpr (HAS_VAL) prefetch_tile<TILE>(src_v, n, next, reverse);
            }
        }
        // the look-back threads load A's first window now: the loads complete while B is ranked
        constexpr int kWin = sizeof(U) <= 8 ? 4 : 8;   // measured best per key size
        S lbw[kWin];
        if (hasA && tid >= kBuckets && tileA > 0) lookback_load(status, int64_t(tileA) - 1, tid - kBuckets, lbw);

        // ---- (1) load and rank tile B (the units of sweep_tile)
        U keys[ITEMS];
        uint64_t vals[HAS_VAL ? ITEMS : 1];
        uint32_t rk[R::kRankRegs];
        uint32_t tvalidB = 0;
        if (hasB) {
            const uint64_t tbase = uint64_t(tileB) * TILE;
            tvalidB = uint32_t((n - tbase) < uint64_t(TILE) ? (n - tbase) : uint64_t(TILE));
            load_items<ITEMS, R::kLanes>(keys, src, n, tbase, slot0, tvalidB, TILE, reverse, KeyTraits<U>::fill());
            if constexpr (HAS_VAL) load_items<ITEMS, R::kLanes>(vals, src_v, n, tbase, slot0, tvalidB, TILE, reverse, uint64_t(0));
            R::template rank<MODE, HOT>(keys, rk, utab, slot0, tvalidB, pass, dmask, hot);
        }
        __syncthreads();                                                        // barrier 1

        // ---- (2a) threads 0..255: B's count of digit tid, publish B's aggregate
        //      (2b) threads 256..511: A's look-back for digit tid - 256, publish A's inclusive prefix
        uint32_t x = 0, run = 0;
        if (tid < kBuckets) {
            if (hasB) {
                uint32_t h0 = 0;
                if constexpr (kSplit) {
                    h0 = R::template total_of<0, R::kUnits / 2>(utab, tid);
                    run = h0 + R::template total_of<R::kUnits / 2, R::kUnits>(utab, tid);
                } else {
                    run = R::total(utab, tid);
                }
                uint32_t count = run;
                if (tid == kBuckets - 1) count -= uint32_t(TILE) - tvalidB;      // the padding slots
                cntB[tid] = count;
                if (tileB != stall_tile)
                    st_relaxed(status + size_t(tileB) * kBuckets + tid,
                               StatusWord<S>::make(tileB == 0 ? kStInclusive : kStAggregate, count));
                x = run;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) misc[2 + warp] = x;
                if constexpr (kSplit) {
                    half[tid] = x - run;              // the digit's prefix within its scan warp
                    half[kBuckets + tid] = h0;
                }
            }
        } else if (hasA) {
            const int d = tid - kBuckets;
            const uint32_t count = cntA[d];
            uint64_t excl = 0;
            bool bad = false;
            if (tileA > 0) {
                bad = !lookback_walk(status, tileA, d, lbw, excl, err_word, abort_word, spin_limit);
                if (tileA != stall_tile)
                    st_relaxed(status + size_t(tileA) * kBuckets + d, StatusWord<S>::make(kStInclusive, excl + count));
            }
            if (bad) misc[1] = 1u;
            gofs[d] = G((long long)(bstart[d] + excl) - (long long)tsA[d]);
        }
        __syncthreads();                                                        // barrier 2

        // ---- (3a) B's tile starts and unit offsets; (3b) all: write A out
        if constexpr (kSplit) {
            if (hasB) {
                const int d = tid & (kBuckets - 1);
                uint32_t before = 0;
                for (int i = 0; i < (d >> 5); ++i) before += misc[2 + i];
                const uint32_t ts = before + half[d];
                if (tid < kBuckets) {
                    R::template offsets_of<0, R::kUnits / 2>(utab, d, ts);
                    tsB[d] = ts;
                } else {
                    R::template offsets_of<R::kUnits / 2, R::kUnits>(utab, d, ts + half[kBuckets + d]);
                }
            }
        } else if (tid < kBuckets && hasB) {
            uint32_t before = 0;
            for (int i = 0; i < warp; ++i) before += misc[2 + i];
            const uint32_t ts = before + x - run;
            R::offsets(utab, tid, ts);
            tsB[tid] = ts;
        }
        if (hasA && misc[1] == 0u && tileA != stall_tile) {
            if (tvalidA == TILE) {
#pragma unroll 4
                for (int i = 0; i < ITEMS; ++i) {
                    const uint32_t s = uint32_t(tid) + uint32_t(i) * THREADS;
                    const U k = stage[s];
                    const G g = gofs[pass_digit<MODE>(k, pass, dmask)] + G(s);
                    if (uint64_t(g) < n) {
                        if (!HAS_VAL || dst) dst[g] = k;
                        if constexpr (HAS_VAL) dst_v[g] = stage_v[s];
                    } else {
                        atomicOr(err_word, kDevFault);  // an offset outside the array: flagged, not written
                    }
                }
            } else {
                for (uint32_t s = tid; s < tvalidA; s += THREADS) {
                    const U k = stage[s];
                    const G g = gofs[pass_digit<MODE>(k, pass, dmask)] + G(s);
                    if (uint64_t(g) < n) {
                        if (!HAS_VAL || dst) dst[g] = k;
                        if constexpr (HAS_VAL) dst_v[g] = stage_v[s];
                    } else {
                        atomicOr(err_word, kDevFault);  // an offset outside the array: flagged, not written
                    }
                }
            }
        }
        __syncthreads();                                                        // barrier 3

        // ---- (4) stage B sorted by digit (padding slots land past tvalidB); clear the unit words
        if (hasB) {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t d = R::template digit_of_item<MODE>(rk, i, keys[i], slot0 + uint32_t(R::kLanes) * i, tvalidB, pass, dmask);
                const uint32_t pos = urow[d] + R::rank_of(rk, i);
                stage[pos] = keys[i];
                if constexpr (HAS_VAL) stage_v[pos] = vals[i];
            }
            R::clear_own(utab);
        }
        if (tid == 0) {
            misc[0] = next;
            misc[1] = 0u;
        }
        __syncthreads();                                                        // barrier 4
        hasA = hasB;
        tileA = tileB;
        tvalidA = tvalidB;
        par ^= 1;
        tileB = hasB ? misc[0] : num_tiles;
    }
}

template <typename U, int MODE, bool HAS_VAL, int THREADS, int ITEMS, typename S>
__global__ void __launch_bounds__(THREADS, 2)
    k_onesweep_pipe(Control *__restrict__ ctrl, const SortArrays arrs, const unsigned long long *__restrict__ bstart_all,
                    S *__restrict__ status, int pass, uint64_t n, uint32_t num_tiles, uint32_t dmask,
                    uint32_t fold_copy) {
    static_assert(THREADS == 2 * kBuckets, "threads 0..255 scan, threads 256..511 look back");
    static_assert(PipeSmem<U, THREADS, ITEMS, HAS_VAL>::kTile <= 65535, "tile ranks are 16-bit");
    extern __shared__ __align__(16) unsigned char smem[];
    const PassPlan plan = ctrl->plan[pass];
    if (!plan.active) {
        // the last pass of a copy form: when every pass was skipped, the copy the plan asks for
        if (fold_copy) copy_step(ctrl, arrs, n, HAS_VAL ? 8u : uint32_t(sizeof(U)));
        return;
    }
    // a crowded pass ranks its hot digits with ballots (the choice is uniform over the launch)
    if (plan.hot == kNoHotPair)
        onesweep_pipe_body<U, MODE, HAS_VAL, THREADS, ITEMS, S, 0>(smem, ctrl, plan, arrs, bstart_all, status, pass, n,
                                                                   num_tiles, dmask);
    else
        onesweep_pipe_body<U, MODE, HAS_VAL, THREADS, ITEMS, S, 1>(smem, ctrl, plan, arrs, bstart_all, status, pass, n,
                                                                   num_tiles, dmask);
}


}  // namespace rsbd8g
