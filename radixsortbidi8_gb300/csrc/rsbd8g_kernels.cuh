// rsbd8g_kernels.cuh - the sm_103a kernels of the stable LSD radix sort.
//
//   k_histogram / k_gather_histogram   all 256-bin digit histograms in one read of the keys,
//                                      with warp-aggregated (__match_any_sync) shared-memory
//                                      atomics; the gather form reads the key through each
//                                      object pointer and writes the filtered keys once
//   k_plan                             exclusive scan of every digit histogram, the reference's
//                                      pass-skip test, and the ping-pong plan of the passes
//   k_onesweep                         one stable scatter pass of a surviving digit: persistent
//                                      CTAs claim tiles in order, rank keys with a warp
//                                      multisplit (__match_any_sync), resolve the tile's global
//                                      bucket offsets with a bounded decoupled look-back, stage the
//                                      tile in shared memory sorted by digit and write it out
//                                      coalesced
//   k_copy                             the plain / reversed copy when parity or all-skipped
//                                      passes need one
#pragma once
#include "rsbd8g_device.cuh"

namespace rsbd8g {

// ---- up-front histograms --------------------------------------------------------------------

// add 1 to h[d] for every lane, aggregated over the lanes of the warp that share d
__device__ __forceinline__ void warp_agg_add(uint32_t *h, uint32_t d, bool valid, uint32_t lane) {
    const uint32_t key = valid ? d : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
    if (valid && lane == uint32_t(__ffs(peers) - 1)) atomicAdd(h + d, uint32_t(__popc(peers)));
}

template <typename U>
__device__ __forceinline__ void count_key(uint32_t *sh, U k, bool valid, uint32_t lane) {
#pragma unroll
    for (int p = 0; p < int(sizeof(U)); ++p) warp_agg_add(sh + p * kBuckets, digit_of(k, p), valid, lane);
}

template <int THREADS, int P>
__device__ __forceinline__ void flush_hist(const uint32_t *sh, unsigned long long *ghist) {
    __syncthreads();
    for (int i = threadIdx.x; i < P * kBuckets; i += THREADS)
        if (sh[i]) atomicAdd(ghist + i, (unsigned long long)sh[i]);
}

template <typename U, int THREADS>
__global__ void __launch_bounds__(THREADS) k_histogram(const U *__restrict__ keys, uint64_t n, Filter f,
                                                       unsigned long long *__restrict__ ghist) {
    constexpr int P = int(sizeof(U));
    constexpr int V = 16 / int(sizeof(U));
    __shared__ uint32_t sh[P * kBuckets];
    for (int i = threadIdx.x; i < P * kBuckets; i += THREADS) sh[i] = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    // scalar head up to 16-byte alignment, vector body, scalar tail
    const uint64_t mis = (reinterpret_cast<uintptr_t>(keys) & 15u) / sizeof(U);
    const uint64_t head = mis ? (uint64_t(V) - mis < n ? uint64_t(V) - mis : n) : 0;
    const uint64_t nvec = (n - head) / V;
    const uint64_t tail0 = head + nvec * V;
    const uint64_t gwarp = (uint64_t(blockIdx.x) * THREADS + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * THREADS) >> 5;
    if (gwarp == 0) {  // head and tail by the first warp of the grid
        for (uint64_t b = 0; b < head; b += 32) {
            const uint64_t i = b + lane;
            const bool ok = i < head;
            count_key(sh, sortkey(ok ? keys[i] : U(0), f), ok, lane);
        }
        for (uint64_t b = tail0; b < n; b += 32) {
            const uint64_t i = b + lane;
            const bool ok = i < n;
            count_key(sh, sortkey(ok ? keys[i] : U(0), f), ok, lane);
        }
    }
    const uint4 *kv = reinterpret_cast<const uint4 *>(keys + head);
    constexpr int UNR = 4;
    for (uint64_t b = gwarp * 32 * UNR; b < nvec; b += nwarps * 32 * UNR) {
        uint4 v[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const uint64_t i = b + u * 32 + lane;
            v[u] = i < nvec ? __ldg(kv + i) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const bool ok = b + u * 32 + lane < nvec;
            U k[V];
            memcpy(k, &v[u], 16);
#pragma unroll
            for (int j = 0; j < V; ++j) count_key(sh, sortkey(k[j], f), ok, lane);
        }
    }
    flush_hist<THREADS, P>(sh, ghist);
}

// indirect form: gather the key through each object pointer, write the filtered key
template <typename U, int THREADS>
__global__ void __launch_bounds__(THREADS) k_gather_histogram(const uint64_t *__restrict__ ptrs, uint64_t n,
                                                              Filter f, int64_t off1, int64_t off2, int level,
                                                              U *__restrict__ keys_out,
                                                              unsigned long long *__restrict__ ghist) {
    constexpr int P = int(sizeof(U));
    __shared__ uint32_t sh[P * kBuckets];
    for (int i = threadIdx.x; i < P * kBuckets; i += THREADS) sh[i] = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t gwarp = (uint64_t(blockIdx.x) * THREADS + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * THREADS) >> 5;
    constexpr int UNR = 4;
    for (uint64_t b = gwarp * 32 * UNR; b < n; b += nwarps * 32 * UNR) {
        U raw[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const uint64_t i = b + u * 32 + lane;
            raw[u] = 0;
            if (i < n) {
                const unsigned char *obj = reinterpret_cast<const unsigned char *>(ptrs[i]) + off1;
                if (level == 2) obj = load_ptr(obj) + off2;
                raw[u] = load_member<U>(obj);
            }
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const uint64_t i = b + u * 32 + lane;
            const bool ok = i < n;
            const U k = sortkey(raw[u], f);
            if (ok) keys_out[i] = k;
            count_key(sh, k, ok, lane);
        }
    }
    flush_hist<THREADS, P>(sh, ghist);
}

// ---- scan, pass-skip and plan -----------------------------------------------------------------

struct PlanArgs {
    const void *in;
    void *out;
    void *buf;
    void *keys_a;
    void *keys_b;
    uint64_t elem_bytes;   // bytes moved per element in the copy step (key bytes, or 8 for pointers)
    uint64_t spin_limit_ns;
    uint32_t inplace;      // radixsort / radixsortnoalloc: sort `in` using `buf`
    uint32_t to_buffer;    // movetobuffer
    uint32_t rev;          // effective isrevorder
    uint32_t indirect;
    uint32_t stall_tile;
    uint32_t passes;       // digits of the key
};

// one CTA of 256 threads
__global__ void __launch_bounds__(256) k_plan(Control *__restrict__ ctrl, const unsigned long long *__restrict__ ghist,
                                              unsigned long long *__restrict__ bstart, uint64_t n, PlanArgs a) {
    __shared__ unsigned long long wsum[8];
    __shared__ int skip[kMaxPasses];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int p = 0; p < int(a.passes); ++p) {
        const unsigned long long h = ghist[p * kBuckets + t];
        // pass-skip: one bucket holds every key (Radixsortbidi8.hpp:12259, :12272, :2903)
        const int all_in_one = __syncthreads_or(h == n);
        unsigned long long x = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        unsigned long long before = 0;
        for (int i = 0; i < w; ++i) before += wsum[i];
        bstart[p * kBuckets + t] = before + x - h;
        if (t == 0) skip[p] = all_in_one;
        __syncthreads();
    }
    if (t != 0) return;
    int k = 0;
    for (int p = 0; p < int(a.passes); ++p) k += !skip[p];
    ctrl->active_passes = uint32_t(k);
    ctrl->spin_limit_ns = a.spin_limit_ns;
    ctrl->stall_tile = a.stall_tile;
    ctrl->copy_mode = kCopyNone;
    ctrl->copy_elem_bytes = a.elem_bytes;
    const void *cur = a.in;               // where the data (values for indirection) is
    const void *curk = a.keys_a;          // indirection: where the filtered keys are
    int i = 0;
    for (int p = 0; p < int(a.passes); ++p) {
        PassPlan &pp = ctrl->plan[p];
        pp.active = !skip[p];
        if (skip[p]) continue;
        ++i;
        void *dst;
        if (a.inplace) dst = (cur == a.in) ? a.buf : const_cast<void *>(a.in);
        else dst = ((k - i) % 2 == 0) ? a.out : a.buf;
        pp.reverse = (i == 1) && a.rev;
        if (a.indirect) {
            pp.src_vals = cur;
            pp.dst_vals = dst;
            pp.src_keys = curk;
            void *dk = (curk == a.keys_a) ? a.keys_b : a.keys_a;
            pp.dst_keys = (i == k) ? nullptr : dk;
            curk = dk;
        } else {
            pp.src_keys = cur;
            pp.dst_keys = dst;
            pp.src_vals = nullptr;
            pp.dst_vals = nullptr;
        }
        cur = dst;
    }
    if (!a.inplace) {
        if (k == 0) {
            ctrl->copy_mode = a.rev ? kCopyReversed : kCopyPlain;
            ctrl->copy_src = a.in;
            ctrl->copy_dst = a.out;
        }
    } else {
        const void *target = a.to_buffer ? a.buf : a.in;
        if (k == 0 && a.rev) {
            ctrl->copy_mode = a.to_buffer ? kCopyReversed : kReverseInPlace;
            ctrl->copy_src = a.in;
            ctrl->copy_dst = const_cast<void *>(target);
        } else if (cur != target) {
            ctrl->copy_mode = kCopyPlain;
            ctrl->copy_src = cur;
            ctrl->copy_dst = const_cast<void *>(target);
        }
    }
}

// ---- the onesweep scatter pass ----------------------------------------------------------------

template <typename U, bool HAS_VAL, int THREADS, int ITEMS>
struct OnesweepSmem {
    static constexpr int kTile = THREADS * ITEMS;
    static constexpr int kWarps = THREADS / 32;
    static constexpr int kHistStride = kBuckets + 1;  // + one slot for out-of-range items
    static constexpr size_t kStageK = size_t(kTile) * sizeof(U);
    static constexpr size_t kStageV = HAS_VAL ? size_t(kTile) * 8 : 0;
    static constexpr size_t kOffV = (kStageK + 15) & ~size_t(15);
    static constexpr size_t kOffHist = kOffV + kStageV;
    static constexpr size_t kOffTileStart = kOffHist + size_t(kWarps) * kHistStride * 4;
    static constexpr size_t kOffGofs = (kOffTileStart + kBuckets * 4 + 15) & ~size_t(15);
    static constexpr size_t kOffBstart = kOffGofs + kBuckets * 8;
    static constexpr size_t kOffMisc = kOffBstart + kBuckets * 8;
    static constexpr size_t kBytes = kOffMisc + 64;
};

template <typename U, bool HAS_VAL, int THREADS, int ITEMS, typename S>
__global__ void __launch_bounds__(THREADS, (sizeof(U) <= 4 && !HAS_VAL) ? 2 : 1)
    k_onesweep(Control *__restrict__ ctrl, const unsigned long long *__restrict__ bstart_all,
               S *__restrict__ status, int pass, uint64_t n, uint32_t num_tiles, Filter f) {
    using L = OnesweepSmem<U, HAS_VAL, THREADS, ITEMS>;
    constexpr int TILE = L::kTile;
    constexpr int WARPS = L::kWarps;
    constexpr int HS = L::kHistStride;
    extern __shared__ __align__(16) unsigned char smem[];
    U *stage_k = reinterpret_cast<U *>(smem);
    uint64_t *stage_v = reinterpret_cast<uint64_t *>(smem + L::kOffV);
    uint32_t *whist = reinterpret_cast<uint32_t *>(smem + L::kOffHist);
    uint32_t *tile_start = reinterpret_cast<uint32_t *>(smem + L::kOffTileStart);
    long long *gofs = reinterpret_cast<long long *>(smem + L::kOffGofs);
    unsigned long long *bstart = reinterpret_cast<unsigned long long *>(smem + L::kOffBstart);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);  // [0] tile, [1] bad, [2..9] scan

    const PassPlan plan = ctrl->plan[pass];
    if (!plan.active) return;
    const U *__restrict__ src_k = static_cast<const U *>(plan.src_keys);
    U *__restrict__ dst_k = static_cast<U *>(plan.dst_keys);
    const uint64_t *__restrict__ src_v = static_cast<const uint64_t *>(plan.src_vals);
    uint64_t *__restrict__ dst_v = static_cast<uint64_t *>(plan.dst_vals);
    const bool reverse = plan.reverse != 0;
    const uint64_t spin_limit = ctrl->spin_limit_ns;
    const uint32_t stall_tile = ctrl->stall_tile;
    S *__restrict__ st_pass = status;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < kBuckets; i += THREADS) bstart[i] = bstart_all[pass * kBuckets + i];
    const Filter fk = HAS_VAL ? Filter{0, 0, 0, 0} : f;   // indirect passes carry filtered keys

    for (;;) {
        if (tid == 0) {
            misc[0] = atomicAdd(&ctrl->tile_counter[pass], 1u);
            misc[1] = 0;
        }
        __syncthreads();
        const uint32_t tile = misc[0];
        if (tile >= num_tiles) break;
        const uint64_t tbase = uint64_t(tile) * TILE;
        const uint32_t tvalid = uint32_t((n - tbase) < uint64_t(TILE) ? (n - tbase) : uint64_t(TILE));

        // zero this warp's digit counters
        uint32_t *wh = whist + warp * HS;
        for (int i = lane; i < HS; i += 32) wh[i] = 0;
        __syncwarp();

        // load ITEMS keys per thread, warp-striped (item i of lane l = tile slot w*32*ITEMS + i*32 + l)
        U keys[ITEMS];
        uint64_t vals[HAS_VAL ? ITEMS : 1];
        uint32_t dig[ITEMS];
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t slot = uint32_t(warp) * 32u * ITEMS + uint32_t(i) * 32u + uint32_t(lane);
            const bool ok = slot < tvalid;
            const uint64_t gi = tbase + slot;
            const uint64_t si = reverse ? (n - 1u - gi) : gi;
            keys[i] = ok ? src_k[si] : U(0);
            if constexpr (HAS_VAL) vals[i] = ok ? src_v[si] : 0ull;
            dig[i] = ok ? digit_of(sortkey(keys[i], fk), pass) : uint32_t(kBuckets);
        }
        // warp multisplit rank: stable in slot order
        uint32_t rank[ITEMS];
        const uint32_t ltmask = lanemask_lt();
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dig[i]);
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) {
                base = wh[dig[i]];
                wh[dig[i]] = base + uint32_t(__popc(peers));
            }
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            rank[i] = base + uint32_t(__popc(peers & ltmask));
            __syncwarp();
        }
        __syncthreads();

        // per digit: exclusive offsets of the warps, tile count; publish the tile aggregate
        uint32_t count = 0;
        if (tid < kBuckets) {
            uint32_t run = 0;
#pragma unroll 4
            for (int w2 = 0; w2 < WARPS; ++w2) {
                const uint32_t c = whist[w2 * HS + tid];
                whist[w2 * HS + tid] = run;
                run += c;
            }
            count = run;
            if (tile != stall_tile)
                st_relaxed(st_pass + size_t(tile) * kBuckets + tid,
                           StatusWord<S>::make(tile == 0 ? kStInclusive : kStAggregate, count));
        }
        // exclusive scan of the tile counts over the digits
        uint32_t x = count;
        if (tid < kBuckets) {
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
            const uint32_t ts = before + x - count;
            tile_start[tid] = ts;
            // decoupled look-back over the predecessors' states for digit tid (bounded wait)
            uint64_t excl = 0;
            bool bad = false;
            if (tile > 0) {
                int64_t j = int64_t(tile) - 1;
                uint32_t spins = 0;
                uint64_t t0 = 0;
                while (j >= 0) {
                    const S wv = ld_relaxed(st_pass + size_t(j) * kBuckets + tid);
                    const uint32_t s = StatusWord<S>::state(wv);
                    if (s == kStInvalid) {
                        if (++spins > 32u) {
                            if (*reinterpret_cast<volatile uint32_t *>(&ctrl->abort)) { bad = true; break; }
                            const uint64_t now = globaltimer_ns();
                            if (t0 == 0) t0 = now;
                            else if (now - t0 > spin_limit) {
                                atomicOr(&ctrl->error, kDevTimeout);
                                atomicExch(&ctrl->abort, 1u);
                                bad = true;
                                break;
                            }
                            __nanosleep(64);
                        }
                        continue;
                    }
                    excl += StatusWord<S>::value(wv);
                    if (s == kStInclusive) break;
                    --j;
                }
                if (tile != stall_tile)
                    st_relaxed(st_pass + size_t(tile) * kBuckets + tid,
                               StatusWord<S>::make(kStInclusive, excl + count));
            }
            if (bad) misc[1] = 1u;
            gofs[tid] = (long long)(bstart[tid] + excl) - (long long)ts;
        }
        __syncthreads();
        const bool tile_bad = misc[1] != 0 || tile == stall_tile;

        // stage the tile in shared memory, sorted by digit
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            if (dig[i] < uint32_t(kBuckets)) {
                const uint32_t pos = tile_start[dig[i]] + wh[dig[i]] + rank[i];
                stage_k[pos] = keys[i];
                if constexpr (HAS_VAL) stage_v[pos] = vals[i];
            }
        }
        __syncthreads();
        // write out: consecutive threads take consecutive slots of a bucket run
        if (!tile_bad) {
            for (uint32_t s = tid; s < tvalid; s += THREADS) {
                const U k = stage_k[s];
                const uint32_t d = digit_of(sortkey(k, fk), pass);
                const long long g = gofs[d] + (long long)s;
                if (g >= 0 && uint64_t(g) < n) {
                    if (dst_k) dst_k[g] = k;
                    if constexpr (HAS_VAL) dst_v[g] = stage_v[s];
                }
            }
        }
        __syncthreads();
    }
}

// ---- copy step --------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ void copy_elems(const Control &c, uint64_t n) {
    const T *src = static_cast<const T *>(c.copy_src);
    T *dst = static_cast<T *>(c.copy_dst);
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

__global__ void __launch_bounds__(256) k_copy(const Control *__restrict__ ctrl, uint64_t n) {
    const Control c = *ctrl;
    if (c.copy_mode == kCopyNone) return;
    switch (c.copy_elem_bytes) {
        case 1: copy_elems<uint8_t>(c, n); break;
        case 2: copy_elems<uint16_t>(c, n); break;
        case 4: copy_elems<uint32_t>(c, n); break;
        default: copy_elems<uint64_t>(c, n); break;
    }
}

}  // namespace rsbd8g
