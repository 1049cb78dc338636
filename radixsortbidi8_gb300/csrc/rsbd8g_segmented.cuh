// rsbd8g_segmented.cuh - batched (segmented) sort: many independent arrays of uneven sizes in one
// stream-ordered launch sequence without host synchronisation (capturable as one CUDA graph).
//
// Segment s is [offsets[s], offsets[s+1]) of the concatenated input; every segment is sorted on
// its own with the semantics of the plain sort (Radixsortbidi8.hpp rsbd8::radixsortcopy).
//   k_seg_classify   small (<= cutoff keys) or large; compacts both lists on the device
//   k_seg_small      persistent CTAs sort each small segment whole in shared memory: a block-local
//                    LSD radix sort over 8-bit digits with the same warp multisplit and the
//                    reference's pass-skip test per segment
//   k_seg_hist       per large segment, all digit histograms in one read (tiles in order)
//   k_seg_plan       per large segment: exclusive scans, pass-skip mask
//   k_seg_sweep      one onesweep pass over the tiles of every large segment: look-back chains
//                    stay inside a segment; each segment ping-pongs by its own surviving passes
//                    (k_seg_sweep_pipe: the same pass with the look-back one tile behind)
//   k_seg_copy       large segments whose every digit was skipped (plain or reversed copy)
#pragma once
#include "rsbd8g_kernels.cuh"

namespace rsbd8g {

struct SegControl {
    uint32_t error;
    uint32_t abort;
    uint32_t nlarge;
    uint32_t nsmall;
    uint32_t ntiles;          // tiles of all large segments
    uint32_t small_counter;
    uint32_t tile_counter[kMaxPasses];
    uint32_t pad[6];
};

struct SegArgs {
    const uint64_t *offsets;  // nsegs + 1
    uint64_t total;           // elements of the concatenated arrays
    uint32_t nsegs;
    uint32_t cutoff;          // largest small segment
    uint32_t tile;            // keys per onesweep tile
    uint32_t rev;
    uint32_t dmask;
    uint32_t nlarge_max;
    SegControl *ctrl;
    uint32_t *large_seg;      // [nlarge_max]
    uint32_t *large_tbase;    // [nlarge_max + 1]
    uint32_t *small_seg;      // [nsegs]
    uint32_t *seg_hist;       // [nlarge_max][P][256]: counts, then bucket starts
    uint32_t *seg_mask;       // [nlarge_max]: surviving digits
    uint32_t *tile_seg;       // [tiles_max]: the large segment (list index) of each tile, by k_seg_hist
    // pointer-table form: segment s lives at ptr_in[s] / ptr_out[s] / ptr_buf[s] (separate arrays;
    // offsets then only give the lengths); null: segment s is at offsets[s] of in / out / buf
    const uint64_t *ptr_in;
    const uint64_t *ptr_out;
    const uint64_t *ptr_buf;
    uint64_t spin_limit_ns;   // bound of every look-back wait
    uint32_t prefetch;        // every array is device memory: tiles may be prefetched into L2
    // per-segment directions (sortingdirection values, one byte per segment); null: dmask and rev
    // above hold for every segment.  rev_ok: the mode honours isrevorder (a uniform property)
    const uint8_t *seg_dir;
    uint32_t rev_ok;
};

// the digit complement (descending sorts) and the effective isrevorder of segment `seg`
__device__ __forceinline__ uint32_t seg_dmask(const SegArgs &a, uint32_t seg) {
    return a.seg_dir ? ((a.seg_dir[seg] & 1u) ? 0xFFu : 0u) : a.dmask;
}
__device__ __forceinline__ bool seg_rev(const SegArgs &a, uint32_t seg) {
    return a.seg_dir ? (((a.seg_dir[seg] >> 1) & 1u) != 0 && a.rev_ok != 0) : a.rev != 0;
}

__device__ __forceinline__ uint64_t seg_len(const uint64_t *off, uint32_t s) { return off[s + 1] - off[s]; }

// where segment `seg` starts in one of the three arrays
template <typename U>
__device__ __forceinline__ U *seg_ptr(const SegArgs &a, const uint64_t *table, const U *base, uint32_t seg) {
    return table ? reinterpret_cast<U *>(table[seg]) : const_cast<U *>(base) + a.offsets[seg];
}

// one CTA of 1024 threads classifies every segment; a single 64-bit atomic per warp hands out
// (list index, tile base) pairs so tile bases grow with the list index
static __global__ void __launch_bounds__(1024) k_seg_classify(SegArgs a) {
    SegControl *c = a.ctrl;
    __shared__ unsigned long long large_ctr;   // (count << 32) | tiles
    __shared__ uint32_t small_ctr;
    __shared__ uint32_t too_long;
    if (threadIdx.x == 0) {
        large_ctr = 0;
        small_ctr = 0;
        too_long = 0;
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = 0; base < a.nsegs; base += blockDim.x) {
        const uint32_t s = base + threadIdx.x;
        const bool ok = s < a.nsegs;
        const uint64_t len = ok ? seg_len(a.offsets, s) : 0;
        if (len >= (uint64_t(1) << 30)) too_long = 1u;
        const bool large = ok && len > a.cutoff;
        const bool small = ok && !large && len > 0;
        const uint32_t tiles = large ? uint32_t((len + a.tile - 1) / a.tile) : 0u;
        // warp-aggregated reservation of list slots and tiles
        const uint32_t lmask = __ballot_sync(0xFFFFFFFFu, large);
        uint32_t tsum = tiles, tpre;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, tsum, o);
            if (lane >= uint32_t(o)) tsum += y;
        }
        tpre = tsum - tiles;
        const uint32_t ttot = __shfl_sync(0xFFFFFFFFu, tsum, 31);
        unsigned long long old = 0;
        if (lane == 0 && lmask)
            old = atomicAdd(&large_ctr, (uint64_t(__popc(lmask)) << 32) | uint64_t(ttot));
        old = __shfl_sync(0xFFFFFFFFu, old, 0);
        if (large) {
            const uint32_t idx = uint32_t(old >> 32) + uint32_t(__popc(lmask & lanemask_lt()));
            if (idx < a.nlarge_max) {
                a.large_seg[idx] = s;
                a.large_tbase[idx] = uint32_t(old) + tpre;
            } else {
                too_long = 1u;      // more large segments than the layout holds: inconsistent offsets
            }
        }
        const uint32_t smask = __ballot_sync(0xFFFFFFFFu, small);
        uint32_t sold = 0;
        if (lane == 0 && smask) sold = atomicAdd(&small_ctr, uint32_t(__popc(smask)));
        sold = __shfl_sync(0xFFFFFFFFu, sold, 0);
        if (small) a.small_seg[sold + uint32_t(__popc(smask & lanemask_lt()))] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // offsets must start at 0 and end at or before `total` (then, being non-decreasing, every
        // segment lies inside the arrays; a decreasing pair shows up as a huge length above)
        if (a.offsets[0] != 0 || a.offsets[a.nsegs] > a.total) too_long = 1u;
        c->nlarge = min(uint32_t(large_ctr >> 32), a.nlarge_max);
        c->ntiles = uint32_t(large_ctr);
        a.large_tbase[c->nlarge] = c->ntiles;
        if (too_long) {
            c->nlarge = 0;
            c->nsmall = 0;
            c->ntiles = 0;
        }
        if (!too_long) c->nsmall = small_ctr;
        if (too_long) {
            c->error |= kDevFault;
            c->abort = 1u;
        }
    }
}

// index of the large segment owning global tile gt (tile bases are non-decreasing)
__device__ __forceinline__ uint32_t seg_of_tile(const uint32_t *tbase, uint32_t nlarge, uint32_t gt) {
    uint32_t lo = 0, hi = nlarge;            // invariant: tbase[lo] <= gt < tbase[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (tbase[mid] <= gt) lo = mid;
        else hi = mid;
    }
    return lo;
}

// all digit histograms of every large segment; CTA c reads a contiguous run of tiles in order
// (and records the segment of each of those tiles for the scatter passes)
template <typename U, int MODE, int THREADS>
__global__ void __launch_bounds__(THREADS) k_seg_hist(SegArgs a, const U *__restrict__ in) {
    constexpr int P = KeyTraits<U>::kDigits;
    constexpr int C = hist_lane_copies<P>();
    extern __shared__ __align__(16) uint32_t shl[];   // C lane-class copies, as in k_histogram
    const SegControl *c = a.ctrl;
    if (c->abort) return;
    const uint32_t T = c->ntiles, nl = c->nlarge;
    if (T == 0) return;
    const uint32_t t0 = uint32_t(uint64_t(T) * blockIdx.x / gridDim.x);
    const uint32_t t1 = uint32_t(uint64_t(T) * (blockIdx.x + 1) / gridDim.x);
    if (t0 >= t1) return;
    for (int i = threadIdx.x; i < C * P * kBuckets; i += THREADS) shl[i] = 0;
    __syncthreads();
    uint32_t *sh = shl + (threadIdx.x & uint32_t(C - 1));
    uint32_t idx = seg_of_tile(a.large_tbase, nl, t0);
    for (uint32_t gt = t0; gt < t1;) {
        while (a.large_tbase[idx + 1] <= gt) ++idx;
        const uint32_t seg = a.large_seg[idx];
        const uint64_t len = seg_len(a.offsets, seg);
        const U *src = seg_ptr(a, a.ptr_in, in, seg);
        const uint32_t dm = seg_dmask(a, seg);
        const uint32_t tend = min(t1, a.large_tbase[idx + 1]);
        for (uint32_t x = gt + threadIdx.x; x < tend; x += THREADS) a.tile_seg[x] = idx;
        const uint64_t k0 = uint64_t(gt - a.large_tbase[idx]) * a.tile;
        const uint64_t k1 = min(len, uint64_t(tend - a.large_tbase[idx]) * a.tile);
        auto count = [&](U raw) {
            const U k = filter_key<MODE>(raw);
#pragma unroll
            for (int p = 0; p < P; ++p) atomicAdd(sh + (p * kBuckets + (digit_of(k, p) ^ dm)) * C, 1u);
        };
        if constexpr (sizeof(U) < 16) {
            // 16-byte loads over the aligned middle of [k0, k1) (as in k_histogram); the keys before
            // the first 16-byte boundary and after the last whole vector by the first warp
            constexpr int V = 16 / int(sizeof(U));
            const U *base = src + k0;
            const uint64_t cnt = k1 > k0 ? k1 - k0 : 0;
            const uint64_t mis = (reinterpret_cast<uintptr_t>(base) & 15u) / sizeof(U);
            const uint64_t head = mis ? (uint64_t(V) - mis < cnt ? uint64_t(V) - mis : cnt) : 0;
            const uint64_t nvec = (cnt - head) / V;
            const uint64_t tail0 = head + nvec * V;
            if (threadIdx.x < 32) {
                for (uint64_t i = threadIdx.x; i < head; i += 32) count(base[i]);
                for (uint64_t i = tail0 + threadIdx.x; i < cnt; i += 32) count(base[i]);
            }
            const uint4 *vp = reinterpret_cast<const uint4 *>(base + head);
            constexpr int UNR = 4;                       // 16-byte loads in flight per thread
            for (uint64_t b = threadIdx.x; b < nvec; b += uint64_t(THREADS) * UNR) {
                uint4 v[UNR];
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    const uint64_t j = b + uint64_t(u) * THREADS;
                    v[u] = j < nvec ? __ldg(vp + j) : make_uint4(0, 0, 0, 0);
                }
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    if (b + uint64_t(u) * THREADS >= nvec) break;
                    U kk[V];
                    memcpy(kk, &v[u], 16);
#pragma unroll
                    for (int q = 0; q < V; ++q) count(kk[q]);
                }
            }
        } else {
            constexpr int UNR = 8;                       // loads in flight per thread
            for (uint64_t b = k0 + threadIdx.x; b < k1; b += uint64_t(THREADS) * UNR) {
                U raw[UNR];
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    const uint64_t i = b + uint64_t(u) * THREADS;
                    raw[u] = i < k1 ? src[i] : U{};
                }
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    if (b + uint64_t(u) * THREADS >= k1) break;
                    count(raw[u]);
                }
            }
        }
        __syncthreads();
        // fold the copies (rotated reads: conflict-free), clear them for the next segment
        uint32_t *gh = a.seg_hist + size_t(idx) * P * kBuckets;
        for (int i = threadIdx.x; i < P * kBuckets; i += THREADS) {
            uint32_t v = 0;
#pragma unroll 8
            for (int cc = 0; cc < C; ++cc) {
                uint32_t *w = shl + i * C + ((cc + i) & (C - 1));
                v += *w;
                *w = 0;
            }
            if (v) atomicAdd(gh + i, v);
        }
        __syncthreads();
        gt = tend;
    }
}

// per large segment (one CTA each): bucket starts in place of the counts, surviving-digit mask
static __global__ void __launch_bounds__(256) k_seg_plan(SegArgs a, int passes) {
    const SegControl *c = a.ctrl;
    if (c->abort) return;
    __shared__ uint32_t wsum[8];
    const uint32_t nl = c->nlarge;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (uint32_t idx = blockIdx.x; idx < nl; idx += gridDim.x) {
        const uint32_t seg = a.large_seg[idx];
        const uint64_t len = seg_len(a.offsets, seg);
        uint32_t mask = 0;
        for (int p = 0; p < passes; ++p) {
            uint32_t *h = a.seg_hist + (size_t(idx) * passes + p) * kBuckets;
            const uint32_t v = h[t];
            const int skip = __syncthreads_or(uint64_t(v) == len);
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) wsum[w] = x;
            __syncthreads();
            uint32_t before = 0;
            for (int i = 0; i < w; ++i) before += wsum[i];
            h[t] = before + x - v;
            if (!skip) mask |= 1u << p;
            __syncthreads();
        }
        if (t == 0) a.seg_mask[idx] = mask;
    }
}

// one onesweep pass over the tiles of every large segment
template <typename U, int MODE, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, onesweep_min_blocks<U, false, THREADS>())
    k_seg_sweep(SegArgs a, int pass, int passes, const U *__restrict__ in, U *__restrict__ out,
                U *__restrict__ buf, uint32_t *__restrict__ status, uint32_t stall_tile) {
    using L = OnesweepSmem<U, false, THREADS, ITEMS>;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long *bstart = reinterpret_cast<unsigned long long *>(smem + L::kOffBstart);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);
    SegControl *c = a.ctrl;
    if (c->abort) return;
    const uint32_t T = c->ntiles;
    const uint64_t spin_limit = a.spin_limit_ns;
    sweep_init_smem<U, MODE, false, THREADS, ITEMS, uint32_t>(smem);
    for (;;) {
        if (threadIdx.x == 0) {
            misc[0] = atomicAdd(&c->tile_counter[pass], 1u);
            misc[1] = 0;
        }
        __syncthreads();
        const uint32_t gt = misc[0];
        if (gt >= T) break;
        const uint32_t idx = a.tile_seg[gt];
        const uint32_t mask = a.seg_mask[idx];
        if (!((mask >> pass) & 1u)) {        // this digit is skipped for the segment
            __syncthreads();
            continue;
        }
        const uint32_t seg = a.large_seg[idx];
        const uint64_t len = seg_len(a.offsets, seg);
        const int k = __popc(mask), i = __popc(mask & ((1u << pass) - 1u)) + 1;
        U *sin = seg_ptr(a, a.ptr_in, in, seg), *sout = seg_ptr(a, a.ptr_out, out, seg);
        U *sbuf = seg_ptr(a, a.ptr_buf, buf, seg);
        const U *src = (i == 1) ? sin : (((k - (i - 1)) % 2 == 0) ? sout : sbuf);
        U *dst = ((k - i) % 2 == 0) ? sout : sbuf;
        const uint32_t *bs = a.seg_hist + (size_t(idx) * passes + pass) * kBuckets;
        for (int j = threadIdx.x; j < kBuckets; j += THREADS) bstart[j] = bs[j];
        SweepTile<U, uint32_t> t;
        t.src_k = src;
        t.dst_k = dst;
        t.src_v = nullptr;
        t.dst_v = nullptr;
        t.status = status + size_t(a.large_tbase[idx]) * kBuckets;
        t.n = len;
        t.tile = gt - a.large_tbase[idx];
        t.reverse = seg_rev(a, seg) && i == 1;
        sweep_tile<U, MODE, false, THREADS, ITEMS, uint32_t>(smem, t, bstart, pass, seg_dmask(a, seg), &c->error, &c->abort,
                                                             spin_limit, stall_tile);
    }
}

// One scatter pass over the tiles of every large segment, pipelined as k_onesweep_pipe: tile B is
// loaded and ranked while tile A (staged in shared memory) waits for its look-back, which threads
// 256..511 resolve while threads 0..255 scan B's counts.  A tile's segment fixes its source,
// destination, length, look-back words and bucket starts; a tile whose segment skips this digit is
// passed over.
struct SegPipeTile {
    const void *src;            // null: the tile's segment skips this digit (the tile is passed over)
    void *dst;
    const uint32_t *bs;        // bucket starts of this pass for the segment (global)
    uint32_t *status;          // look-back words of the segment's tile 0
    uint64_t n;                // keys of the segment
    uint32_t tile;             // tile index within the segment
    uint32_t reverse;
    uint32_t dmask;            // the segment's digit complement (descending sorts)
};

template <typename U>
__device__ __forceinline__ bool seg_pipe_tile(const SegArgs &a, int pass, int passes, const U *in, U *out, U *buf,
                                              uint32_t *status, uint32_t gt, SegPipeTile &t) {
    const uint32_t idx = a.tile_seg[gt];
    const uint32_t mask = a.seg_mask[idx];
    t.src = nullptr;
    if (!((mask >> pass) & 1u)) return false;          // this digit is skipped for the segment
    const uint32_t seg = a.large_seg[idx];
    const int k = __popc(mask), i = __popc(mask & ((1u << pass) - 1u)) + 1;
    U *sin = seg_ptr(a, a.ptr_in, in, seg), *sout = seg_ptr(a, a.ptr_out, out, seg);
    U *sbuf = seg_ptr(a, a.ptr_buf, buf, seg);
    t.src = (i == 1) ? sin : (((k - (i - 1)) % 2 == 0) ? sout : sbuf);
    t.dst = ((k - i) % 2 == 0) ? sout : sbuf;
    t.bs = a.seg_hist + (size_t(idx) * passes + pass) * kBuckets;
    t.status = status + size_t(a.large_tbase[idx]) * kBuckets;
    t.n = seg_len(a.offsets, seg);
    t.tile = gt - a.large_tbase[idx];
    t.reverse = (seg_rev(a, seg) && i == 1) ? 1u : 0u;
    t.dmask = seg_dmask(a, seg);
    return true;
}

template <typename U, int MODE, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, 2)
    k_seg_sweep_pipe(SegArgs a, int pass, int passes, const U *__restrict__ in, U *__restrict__ out,
                     U *__restrict__ buf, uint32_t *__restrict__ status, uint32_t stall_tile) {
    static_assert(THREADS == 2 * kBuckets, "threads 0..255 scan, threads 256..511 look back");
    using L = PipeSmem<U, THREADS, ITEMS>;
    static_assert(L::kTile <= 65535, "tile ranks are 16-bit");
    constexpr int TILE = L::kTile;
    using R = TileRank<THREADS, ITEMS, rank_lanes<ITEMS>(), sizeof(U) == 8>;   // dense ranks: 8-byte keys
    extern __shared__ __align__(16) unsigned char smem[];
    U *stage = reinterpret_cast<U *>(smem);
    uint32_t *utab = reinterpret_cast<uint32_t *>(smem + L::kOffUnits);
    int32_t *gofs = reinterpret_cast<int32_t *>(smem + L::kOffGofs);   // segments hold fewer than 2^30 keys
    uint32_t *tsall = reinterpret_cast<uint32_t *>(smem + L::kOffTs);
    uint32_t *cntall = reinterpret_cast<uint32_t *>(smem + L::kOffCnt);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);   // [0] next tile [1] bad [2..9] scan
    SegControl *c = a.ctrl;
    if (c->abort) return;
    // the descriptors of the claimed tiles, two slots used in turn: thread 0 looks a tile up once
    // when it claims it and the CTA reads the descriptor from here one iteration later
    static_assert(2 * sizeof(SegPipeTile) <= 128, "descriptor slots fit the auxiliary area");
    SegPipeTile *slots = reinterpret_cast<SegPipeTile *>(smem + L::kOffAux);
    const uint32_t T = c->ntiles;
    const uint64_t spin_limit = a.spin_limit_ns;
    uint32_t *err_word = &c->error;
    uint32_t *abort_word = &c->abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t *urow = R::row(utab);
    const uint32_t slot0 = R::slot0();

    for (int i = tid; i < R::kWords; i += THREADS) utab[i] = 0u;
    if (tid == 0) {
        const uint32_t g = atomicAdd(&c->tile_counter[pass], 1u);
        misc[0] = g;
        misc[1] = 0u;
        if (g < T) seg_pipe_tile<U>(a, pass, passes, in, out, buf, status, g, slots[0]);
    }
    __syncthreads();
    uint32_t gtB = misc[0];
    bool hasA = false;
    SegPipeTile A{}, B{};
    uint32_t tvalidA = 0;
    int par = 0;
    for (uint32_t it = 0;; ++it) {
        const bool claimed = gtB < T;
        if (!hasA && !claimed) break;
        if (claimed) B = slots[it & 1u];
        const bool hasB = claimed && B.src != nullptr;
        uint32_t *tsB = tsall + par * kBuckets, *tsA = tsall + (par ^ 1) * kBuckets;
        uint32_t *cntB = cntall + par * kBuckets, *cntA = cntall + (par ^ 1) * kBuckets;
        uint32_t next = 0xFFFFFFFFu;
        if (claimed && tid == 0) {
            next = atomicAdd(&c->tile_counter[pass], 1u);   // the tile after B: its keys go to L2 now
            SegPipeTile &N = slots[(it & 1u) ^ 1u];
            if (next < T && seg_pipe_tile<U>(a, pass, passes, in, out, buf, status, next, N) && a.prefetch)
                prefetch_tile<TILE>(static_cast<const U *>(N.src), N.n, N.tile, N.reverse != 0);
        }
        // the look-back threads load A's first window now: the loads complete while B is ranked
        constexpr int kWin = 4;
        uint32_t lbw[kWin];
        if (hasA && tid >= kBuckets && A.tile > 0) lookback_load(A.status, int64_t(A.tile) - 1, tid - kBuckets, lbw);

        U keys[ITEMS];
        uint32_t rk[R::kRankRegs];
        uint32_t tvalidB = 0;
        if (hasB) {
            const U *src = static_cast<const U *>(B.src);
            const uint64_t n = B.n;
            const uint64_t tbase = uint64_t(B.tile) * TILE;
            tvalidB = uint32_t((n - tbase) < uint64_t(TILE) ? (n - tbase) : uint64_t(TILE));
            load_items<ITEMS, R::kLanes>(keys, src, n, tbase, slot0, tvalidB, TILE, B.reverse != 0, KeyTraits<U>::fill());
            R::template rank<MODE>(keys, rk, utab, slot0, tvalidB, pass, B.dmask);
        }
        __syncthreads();                                                        // barrier 1

        uint32_t x = 0, run = 0;
        if (tid < kBuckets) {
            if (hasB) {
                run = R::total(utab, tid);
                uint32_t count = run;
                if (tid == kBuckets - 1) count -= uint32_t(TILE) - tvalidB;      // the padding slots
                cntB[tid] = count;
                if (B.tile != stall_tile)
                    st_relaxed(B.status + size_t(B.tile) * kBuckets + tid,
                               StatusWord<uint32_t>::make(B.tile == 0 ? kStInclusive : kStAggregate, count));
                x = run;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) misc[2 + warp] = x;
            }
        } else if (hasA) {
            const int d = tid - kBuckets;
            const uint32_t count = cntA[d];
            uint64_t excl = 0;
            bool bad = false;
            if (A.tile > 0) {
                bad = !lookback_walk(A.status, A.tile, d, lbw, excl, err_word, abort_word, spin_limit);
                if (A.tile != stall_tile)
                    st_relaxed(A.status + size_t(A.tile) * kBuckets + d,
                               StatusWord<uint32_t>::make(kStInclusive, excl + count));
            }
            if (bad) misc[1] = 1u;
            gofs[d] = int32_t((long long)(uint64_t(A.bs[d]) + excl) - (long long)tsA[d]);
        }
        __syncthreads();                                                        // barrier 2

        if (tid < kBuckets && hasB) {
            uint32_t before = 0;
            for (int i = 0; i < warp; ++i) before += misc[2 + i];
            const uint32_t ts = before + x - run;
            R::offsets(utab, tid, ts);
            tsB[tid] = ts;
        }
        if (hasA && misc[1] == 0u && A.tile != stall_tile) {
            U *dst = static_cast<U *>(A.dst);
            const uint64_t n = A.n;
            for (uint32_t s = tid; s < tvalidA; s += THREADS) {
                const U k = stage[s];
                const int32_t g = gofs[pass_digit<MODE>(k, pass, A.dmask)] + int32_t(s);
                if (uint64_t(g) < n) dst[g] = k;
                else atomicOr(err_word, kDevFault);     // an offset outside the segment: flagged, not written
            }
        }
        __syncthreads();                                                        // barrier 3

        if (hasB) {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t d = R::template digit_of_item<MODE>(rk, i, keys[i], slot0 + uint32_t(R::kLanes) * i, tvalidB, pass, B.dmask);
                stage[urow[d] + R::rank_of(rk, i)] = keys[i];
            }
            R::clear_own(utab);
        }
        if (tid == 0) {
            misc[0] = next;
            misc[1] = 0u;
        }
        __syncthreads();                                                        // barrier 4
        // a passed-over tile leaves the pending tile as it was
        if (hasB) {
            hasA = true;
            A = B;
            tvalidA = tvalidB;
            par ^= 1;
        } else {
            hasA = false;
        }
        gtB = claimed ? misc[0] : T;
    }
}

// large segments with every digit skipped: plain or reversed copy (one warp per segment)
template <typename U>
__global__ void __launch_bounds__(256) k_seg_copy(SegArgs a, const U *__restrict__ in, U *__restrict__ out) {
    const SegControl *c = a.ctrl;
    if (c->abort) return;
    const uint32_t nl = c->nlarge;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < nl; idx += (gridDim.x * blockDim.x) >> 5) {
        if (a.seg_mask[idx]) continue;
        const uint32_t seg = a.large_seg[idx];
        const uint64_t len = seg_len(a.offsets, seg);
        const U *src = seg_ptr(a, a.ptr_in, in, seg);
        U *dst = seg_ptr(a, a.ptr_out, out, seg);
        const bool rev = seg_rev(a, seg);
        for (uint64_t i = lane; i < len; i += 32) dst[i] = src[rev ? len - 1 - i : i];
    }
}

// ---- small segments: whole-segment LSD radix sort in shared memory ----------------------------

template <typename U, int THREADS, int ITEMS>
struct SmallSmem {
    static constexpr int kCap = THREADS * ITEMS;
    static constexpr int kWarps = THREADS / 32;
    static constexpr int kStride = kBuckets + 1;                 // + one bucket for idle lanes
    static constexpr size_t kOffB = (size_t(kCap) * sizeof(U) + 15) & ~size_t(15);
    static constexpr size_t kOffR = kOffB + ((size_t(kCap) * sizeof(U) + 15) & ~size_t(15));
    static constexpr size_t kOffWofs = kOffR + size_t(kCap) * 4;
    static constexpr size_t kOffWmask = kOffWofs + size_t(kWarps) * kStride * 4;
    static constexpr size_t kOffMisc = kOffWmask + size_t(kWarps) * kStride * 4;
    static constexpr size_t kBytes = kOffMisc + 64;
};

template <typename U, int MODE, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS) k_seg_small(SegArgs a, const U *__restrict__ in, U *__restrict__ out) {
    using L = SmallSmem<U, THREADS, ITEMS>;
    constexpr int P = KeyTraits<U>::kDigits;
    constexpr int WARPS = L::kWarps;
    constexpr int ST = L::kStride;
    static_assert(THREADS >= kBuckets, "one thread per digit");
    extern __shared__ __align__(16) unsigned char smem[];
    U *A = reinterpret_cast<U *>(smem);
    U *B = reinterpret_cast<U *>(smem + L::kOffB);
    uint32_t *R = reinterpret_cast<uint32_t *>(smem + L::kOffR);
    uint32_t *wofs = reinterpret_cast<uint32_t *>(smem + L::kOffWofs);
    uint32_t *wmaskall = reinterpret_cast<uint32_t *>(smem + L::kOffWmask);
    uint32_t *misc = reinterpret_cast<uint32_t *>(smem + L::kOffMisc);   // [0] job [1] skip [2..9] scan
    SegControl *c = a.ctrl;
    if (c->abort) return;
    const uint32_t ns = c->nsmall;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t *wcnt = wofs + warp * ST;
    uint32_t *wmask = wmaskall + warp * ST;
    const uint32_t ltmask = lanemask_lt();
    for (int i = tid; i < WARPS * ST; i += THREADS) wmaskall[i] = 0u;
    for (;;) {
        if (tid == 0) misc[0] = atomicAdd(&c->small_counter, 1u);
        __syncthreads();
        const uint32_t job = misc[0];
        if (job >= ns) break;
        const uint32_t seg = a.small_seg[job];
        const uint32_t len = uint32_t(seg_len(a.offsets, seg));
        const U *sin = seg_ptr(a, a.ptr_in, in, seg);
        U *sout = seg_ptr(a, a.ptr_out, out, seg);
        const bool rev = seg_rev(a, seg);
        const uint32_t dm = seg_dmask(a, seg);
        for (uint32_t i = tid; i < len; i += THREADS) A[i] = sin[rev ? len - 1u - i : i];
        // warp w ranks slots [w * chunk, min((w + 1) * chunk, len)) in steps of 32
        const uint32_t chunk = ((len + WARPS - 1) / WARPS + 31u) & ~31u;
        const uint32_t w0 = min(len, uint32_t(warp) * chunk), w1 = min(len, w0 + chunk);
        U *src = A, *dst = B;
        for (int p = 0; p < P; ++p) {
            for (int i = lane; i < ST; i += 32) wcnt[i] = 0u;
            if (tid == 0) misc[1] = 0u;
            __syncthreads();
            for (uint32_t b = w0; b < w1; b += 32) {
                const uint32_t slot = b + uint32_t(lane);
                const bool ok = slot < w1;
                const uint32_t d = ok ? pass_digit<MODE>(src[slot], p, dm) : uint32_t(kBuckets);
                atomicOr(wmask + d, 1u << lane);
                __syncwarp();
                const uint32_t peers = wmask[d];
                const uint32_t before = wcnt[d];
                __syncwarp();
                const uint32_t lower = uint32_t(__popc(peers & ltmask));
                if (lower == 0) {
                    wcnt[d] = before + uint32_t(__popc(peers));
                    wmask[d] = 0u;
                }
                __syncwarp();
                if (ok) R[slot] = ((before + lower) << 8) | d;
            }
            __syncthreads();
            uint32_t run = 0, x = 0;
            if (tid < kBuckets) {
#pragma unroll
                for (int w2 = 0; w2 < WARPS; ++w2) {
                    const uint32_t cc = wofs[w2 * ST + tid];
                    wofs[w2 * ST + tid] = run;
                    run += cc;
                }
                if (run == len) misc[1] = 1u;        // pass-skip: one bucket holds every key
                x = run;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) misc[2 + warp] = x;
            }
            __syncthreads();
            const bool skip = misc[1] != 0;
            if (tid < kBuckets && !skip) {
                uint32_t before = 0;
                for (int i = 0; i < warp; ++i) before += misc[2 + i];
                const uint32_t ts = before + x - run;
#pragma unroll
                for (int w2 = 0; w2 < WARPS; ++w2) wofs[w2 * ST + tid] += ts;
            }
            __syncthreads();
            if (!skip) {
                for (uint32_t slot = w0 + uint32_t(lane); slot < w1; slot += 32) {
                    const uint32_t v = R[slot];
                    dst[wcnt[v & 0xFFu] + (v >> 8)] = src[slot];
                }
                U *tmp = src;
                src = dst;
                dst = tmp;
            }
            __syncthreads();
        }
        for (uint32_t i = tid; i < len; i += THREADS) sout[i] = src[i];
        __syncthreads();
    }
}

}  // namespace rsbd8g
