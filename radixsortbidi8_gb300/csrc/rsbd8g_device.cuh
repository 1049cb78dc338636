// rsbd8g_device.cuh - device code of the GB300 stable LSD radix sort.
//
// Sorting semantics follow Radixsortbidi8.hpp (namespace rsbd8):
//   * the filtered sort key K(b) of each of the 8 filter combinations:
//     filterinput (Radixsortbidi8.hpp:10006-10027) plus the virtual MSB flip of the
//     signed/floating-point modes and the virtual LSB flip of tiered absolute
//     floating point done by the offsets generators (Radixsortbidi8.hpp:11629-11806);
//   * the up-front histogram of every digit in one read of the keys
//     (radixsortnoallocmultiinitmt, Radixsortbidi8.hpp:28919) and the pass-skip test
//     "one bucket holds every key" (generateoffsets*, Radixsortbidi8.hpp:12238-12440);
//   * one stable scatter per surviving digit that stores the original key bits
//     (radixsortnoallocmultisortmain, Radixsortbidi8.hpp:31782-31982).
// The GPU uses 8-bit digits throughout (the reference uses 11-bit digits for 32/64-bit
// keys); a stable LSD sort's output depends only on the key order, so the result is
// identical.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace rsbd8g {

constexpr int kRadixBits = 8;
constexpr int kBuckets = 1 << kRadixBits;
constexpr int kMaxPasses = 16;   // 128-bit keys: 16 digit passes

// device status bits (Control::error)
enum : uint32_t { kDevTimeout = 1u, kDevFault = 2u };

// look-back status word states (top two bits)
enum : uint32_t { kStInvalid = 0u, kStAggregate = 1u, kStInclusive = 2u };

// copy step after the scatter passes (Control::copy_mode)
enum : uint32_t { kCopyNone = 0u, kCopyPlain = 1u, kCopyReversed = 2u, kReverseInPlace = 3u };

struct Filter {
    uint32_t absv, sign, fltp, desc;
};

// The arrays of one sort reach the scatter and copy kernels as a kernel parameter; the plan in
// the control block (scratch memory, which the caller owns) names them by index.  So no address
// is ever read from scratch: a control block damaged by a caller's stray write gives wrong
// results and a fault flag, never an access outside the sort's own arrays.
enum : uint32_t { kArrIn = 0u, kArrOut = 1u, kArrBuf = 2u, kArrKeysA = 3u, kArrKeysB = 4u, kArrCount = 5u,
                  kArrNone = 0xFFu };
struct SortArrays {
    const void *p[kArrCount];   // input, output, buffer, indirect key arrays A and B (null if unused)
};
// array `sel`; null for kArrNone; `fallback` (with *bad set) for an index that names no array.
// Selects over constant indices, so the parameter array is never indexed at run time (which
// would copy it to local memory).
__host__ __device__ __forceinline__ void *sort_array(const SortArrays &a, uint32_t sel, uint32_t fallback, bool *bad) {
    if (sel == kArrNone) return nullptr;
    const void *r = nullptr, *f = nullptr;
#pragma unroll
    for (uint32_t i = 0; i < kArrCount; ++i) {
        r = sel == i ? a.p[i] : r;
        f = fallback == i ? a.p[i] : f;
    }
    if (!r) {
        *bad = true;
        r = f;
    }
    return const_cast<void *>(r);
}

struct PassPlan {
    uint32_t src_keys;     // SortArrays indices
    uint32_t dst_keys;     // kArrNone on the last indirect pass (keys are dropped)
    uint32_t src_vals;     // indirect: object pointers (kArrNone for direct sorts)
    uint32_t dst_vals;
    uint32_t active;
    uint32_t reverse;      // read the source back to front (isrevorder, first surviving pass)
    uint32_t hot;          // crowded digits of the pass, ranked with ballots: (digit1 << 16) | digit0,
                           // kNoHot in a half for none (see TileRank)
    uint32_t pad1;
};
constexpr uint32_t kNoHot = 0x100u;                       // not a digit: matches no key
constexpr uint32_t kNoHotPair = (kNoHot << 16) | kNoHot;

struct Control {
    uint32_t error;
    uint32_t abort;
    uint32_t tile_counter[kMaxPasses];
    uint32_t active_passes;
    uint32_t copy_mode;
    uint32_t copy_src;     // SortArrays indices
    uint32_t copy_dst;
    uint32_t stall_tile;   // diagnostics: this tile never publishes (0xFFFFFFFF = off)
    uint32_t prefetch;     // 1: every array is device memory, so tiles may be prefetched into L2
    uint32_t hist_done;    // histogram CTAs finished (the last one computes the plan)
    uint32_t pad0;
    uint64_t spin_limit_ns;
    PassPlan plan[kMaxPasses];
};
static_assert(sizeof(Control) <= 1024, "control block must fit its slot");

// ---- key filter -----------------------------------------------------------------------

// K(b): transform raw key bits into an unsigned key whose ascending order is the reference's
// ascending order for the filter combination MODE = isabsvalue | issignmode << 1 | isfltpmode << 2
// (the low three bits of the resolved sortingmode).  Descending sorts use the complement ~K,
// which the kernels apply per digit.
template <int MODE, typename U>
__host__ __device__ __forceinline__ U filter_key(U b) {
    constexpr bool ABS = (MODE & 1) != 0, SIGN = (MODE & 2) != 0, FLTP = (MODE & 4) != 0;
    constexpr int W = int(sizeof(U)) * 8;
    constexpr U sb = U(U(1) << (W - 1));
    using I = typename std::make_signed<U>::type;
    if constexpr (ABS != FLTP) {
        const U s = U(I(b) >> (W - 1));            // sign mask: all ones for negative keys
        if constexpr (ABS) {
            if constexpr (SIGN) return U(U(b + s) ^ s);                      // absolute signed
            else return U(U(b << 1) ^ s);                                    // tiered absolute signed
        } else {
            const U m = U(b & U(~sb));
            if constexpr (SIGN) return U(U(U(m + s) ^ s) ^ sb);              // floating point, MSB flip
            else return U(m ^ s);                                            // inside-out floating point
        }
    } else if constexpr (ABS) {
        if constexpr (SIGN) return U(b & U(~sb));                           // absolute floating point
        else return U(U(U(b << 1) | U(b >> (W - 1))) ^ U(1));                // tiered abs float: rotl 1, LSB flip
    } else {
        if constexpr (SIGN) return U(b ^ sb);                                // signed, MSB flip
        else return b;                                                       // unsigned
    }
}

template <typename U>
__device__ __forceinline__ uint32_t digit_of(U k, int pass) {
    return uint32_t(k >> (pass * kRadixBits)) & (kBuckets - 1);
}

// ---- wide keys --------------------------------------------------------------------------
// Two little-endian 64-bit words in 16-byte storage, as the reference's test128 / longdoubletest128
// (Radixsortbidi8.hpp:1061-1100, :1969-2404).  KeyWide<64>: a 128-bit key (integer, or a float
// word with the sign in bit 127).  KeyWide<16>: x87 extended precision, 64-bit significand in
// `lo`, sign and 15-bit exponent in the low 16 bits of `hi` (sign = bit 79 of the key); the upper
// 48 bits of `hi` are padding: ignored by the ordering, moved with the element.
template <int HB>
struct alignas(16) KeyWide {
    uint64_t lo, hi;
    static constexpr int kHighBits = HB;
    static constexpr uint64_t kHighMask = HB == 64 ? ~uint64_t(0) : ((uint64_t(1) << HB) - 1u);
};
using KeyU128 = KeyWide<64>;
using KeyX87 = KeyWide<16>;

template <typename U> struct KeyTraits {
    static constexpr int kDigits = int(sizeof(U));    // 8-bit digit passes
    __host__ __device__ static constexpr U fill() { return U(~U(0)); }
};
template <int HB> struct KeyTraits<KeyWide<HB>> {
    static constexpr int kDigits = 8 + HB / 8;
    __host__ __device__ static constexpr KeyWide<HB> fill() { return KeyWide<HB>{~uint64_t(0), ~uint64_t(0)}; }
};

// the complement of a filtered key (descending order), within the key's bits
template <typename U>
__host__ __device__ __forceinline__ U key_not(U k) { return U(~k); }
template <int HB>
__host__ __device__ __forceinline__ KeyWide<HB> key_not(KeyWide<HB> k) {
    return KeyWide<HB>{~k.lo, ~k.hi & KeyWide<HB>::kHighMask};
}

template <int HB>
__device__ __forceinline__ uint32_t digit_of(KeyWide<HB> k, int pass) {
    return uint32_t(pass < 8 ? (k.lo >> (pass * kRadixBits)) : (k.hi >> ((pass - 8) * kRadixBits))) & (kBuckets - 1);
}

// K(b) of the same 8 filter combinations on the (64 + HB)-bit key; the result keeps `hi` within
// HB bits, so the padding of an x87 key never reaches a digit
template <int MODE, int HB>
__host__ __device__ __forceinline__ KeyWide<HB> filter_key(KeyWide<HB> b) {
    using K = KeyWide<HB>;
    constexpr bool ABS = (MODE & 1) != 0, SIGN = (MODE & 2) != 0, FLTP = (MODE & 4) != 0;
    constexpr uint64_t hm = K::kHighMask, sb = uint64_t(1) << (HB - 1);
    uint64_t lo = b.lo, hi = b.hi & hm;
    const uint64_t s = (hi & sb) ? ~uint64_t(0) : 0u;   // sign mask, both words
    auto add_s = [&](uint64_t l, uint64_t h) {          // (l, h) + (s, s), two's complement
        const uint64_t r = l + s;
        return K{r, (h + s + uint64_t(r < l)) & hm};
    };
    auto shl1 = [&](uint64_t l, uint64_t h) { return K{l << 1, ((h << 1) | (l >> 63)) & hm}; };
    if constexpr (ABS != FLTP) {
        if constexpr (ABS) {
            if constexpr (SIGN) {                                            // absolute signed
                K r = add_s(lo, hi);
                return K{r.lo ^ s, (r.hi ^ s) & hm};
            } else {                                                         // tiered absolute signed
                K r = shl1(lo, hi);
                return K{r.lo ^ s, (r.hi ^ s) & hm};
            }
        } else {
            const uint64_t mh = hi & ~sb;
            if constexpr (SIGN) {                                            // floating point, MSB flip
                K r = add_s(lo, mh);
                return K{r.lo ^ s, ((r.hi ^ s) & hm) ^ sb};
            } else {                                                         // inside-out floating point
                return K{lo ^ s, (mh ^ s) & hm};
            }
        }
    } else if constexpr (ABS) {
        if constexpr (SIGN) return K{lo, hi & ~sb};                          // absolute floating point
        K r = shl1(lo, hi);                                                  // tiered abs float: rotl 1, LSB flip
        return K{(r.lo | (hi >> (HB - 1))) ^ 1u, r.hi};
    } else {
        if constexpr (SIGN) return K{lo, hi ^ sb};                           // signed, MSB flip
        return K{lo, hi};                                                    // unsigned
    }
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint64_t *p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// status word helpers: state in the top two bits, count below
template <typename S> struct StatusWord;
template <> struct StatusWord<uint32_t> {
    static constexpr int kShift = 30;
    __device__ static uint32_t make(uint32_t st, uint64_t v) { return (st << kShift) | uint32_t(v); }
    __device__ static uint32_t state(uint32_t w) { return w >> kShift; }
    __device__ static uint64_t value(uint32_t w) { return w & ((1u << kShift) - 1u); }
};
template <> struct StatusWord<uint64_t> {
    static constexpr int kShift = 62;
    __device__ static uint64_t make(uint32_t st, uint64_t v) { return (uint64_t(st) << kShift) | v; }
    __device__ static uint32_t state(uint64_t w) { return uint32_t(w >> kShift); }
    __device__ static uint64_t value(uint64_t w) { return w & ((uint64_t(1) << kShift) - 1u); }
};

// load the raw bits of a key through an object pointer (unaligned members allowed)
template <typename U>
__device__ __forceinline__ U load_member(const unsigned char *p) {
    if ((reinterpret_cast<uintptr_t>(p) & (sizeof(U) - 1)) == 0) return *reinterpret_cast<const U *>(p);
    U v = 0;
#pragma unroll
    for (int i = 0; i < int(sizeof(U)); ++i) v |= U(U(p[i]) << (8 * i));
    return v;
}

template <int HB>
__device__ __forceinline__ KeyWide<HB> load_member_wide(const unsigned char *p) {
    if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) return *reinterpret_cast<const KeyWide<HB> *>(p);
    KeyWide<HB> v{0, 0};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        v.lo |= uint64_t(p[i]) << (8 * i);
        v.hi |= uint64_t(p[8 + i]) << (8 * i);
    }
    return v;
}
template <>
__device__ __forceinline__ KeyU128 load_member<KeyU128>(const unsigned char *p) { return load_member_wide<64>(p); }
template <>
__device__ __forceinline__ KeyX87 load_member<KeyX87>(const unsigned char *p) { return load_member_wide<16>(p); }

__device__ __forceinline__ const unsigned char *load_ptr(const unsigned char *p) {
    if ((reinterpret_cast<uintptr_t>(p) & 7u) == 0) return *reinterpret_cast<const unsigned char *const *>(p);
    uint64_t v = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) v |= uint64_t(p[i]) << (8 * i);
    return reinterpret_cast<const unsigned char *>(v);
}

}  // namespace rsbd8g
