// ref_adapter.cpp - exposes the reference's own CPU sort (Radixsortbidi8.hpp) to the
// oracle tests through plain extern "C" functions.  Test infrastructure only.
//
// This file holds no reference code: it includes the reference header from the
// reference tree (the build recipe passes -I to it) and instantiates its public
// templates, exactly as a user of the reference would:
//   rsbd8::radixsortcopy<direction, mode>(count, input, output)   Radixsortbidi8.hpp:60476
//   rsbd8::radixsort<direction, mode>(count, input)               Radixsortbidi8.hpp:60398
//   rsbd8::radixsortcopy<T, offset, direction, mode>(count, in, out) (type+offset indirection)
//                                                                 Radixsortbidi8.hpp:61359-61739
//   rsbd8::radixsortcopy<&S::member, direction, mode>(count, in, out) (member pointer)
//                                                                 Radixsortbidi8.hpp:61242
// Only the modes that are sound at the pinned snapshot are instantiated: the
// regular absolute modes write out of bounds and tiered-absolute floating point
// returns a wrong order, so those are never run (their oracle is the C restatement).
//
// The build compiles this file once per REF_PART value so the instantiations
// spread over several translation units (the header is large).
#include "Radixsortbidi8.hpp"
#include <cstdint>

using rsbd8::sortingdirection;
using rsbd8::sortingmode;

namespace {
template<sortingdirection D, sortingmode M, typename T>
int copy_impl(std::uint64_t n, void const *in, void *out) {
	return rsbd8::radixsortcopy<D, M>(n, static_cast<T const *>(in), static_cast<T *>(out)) ? 0 : -2;
}
template<sortingdirection D, sortingmode M, typename T>
int inplace_impl(std::uint64_t n, void *a) {
	return rsbd8::radixsort<D, M>(n, static_cast<T *>(a)) ? 0 : -2;
}
// 24-byte record used by the indirection cases: {u64 id; key at byte 8; u32 tag; u32 pad}
struct rec24 { std::uint64_t id; double key; std::uint32_t tag; std::uint32_t pad; };
static_assert(sizeof(rec24) == 24);
template<sortingdirection D, sortingmode M, typename T>
int indirect_impl(std::uint64_t n, void const *in, void *out) {
	return rsbd8::radixsortcopy<T, 8, D, M>(n, static_cast<rec24 *const *>(in), static_cast<rec24 **>(out)) ? 0 : -2;
}
// 16-byte key as a plain class: two little-endian 64-bit words
struct k128 { std::uint64_t lo, hi; };
static_assert(sizeof(k128) == 16);
static_assert(sizeof(long double) == 16, "x86-64 long double: x87 extended precision in 16 bytes");
template<sortingdirection D>
int member_impl(std::uint64_t n, void const *in, void *out) {
	return rsbd8::radixsortcopy<&rec24::key, D>(n, static_cast<rec24 *const *>(in), static_cast<rec24 **>(out)) ? 0 : -2;
}
}// namespace

#define RSBD8REF_DIRS(X, ...) X(__VA_ARGS__, ascfwdorder, 0) X(__VA_ARGS__, dscfwdorder, 1) \
	X(__VA_ARGS__, ascrevorder, 2) X(__VA_ARGS__, dscrevorder, 3)
#define RSBD8REF_COPY(T, tn, M, mv, D, dv) extern "C" int rsbd8ref_copy_##tn##_m##mv##_d##dv( \
	std::uint64_t n, void const *in, void *out) { return copy_impl<sortingdirection::D, sortingmode::M, T>(n, in, out); }
#define RSBD8REF_INPLACE(T, tn, M, mv, D, dv) extern "C" int rsbd8ref_inplace_##tn##_m##mv##_d##dv( \
	std::uint64_t n, void *a) { return inplace_impl<sortingdirection::D, sortingmode::M, T>(n, a); }
#define RSBD8REF_INDIRECT(T, tn, M, mv, D, dv) extern "C" int rsbd8ref_indirect8_##tn##_m##mv##_d##dv( \
	std::uint64_t n, void const *in, void *out) { return indirect_impl<sortingdirection::D, sortingmode::M, T>(n, in, out); }
#define RSBD8REF_MEMBER(unused, D, dv) extern "C" int rsbd8ref_member_key_d##dv( \
	std::uint64_t n, void const *in, void *out) { return member_impl<sortingdirection::D>(n, in, out); }

#if REF_PART == 0
// native mode on every plain key type, all four directions
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint8_t, u8, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, std::int8_t, i8, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint16_t, u16, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, std::int16_t, i16, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint32_t, u32, native, 64)
#elif REF_PART == 1
RSBD8REF_DIRS(RSBD8REF_COPY, std::int32_t, i32, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, float, f32, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint64_t, u64, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, std::int64_t, i64, native, 64)
RSBD8REF_DIRS(RSBD8REF_COPY, double, f64, native, 64)
#elif REF_PART == 2
// forced modes on 16-bit keys (the mode bits, not the type, pick the filter)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint16_t, u16, forceunsigned, 0)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint16_t, u16, forcetieredabssigned, 1)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint16_t, u16, forcesigned, 2)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint16_t, u16, specialfloatingp, 4)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint16_t, u16, forcefloatingp, 6)
#elif REF_PART == 3
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint32_t, u32, forcetieredabssigned, 1)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint32_t, u32, forcesigned, 2)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint32_t, u32, specialfloatingp, 4)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint32_t, u32, forcefloatingp, 6)
RSBD8REF_DIRS(RSBD8REF_COPY, std::int32_t, i32, nativetieredabs, 66)
#elif REF_PART == 4
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint64_t, u64, forcetieredabssigned, 1)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint64_t, u64, forcesigned, 2)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint64_t, u64, specialfloatingp, 4)
RSBD8REF_DIRS(RSBD8REF_COPY, std::uint64_t, u64, forcefloatingp, 6)
RSBD8REF_DIRS(RSBD8REF_COPY, std::int64_t, i64, nativetieredabs, 66)
#elif REF_PART == 5
// first-level type+offset indirection: key at byte 8 of a 24-byte record
RSBD8REF_DIRS(RSBD8REF_INDIRECT, std::uint32_t, u32, native, 64)
RSBD8REF_DIRS(RSBD8REF_INDIRECT, float, f32, native, 64)
RSBD8REF_DIRS(RSBD8REF_INDIRECT, std::int64_t, i64, native, 64)
RSBD8REF_DIRS(RSBD8REF_INDIRECT, double, f64, native, 64)
RSBD8REF_DIRS(RSBD8REF_INDIRECT, std::uint16_t, u16, native, 64)
#elif REF_PART == 6
RSBD8REF_DIRS(RSBD8REF_MEMBER, 0)
// in-place radixsort
RSBD8REF_DIRS(RSBD8REF_INPLACE, std::uint32_t, u32, native, 64)
RSBD8REF_DIRS(RSBD8REF_INPLACE, float, f32, native, 64)
RSBD8REF_DIRS(RSBD8REF_INPLACE, std::int64_t, i64, native, 64)
RSBD8REF_DIRS(RSBD8REF_INPLACE, double, f64, native, 64)
RSBD8REF_DIRS(RSBD8REF_INPLACE, std::int16_t, i16, native, 64)
#elif REF_PART == 7
// 16-byte keys: a 16-byte class (two little-endian 64-bit words; the reference's test128 with
// the mode bits of the call) under the sound forced modes, and long double (x87 extended
// precision in 16-byte storage on x86-64: the reference's longdoubletest128)
RSBD8REF_DIRS(RSBD8REF_COPY, k128, w128, forceunsigned, 0)
RSBD8REF_DIRS(RSBD8REF_COPY, k128, w128, forcetieredabssigned, 1)
RSBD8REF_DIRS(RSBD8REF_COPY, k128, w128, forcesigned, 2)
RSBD8REF_DIRS(RSBD8REF_COPY, k128, w128, specialfloatingp, 4)
RSBD8REF_DIRS(RSBD8REF_COPY, k128, w128, forcefloatingp, 6)
RSBD8REF_DIRS(RSBD8REF_COPY, long double, x87, native, 64)
#else
#error "REF_PART must be 0..7"
#endif
