// rsbd8.hpp - header-only C++ facade of the GB300 radix sort with the template API of
// Radixsortbidi8.hpp (namespace rsbd8): the same function names, template parameters,
// argument order and bool results, over the C ABI of rsbd8g.h.  Arrays are device-resident
// (cudaMalloc / managed / system memory the GPU can reach); the sort runs on the stream set
// with rsbd8::setstream() (default: the legacy default stream).
//
// Kept from the reference:
//   sortingmode / sortingdirection values                 Radixsortbidi8.hpp:212-265
//   mode resolution from the key type (std::is_signed_v, std::is_floating_point_v on the
//   declared type, so enumerations sort as unsigned)      Radixsortbidi8.hpp:59778-59904
//   radixsort / radixsortcopy (allocate, return false only when allocation fails)
//                                                         Radixsortbidi8.hpp:60398, :60476
//   radixsortnoalloc / radixsortcopynoalloc (caller buffer; pzeroedindices is the device
//   scratch, sized by rsbd8::gpuscratchbytes; allowedthreads and pfuturesplaceholder are
//   accepted and have no GPU meaning)                     Radixsortbidi8.hpp:60129, :60163
//   indirection: member object pointer, pointer member (second level), getter member
//   function (+ arguments), type+offset (<T, offset1, ..., offset2>), and simple
//   second-level arrays (T *const *)                      Radixsortbidi8.hpp:60590-61739
//   index arguments and isindexed2 of the indirect forms (folded into one byte offset)
//                                                         Radixsortbidi8.hpp:2412-2470, :2787-2813
//   8-bit keys: the single-part noalloc forms without a buffer argument
//                                                         Radixsortbidi8.hpp:60193-60395
//   16-byte keys: 128-bit integers and classes (test128), long double (x87 in 16 bytes:
//   longdoubletest128; binary128 where long double is that)   Radixsortbidi8.hpp:1061-2404, :2849
// Getters are evaluated on the host for every element (C++ member functions cannot be
// called from the device), so their objects must be host-accessible; the keys then travel
// to the device and the pointers are sorted there.  The noalloc getter forms keep those keys
// in the tail of the caller's scratch (rsbd8::gpuscratchbytesgetter).
#pragma once

#include <cuda_runtime_api.h>

#include <cfloat>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <type_traits>
#include <utility>
#include <vector>

#include "rsbd8g.h"

namespace rsbd8 {

enum struct sortingmode : unsigned char {
    native = 64u, nativeabs = 65u, nativetieredabs = 66u,
    forceunsigned = 0u, specialsigned = forceunsigned, forcesigned = 1u << 1, forceabssigned = 1u | 1u << 1,
    forcefloatingp = 1u << 1 | 1u << 2, forceabsfloatingp = 1u | 1u << 1 | 1u << 2,
    specialunsigned = forceabsfloatingp, specialfloatingp = 1u << 2, forcetieredabsfloatingp = 1u | 1u << 2,
    forcetieredabssigned = 1u
};

enum struct sortingdirection : unsigned char {
    ascfwdorder = 0u, dscrevorder = 1u | 1u << 1, dscfwdorder = 1u, ascrevorder = 1u << 1
};

namespace gpu_detail {

inline rsbd8g_stream &stream_slot() {
    static thread_local rsbd8g_stream s = nullptr;
    return s;
}

// 128-bit integers count as integers even where the standard library does not say so
template <typename T>
constexpr bool isint128{
#ifdef __SIZEOF_INT128__
    std::is_same_v<std::remove_cv_t<T>, __int128> || std::is_same_v<std::remove_cv_t<T>, unsigned __int128>
#else
    false
#endif
};

// 16-byte keys: 128-bit integers, 16-byte classes, and long double where it fills 16 bytes
// (x87 extended precision on x86-64, IEEE binary128 on AArch64)
template <typename T>
constexpr bool iskeytype{(std::is_arithmetic_v<T> || std::is_enum_v<T> || isint128<T> ||
                          ((std::is_class_v<T> || std::is_union_v<T>) && std::is_trivially_copyable_v<T>)) &&
                         (sizeof(T) == 1 || sizeof(T) == 2 || sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16)};

template <typename T>
constexpr bool isx87{std::is_same_v<std::remove_cv_t<T>, long double> && LDBL_MANT_DIG == 64 && sizeof(T) == 16};

template <typename T>
constexpr uint32_t keykind{isx87<T>                                  ? uint32_t(RSBD8G_KIND_X87)
                           : std::is_floating_point_v<T>               ? uint32_t(RSBD8G_KIND_FLOAT)
#ifdef __SIZEOF_INT128__
                           : std::is_same_v<std::remove_cv_t<T>, __int128> ? uint32_t(RSBD8G_KIND_SIGNED)
#endif
                           : std::is_signed_v<T>                       ? uint32_t(RSBD8G_KIND_SIGNED)
                                                                       : uint32_t(RSBD8G_KIND_UNSIGNED)};

template <sortingdirection direction, sortingmode mode, typename T>
inline rsbd8g_desc makedesc(uint32_t indirection = RSBD8G_DIRECT, std::ptrdiff_t offset1 = 0,
                            std::ptrdiff_t offset2 = 0) {
    rsbd8g_desc d{};
    d.key_bytes = uint32_t(sizeof(T));
    d.key_kind = keykind<std::remove_cv_t<T>>;
    d.mode = uint32_t(mode);
    d.direction = uint32_t(direction);
    d.indirection = indirection;
    d.flags = 0;
    d.offset1 = int64_t(offset1);
    d.offset2 = int64_t(offset2);
    return d;
}

// byte offset of a data member (the reference's getoffsetof, Radixsortbidi8.hpp:719), at run time
template <auto member, typename C, typename M>
inline std::ptrdiff_t memberoffset(M C::*) {
    alignas(C) static unsigned char storage[sizeof(C)];
    C *c = reinterpret_cast<C *>(storage);
    return reinterpret_cast<unsigned char const *>(&(c->*member)) - storage;
}

template <auto member>
struct memberinfo;
template <typename C, typename M, M C::*member>
struct memberinfo<member> {
    using classtype = C;
    using membertype = std::remove_cv_t<M>;
};

inline bool ok(rsbd8g_status s) { return s == RSBD8G_OK; }

}  // namespace gpu_detail

// Select the CUDA stream (a cudaStream_t) the following calls of this thread run on.
inline void setstream(rsbd8g_stream stream) noexcept { gpu_detail::stream_slot() = stream; }

// Scratch bytes (device) the noalloc forms need; the stand-in for the index buffer that
// rsbd8::allocatearray sizes in the reference (Radixsortbidi8.hpp:59928).
// For 8-bit keys it also holds the ping-pong buffer of the single-part forms.
template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::size_t gpuscratchbytes(std::size_t count) noexcept {
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    std::size_t b = 0;
    if (rsbd8g_scratch_bytes(&d, count, &b) != RSBD8G_OK) return 0;
    return sizeof(T) == 1 ? ((b + 255u) & ~std::size_t(255u)) + count : b;
}

// ---- plain arrays ------------------------------------------------------------------------------

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<T>, bool>
radixsortcopy(std::size_t count, T const *input, T *output, int mmapflags = 0) noexcept {
    static_cast<void>(mmapflags);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    return gpu_detail::ok(rsbd8g_radixsortcopy(&d, count, input, output, gpu_detail::stream_slot()));
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<T>, bool>
radixsort(std::size_t count, T *input, int mmapflags = 0) noexcept {
    static_cast<void>(mmapflags);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    return gpu_detail::ok(rsbd8g_radixsort(&d, count, input, gpu_detail::stream_slot()));
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::enable_if_t<gpu_detail::iskeytype<T>, void>
radixsortcopynoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                     T const *input, T *output, T *buffer) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    rsbd8g_radixsortcopynoalloc(&d, count, pzeroedindices, gpuscratchbytes<direction, mode, T>(count), input, output,
                                buffer, gpu_detail::stream_slot());
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::enable_if_t<gpu_detail::iskeytype<T>, void>
radixsortcopynoalloc(std::size_t count, void *pzeroedindices, T const *input, T *output, T *buffer) noexcept {
    radixsortcopynoalloc<direction, mode, T>(count, 1u, nullptr, pzeroedindices, input, output, buffer);
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::enable_if_t<gpu_detail::iskeytype<T>, void>
radixsortnoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                 T *input, T *buffer, bool movetobuffer = false) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    rsbd8g_radixsortnoalloc(&d, count, pzeroedindices, gpuscratchbytes<direction, mode, T>(count), input, buffer,
                            movetobuffer ? 1 : 0, gpu_detail::stream_slot());
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::enable_if_t<gpu_detail::iskeytype<T>, void>
radixsortnoalloc(std::size_t count, void *pzeroedindices, T *input, T *buffer, bool movetobuffer = false) noexcept {
    radixsortnoalloc<direction, mode, T>(count, 1u, nullptr, pzeroedindices, input, buffer, movetobuffer);
}

// single-part forms of 8-bit keys: no buffer argument, the buffer sits at the end of the scratch
template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::enable_if_t<gpu_detail::iskeytype<T> && sizeof(T) == 1, void>
radixsortcopynoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                     T const *input, T *output) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    const std::size_t all = gpuscratchbytes<direction, mode, T>(count), own = all - count;
    rsbd8g_radixsortcopynoalloc(&d, count, pzeroedindices, own, input, output,
                                static_cast<unsigned char *>(pzeroedindices) + own, gpu_detail::stream_slot());
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::enable_if_t<gpu_detail::iskeytype<T> && sizeof(T) == 1, void>
radixsortnoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                 T *input) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    const std::size_t all = gpuscratchbytes<direction, mode, T>(count), own = all - count;
    rsbd8g_radixsortnoalloc(&d, count, pzeroedindices, own, input,
                            static_cast<unsigned char *>(pzeroedindices) + own, 0, gpu_detail::stream_slot());
}

// ---- indirection: where the key sits --------------------------------------------------------------
// In the member-object-pointer, type+offset and simple second-level forms the key of element i
// lies at byte
//     offset1 + indirection2 + (index1 + index2) * sizeof(key)
// of the object input[i] points to: indirection2 and every index argument only move the key within
// the object (splitgetobject Radixsortbidi8.hpp:2412-2470, indirectinput1 :2740-2770,
// indirectinput2 :2787-2813), so they fold into one byte offset shared by all elements.
// A data member or type+offset form whose type is itself a pointer makes the reference stop at a
// static assertion ("third level indirection", Radixsortbidi8.hpp:2762-2764); the facade gives it
// the natural meaning instead: the pointer at offset1 (+ index1 pointers) is loaded and the key
// sits at indirection2 + index2 * sizeof(key) behind it.

namespace gpu_detail {

template <typename... A>
constexpr bool indicesok{sizeof...(A) <= 2 && (std::is_integral_v<std::remove_cv_t<std::remove_reference_t<A>>> && ...)};

template <bool isindexed2, typename... A>
constexpr void checkindices() {
    static_assert(indicesok<A...>, "at most two integer index arguments");
    static_assert(!isindexed2 || sizeof...(A) >= 1, "isindexed2 needs an index argument");
    static_assert(sizeof...(A) < 2 || isindexed2, "two index arguments need isindexed2");
}

// descriptor of an indirect sort of keys of type K; pointerlevel: the object holds a pointer to
// the key's object instead of the key
template <sortingdirection direction, sortingmode mode, typename K, bool pointerlevel, bool isindexed2,
          typename... A>
inline rsbd8g_desc indirectdesc(std::ptrdiff_t offset1, std::ptrdiff_t indirection2, A... index) {
    checkindices<isindexed2, A...>();
    std::ptrdiff_t ix[2]{0, 0};
    [[maybe_unused]] std::size_t k = 0;
    ((ix[k++] = std::ptrdiff_t(index)), ...);
    if constexpr (!pointerlevel) {
        return makedesc<direction, mode, K>(RSBD8G_MEMBER,
                                            offset1 + indirection2 + (ix[0] + ix[1]) * std::ptrdiff_t(sizeof(K)));
    } else {
        // one index: first level unless isindexed2; two indices: first and second level
        const std::ptrdiff_t i1 = (sizeof...(A) == 2 || !isindexed2) ? ix[0] : 0;
        const std::ptrdiff_t i2 = sizeof...(A) == 2 ? ix[1] : (isindexed2 ? ix[0] : 0);
        return makedesc<direction, mode, K>(RSBD8G_MEMBER2, offset1 + i1 * std::ptrdiff_t(sizeof(void *)),
                                            indirection2 + i2 * std::ptrdiff_t(sizeof(K)));
    }
}

inline std::size_t scratchfor(const rsbd8g_desc &d, std::size_t count) {
    std::size_t b = 0;
    return rsbd8g_scratch_bytes(&d, count, &b) == RSBD8G_OK ? b : 0;
}

inline bool copyindirect(const rsbd8g_desc &d, std::size_t count, const void *input, void *output) {
    return ok(rsbd8g_radixsortcopy(&d, count, input, output, stream_slot()));
}

inline bool sortindirect(const rsbd8g_desc &d, std::size_t count, void *input) {
    return ok(rsbd8g_radixsort(&d, count, input, stream_slot()));
}

inline void copyindirectnoalloc(const rsbd8g_desc &d, std::size_t count, void *scratch, const void *input,
                                void *output, void *buffer) {
    rsbd8g_radixsortcopynoalloc(&d, count, scratch, scratchfor(d, count), input, output, buffer, stream_slot());
}

inline void sortindirectnoalloc(const rsbd8g_desc &d, std::size_t count, void *scratch, void *input, void *buffer,
                                bool movetobuffer) {
    rsbd8g_radixsortnoalloc(&d, count, scratch, scratchfor(d, count), input, buffer, movetobuffer ? 1 : 0,
                            stream_slot());
}

}  // namespace gpu_detail

// Scratch bytes (device) of the noalloc forms with indirection, for keys of type K.
template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename K>
inline std::size_t gpuscratchbytesindirect(std::size_t count) noexcept {
    return gpu_detail::scratchfor(gpu_detail::makedesc<direction, mode, K>(RSBD8G_MEMBER), count);
}

// ---- simple second-level arrays: T *const *input, the key of type T at the folded offset ---------

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          std::ptrdiff_t indirection2 = 0, bool isindexed2 = false, typename T, typename... A>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<T>> && gpu_detail::indicesok<A...>, bool>
radixsortcopy(std::size_t count, T *const *input, T **output, int mmapflags = 0, A... index) noexcept {
    static_cast<void>(mmapflags);
    return gpu_detail::copyindirect(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<T>, false, isindexed2>(0, indirection2, index...),
        count, input, output);
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          std::ptrdiff_t indirection2 = 0, bool isindexed2 = false, typename T, typename... A>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<T>> && gpu_detail::indicesok<A...>, bool>
radixsort(std::size_t count, T **input, int mmapflags = 0, A... index) noexcept {
    static_cast<void>(mmapflags);
    return gpu_detail::sortindirect(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<T>, false, isindexed2>(0, indirection2, index...),
        count, input);
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          std::ptrdiff_t indirection2 = 0, bool isindexed2 = false, typename T, typename... A>
inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<T>> && gpu_detail::indicesok<A...>, void>
radixsortcopynoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                     T *const *input, T **output, T **buffer, A... index) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    gpu_detail::copyindirectnoalloc(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<T>, false, isindexed2>(0, indirection2, index...),
        count, pzeroedindices, input, output, buffer);
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          std::ptrdiff_t indirection2 = 0, bool isindexed2 = false, typename T, typename... A>
inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<T>> && gpu_detail::indicesok<A...>, void>
radixsortnoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                 T **input, T **buffer, bool movetobuffer = false, A... index) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    gpu_detail::sortindirectnoalloc(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<T>, false, isindexed2>(0, indirection2, index...),
        count, pzeroedindices, input, buffer, movetobuffer);
}

// ---- member object pointer: the key member (or a pointer member, see above) ---------------------

namespace gpu_detail {

template <auto member>
using memberkey = std::remove_cv_t<std::remove_pointer_t<typename memberinfo<member>::membertype>>;

template <auto member>
constexpr bool memberispointer{std::is_pointer_v<typename memberinfo<member>::membertype>};

template <auto indirection1, sortingdirection direction, sortingmode mode, std::ptrdiff_t indirection2,
          bool isindexed2, typename... A>
inline rsbd8g_desc memberdesc(A... index) {
    static_assert(iskeytype<memberkey<indirection1>>, "unsupported key type");
    return indirectdesc<direction, mode, memberkey<indirection1>, memberispointer<indirection1>, isindexed2>(
        memberoffset<indirection1>(indirection1), indirection2, index...);
}

}  // namespace gpu_detail

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
[[nodiscard]] inline std::enable_if_t<std::is_member_object_pointer_v<decltype(indirection1)> &&
                                          gpu_detail::indicesok<A...>, bool>
radixsortcopy(std::size_t count, V *const *input, V **output, int mmapflags = 0, A... index) noexcept {
    static_cast<void>(mmapflags);
    return gpu_detail::copyindirect(
        gpu_detail::memberdesc<indirection1, direction, mode, indirection2, isindexed2>(index...), count, input,
        output);
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
[[nodiscard]] inline std::enable_if_t<std::is_member_object_pointer_v<decltype(indirection1)> &&
                                          gpu_detail::indicesok<A...>, bool>
radixsort(std::size_t count, V **input, int mmapflags = 0, A... index) noexcept {
    static_cast<void>(mmapflags);
    return gpu_detail::sortindirect(
        gpu_detail::memberdesc<indirection1, direction, mode, indirection2, isindexed2>(index...), count, input);
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
inline std::enable_if_t<std::is_member_object_pointer_v<decltype(indirection1)> && gpu_detail::indicesok<A...>, void>
radixsortcopynoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                     V *const *input, V **output, V **buffer, A... index) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    gpu_detail::copyindirectnoalloc(
        gpu_detail::memberdesc<indirection1, direction, mode, indirection2, isindexed2>(index...), count,
        pzeroedindices, input, output, buffer);
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
inline std::enable_if_t<std::is_member_object_pointer_v<decltype(indirection1)> && gpu_detail::indicesok<A...>, void>
radixsortnoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                 V **input, V **buffer, bool movetobuffer = false, A... index) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    gpu_detail::sortindirectnoalloc(
        gpu_detail::memberdesc<indirection1, direction, mode, indirection2, isindexed2>(index...), count,
        pzeroedindices, input, buffer, movetobuffer);
}

// ---- getter member function (evaluated on the host), with optional extra arguments ----------------
// The key of element i is what input[i]->*getter returns (splitgetfunction, Radixsortbidi8.hpp:
// 2646-2706; indirectinput1 :2768-2784): the returned value itself, or -- when the getter returns a
// pointer or an lvalue reference -- the key at byte indirection2 behind it, the index2-th key there
// with isindexed2 (indirectinput2 :2806-2812).  With isindexed2 the first extra argument is index2
// and the others go to the getter.  The facade calls the getter on the host for every element (the
// objects, and what the getter returns a pointer to, must be host-accessible), copies the keys to
// the device and sorts the pointers by them there.

namespace gpu_detail {

template <auto getter, typename V, typename... A>
using getterresult = decltype((std::declval<V *>()->*getter)(std::declval<A>()...));

// the getter's result type with the extra arguments it is called with (index2 split off)
template <auto getter, bool isindexed2, typename V, typename... A>
struct gettercall;
template <auto getter, typename V, typename... A>
struct gettercall<getter, false, V, A...> {
    using result = getterresult<getter, V, A...>;
};
template <auto getter, typename V, typename I, typename... A>
struct gettercall<getter, true, V, I, A...> {
    static_assert(std::is_integral_v<std::remove_cv_t<std::remove_reference_t<I>>>, "isindexed2: the first extra argument is the index");
    using result = getterresult<getter, V, A...>;
};

template <typename R>
constexpr bool getterpoints{std::is_lvalue_reference_v<R> || std::is_pointer_v<std::remove_reference_t<R>>};

template <typename R>
using getterkey = std::remove_cv_t<std::conditional_t<std::is_lvalue_reference_v<R>, std::remove_reference_t<R>,
                                                      std::remove_pointer_t<std::remove_reference_t<R>>>>;

// the key of one element from the getter's result
template <typename K, std::ptrdiff_t indirection2, typename R>
inline K keyfromresult(R &&r, std::ptrdiff_t index2) {
    K k;
    if constexpr (std::is_lvalue_reference_v<R>) {
        const unsigned char *b = reinterpret_cast<const unsigned char *>(std::addressof(r));
        std::memcpy(&k, b + indirection2 + index2 * std::ptrdiff_t(sizeof(K)), sizeof(K));
    } else if constexpr (std::is_pointer_v<std::remove_reference_t<R>>) {
        const unsigned char *b = reinterpret_cast<const unsigned char *>(r);
        std::memcpy(&k, b + indirection2 + index2 * std::ptrdiff_t(sizeof(K)), sizeof(K));
    } else {
        std::memcpy(&k, &r, sizeof(K));
    }
    return k;
}

template <auto getter, std::ptrdiff_t indirection2, typename K, typename V, typename... A>
inline void getkeys(std::size_t count, V *const *p, K *keys, std::false_type, A &&...a) {
    for (std::size_t i = 0; i < count; ++i) keys[i] = keyfromresult<K, indirection2>((p[i]->*getter)(a...), 0);
}
template <auto getter, std::ptrdiff_t indirection2, typename K, typename V, typename I, typename... A>
inline void getkeys(std::size_t count, V *const *p, K *keys, std::true_type, I &&index2, A &&...a) {
    for (std::size_t i = 0; i < count; ++i)
        keys[i] = keyfromresult<K, indirection2>((p[i]->*getter)(a...), std::ptrdiff_t(index2));
}

template <auto getter, std::ptrdiff_t indirection2, bool isindexed2, typename V, typename... A>
struct getterinfo {
    using R = typename gettercall<getter, isindexed2, V, A...>::result;
    using K = getterkey<R>;
    static_assert(getterpoints<R> || (!isindexed2 && indirection2 == 0),
                  "a getter that returns the key itself takes neither indirection2 nor isindexed2");
    static_assert(!std::is_pointer_v<K>, "third level indirection is not supported");
    static_assert(iskeytype<K>, "unsupported key type");
};

// the pointers of input (device or host memory) on the host, ordered after the stream's work
template <typename V>
inline bool hostpointers(std::size_t count, V *const *input, std::vector<V *> &ptrs) {
    ptrs.resize(count);
    return cudaMemcpyAsync(ptrs.data(), input, count * sizeof(V *), cudaMemcpyDefault,
                           reinterpret_cast<cudaStream_t>(stream_slot())) == cudaSuccess &&
           cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream_slot())) == cudaSuccess;
}

// every element's key evaluated on the host, then copied to `dkeys` (device) on the stream
template <auto getter, std::ptrdiff_t indirection2, bool isindexed2, typename V, typename... A>
inline bool hostkeys(std::size_t count, V *const *input, void *dkeys, A &&...a) {
    using K = typename getterinfo<getter, indirection2, isindexed2, V, A...>::K;
    std::vector<V *> ptrs;
    if (!hostpointers(count, input, ptrs)) return false;
    std::vector<K> keys(count);
    getkeys<getter, indirection2, K>(count, ptrs.data(), keys.data(), std::bool_constant<isindexed2>{},
                                     std::forward<A>(a)...);
    // a copy from pageable memory is staged before the call returns: `keys` may go
    return cudaMemcpyAsync(dkeys, keys.data(), count * sizeof(K), cudaMemcpyHostToDevice,
                           reinterpret_cast<cudaStream_t>(stream_slot())) == cudaSuccess;
}

inline std::size_t keyedscratch(const rsbd8g_desc &d, std::size_t count) {
    std::size_t b = 0;
    return rsbd8g_scratch_bytes(&d, count, &b) == RSBD8G_OK ? (b + 255u) & ~std::size_t(255u) : 0;
}

}  // namespace gpu_detail

// Scratch bytes (device) of the noalloc forms with a getter whose keys have type K: the sort's own
// scratch, then room for the keys the host evaluates.
template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename K>
inline std::size_t gpuscratchbytesgetter(std::size_t count) noexcept {
    return gpu_detail::keyedscratch(gpu_detail::makedesc<direction, mode, K>(RSBD8G_KEYED), count) + count * sizeof(K);
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... vararguments>
[[nodiscard]] inline std::enable_if_t<std::is_member_function_pointer_v<decltype(indirection1)>, bool>
radixsortcopy(std::size_t count, V *const *input, V **output, int mmapflags = 0, vararguments &&...varparameters) {
    using info = gpu_detail::getterinfo<indirection1, indirection2, isindexed2, V, vararguments...>;
    using K = typename info::K;
    static_cast<void>(mmapflags);
    if (count < 2) {
        if (count == 1) return cudaMemcpy(output, input, sizeof(V *), cudaMemcpyDefault) == cudaSuccess;
        return true;
    }
    void *dkeys = nullptr;
    if (cudaMalloc(&dkeys, count * sizeof(K)) != cudaSuccess) return false;
    bool good = gpu_detail::hostkeys<indirection1, indirection2, isindexed2>(
        count, input, dkeys, std::forward<vararguments>(varparameters)...);
    if (good) {
        rsbd8g_desc d = gpu_detail::makedesc<direction, mode, K>(RSBD8G_KEYED);
        good = gpu_detail::ok(rsbd8g_radixsortcopy_keyed(&d, count, dkeys, input, output, gpu_detail::stream_slot()));
    }
    cudaFree(dkeys);
    return good;
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... vararguments>
[[nodiscard]] inline std::enable_if_t<std::is_member_function_pointer_v<decltype(indirection1)>, bool>
radixsort(std::size_t count, V **input, int mmapflags = 0, vararguments &&...varparameters) {
    if (count < 2) return true;
    V **tmp = nullptr;
    if (cudaMalloc(reinterpret_cast<void **>(&tmp), count * sizeof(V *)) != cudaSuccess) return false;
    bool good = radixsortcopy<indirection1, direction, mode, indirection2, isindexed2, V>(
        count, input, tmp, mmapflags, std::forward<vararguments>(varparameters)...);
    if (good) good = cudaMemcpy(input, tmp, count * sizeof(V *), cudaMemcpyDefault) == cudaSuccess;
    cudaFree(tmp);
    return good;
}

// The noalloc forms with a getter: pzeroedindices is device scratch of gpuscratchbytesgetter<...,
// K>(count) bytes; the keys evaluated on the host are stored in its tail.  These forms wait for the
// stream before they read the input pointers on the host; the sort itself is stream-ordered.
template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... vararguments>
inline std::enable_if_t<std::is_member_function_pointer_v<decltype(indirection1)>, void>
radixsortcopynoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                     V *const *input, V **output, V **buffer, vararguments &&...varparameters) {
    using K = typename gpu_detail::getterinfo<indirection1, indirection2, isindexed2, V, vararguments...>::K;
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    if (count < 2) {
        if (count == 1) cudaMemcpy(output, input, sizeof(V *), cudaMemcpyDefault);
        return;
    }
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, K>(RSBD8G_KEYED);
    const std::size_t own = gpu_detail::keyedscratch(d, count);
    void *dkeys = static_cast<unsigned char *>(pzeroedindices) + own;
    if (!gpu_detail::hostkeys<indirection1, indirection2, isindexed2>(count, input, dkeys,
                                                                        std::forward<vararguments>(varparameters)...))
        return;
    rsbd8g_radixsortcopynoalloc_keyed(&d, count, dkeys, pzeroedindices, own, input, output, buffer,
                                      gpu_detail::stream_slot());
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... vararguments>
inline std::enable_if_t<std::is_member_function_pointer_v<decltype(indirection1)>, void>
radixsortnoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                 V **input, V **buffer, bool movetobuffer = false, vararguments &&...varparameters) {
    using K = typename gpu_detail::getterinfo<indirection1, indirection2, isindexed2, V, vararguments...>::K;
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    if (count < 2) {
        if (count == 1 && movetobuffer) cudaMemcpy(buffer, input, sizeof(V *), cudaMemcpyDefault);
        return;
    }
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, K>(RSBD8G_KEYED);
    const std::size_t own = gpu_detail::keyedscratch(d, count);
    void *dkeys = static_cast<unsigned char *>(pzeroedindices) + own;
    if (!gpu_detail::hostkeys<indirection1, indirection2, isindexed2>(count, input, dkeys,
                                                                        std::forward<vararguments>(varparameters)...))
        return;
    rsbd8g_radixsortnoalloc_keyed(&d, count, dkeys, pzeroedindices, own, input, buffer, movetobuffer ? 1 : 0,
                                  gpu_detail::stream_slot());
}

// ---- type + offset: <T, indirection1, direction, mode, indirection2, isindexed2> ------------------
// T not a pointer: the key of type T at byte indirection1 (folded with indirection2 and the
// indices as above).  T a pointer type U *: the pointer at byte indirection1, the key of type U
// behind it (see above).

template <typename T, std::ptrdiff_t indirection1 = 0, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
[[nodiscard]] inline std::enable_if_t<
    gpu_detail::iskeytype<std::remove_cv_t<std::remove_pointer_t<T>>> && gpu_detail::indicesok<A...>, bool>
radixsortcopy(std::size_t count, V *const *input, V **output, int mmapflags = 0, A... index) noexcept {
    static_cast<void>(mmapflags);
    return gpu_detail::copyindirect(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<std::remove_pointer_t<T>>, std::is_pointer_v<T>,
                                 isindexed2>(indirection1, indirection2, index...),
        count, input, output);
}

template <typename T, std::ptrdiff_t indirection1 = 0, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
[[nodiscard]] inline std::enable_if_t<
    gpu_detail::iskeytype<std::remove_cv_t<std::remove_pointer_t<T>>> && gpu_detail::indicesok<A...>, bool>
radixsort(std::size_t count, V **input, int mmapflags = 0, A... index) noexcept {
    static_cast<void>(mmapflags);
    return gpu_detail::sortindirect(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<std::remove_pointer_t<T>>, std::is_pointer_v<T>,
                                 isindexed2>(indirection1, indirection2, index...),
        count, input);
}

template <typename T, std::ptrdiff_t indirection1 = 0, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<std::remove_pointer_t<T>>> &&
                            gpu_detail::indicesok<A...>, void>
radixsortcopynoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                     V *const *input, V **output, V **buffer, A... index) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    gpu_detail::copyindirectnoalloc(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<std::remove_pointer_t<T>>, std::is_pointer_v<T>,
                                 isindexed2>(indirection1, indirection2, index...),
        count, pzeroedindices, input, output, buffer);
}

template <typename T, std::ptrdiff_t indirection1 = 0, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... A>
inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<std::remove_pointer_t<T>>> &&
                            gpu_detail::indicesok<A...>, void>
radixsortnoalloc(std::size_t count, unsigned allowedthreads, void *pfuturesplaceholder, void *pzeroedindices,
                 V **input, V **buffer, bool movetobuffer = false, A... index) noexcept {
    static_cast<void>(allowedthreads);
    static_cast<void>(pfuturesplaceholder);
    gpu_detail::sortindirectnoalloc(
        gpu_detail::indirectdesc<direction, mode, std::remove_cv_t<std::remove_pointer_t<T>>, std::is_pointer_v<T>,
                                 isindexed2>(indirection1, indirection2, index...),
        count, pzeroedindices, input, buffer, movetobuffer);
}

}  // namespace rsbd8
