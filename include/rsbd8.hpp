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
// Getters are evaluated on the host for every element (C++ member functions cannot be
// called from the device), so their objects must be host-accessible; the keys then travel
// to the device and the pointers are sorted there.  Indexed second-level indirection
// (isindexed2 = true) is not available on this path.
#pragma once

#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
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

template <typename T>
constexpr bool iskeytype{(std::is_arithmetic_v<T> || std::is_enum_v<T> ||
                          ((std::is_class_v<T> || std::is_union_v<T>) && std::is_trivially_copyable_v<T>)) &&
                         (sizeof(T) == 1 || sizeof(T) == 2 || sizeof(T) == 4 || sizeof(T) == 8)};

template <typename T>
constexpr uint32_t keykind{std::is_floating_point_v<T> ? uint32_t(RSBD8G_KIND_FLOAT)
                           : std::is_signed_v<T>        ? uint32_t(RSBD8G_KIND_SIGNED)
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
template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          typename T>
inline std::size_t gpuscratchbytes(std::size_t count) noexcept {
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>();
    std::size_t b = 0;
    return rsbd8g_scratch_bytes(&d, count, &b) == RSBD8G_OK ? b : 0;
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

// ---- simple second-level arrays: T *const *input, key at byte indirection2 behind each pointer -----

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          std::ptrdiff_t indirection2 = 0, bool isindexed2 = false, typename T>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<T>>, bool>
radixsortcopy(std::size_t count, T *const *input, T **output, int mmapflags = 0) noexcept {
    static_assert(!isindexed2, "indexed second-level indirection is not available on the GPU path");
    static_cast<void>(mmapflags);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, std::remove_cv_t<T>>(RSBD8G_MEMBER, indirection2);
    return gpu_detail::ok(rsbd8g_radixsortcopy(&d, count, input, output, gpu_detail::stream_slot()));
}

template <sortingdirection direction = sortingdirection::ascfwdorder, sortingmode mode = sortingmode::native,
          std::ptrdiff_t indirection2 = 0, bool isindexed2 = false, typename T>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<T>>, bool>
radixsort(std::size_t count, T **input, int mmapflags = 0) noexcept {
    static_assert(!isindexed2, "indexed second-level indirection is not available on the GPU path");
    static_cast<void>(mmapflags);
    rsbd8g_desc d = gpu_detail::makedesc<direction, mode, std::remove_cv_t<T>>(RSBD8G_MEMBER, indirection2);
    return gpu_detail::ok(rsbd8g_radixsort(&d, count, input, gpu_detail::stream_slot()));
}

// ---- member object pointer (key member, or a pointer member for second-level indirection) --------

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V>
[[nodiscard]] inline std::enable_if_t<std::is_member_object_pointer_v<decltype(indirection1)>, bool>
radixsortcopy(std::size_t count, V *const *input, V **output, int mmapflags = 0) noexcept {
    static_assert(!isindexed2, "indexed second-level indirection is not available on the GPU path");
    static_cast<void>(mmapflags);
    using M = typename gpu_detail::memberinfo<indirection1>::membertype;
    const std::ptrdiff_t off = gpu_detail::memberoffset<indirection1>(indirection1);
    if constexpr (std::is_pointer_v<M>) {
        using T = std::remove_cv_t<std::remove_pointer_t<M>>;
        static_assert(gpu_detail::iskeytype<T>, "unsupported key type");
        rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>(RSBD8G_MEMBER2, off, indirection2);
        return gpu_detail::ok(rsbd8g_radixsortcopy(&d, count, input, output, gpu_detail::stream_slot()));
    } else {
        static_assert(gpu_detail::iskeytype<M>, "unsupported key type");
        rsbd8g_desc d = gpu_detail::makedesc<direction, mode, M>(RSBD8G_MEMBER, off);
        return gpu_detail::ok(rsbd8g_radixsortcopy(&d, count, input, output, gpu_detail::stream_slot()));
    }
}

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V>
[[nodiscard]] inline std::enable_if_t<std::is_member_object_pointer_v<decltype(indirection1)>, bool>
radixsort(std::size_t count, V **input, int mmapflags = 0) noexcept {
    static_assert(!isindexed2, "indexed second-level indirection is not available on the GPU path");
    static_cast<void>(mmapflags);
    using M = typename gpu_detail::memberinfo<indirection1>::membertype;
    const std::ptrdiff_t off = gpu_detail::memberoffset<indirection1>(indirection1);
    if constexpr (std::is_pointer_v<M>) {
        using T = std::remove_cv_t<std::remove_pointer_t<M>>;
        rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>(RSBD8G_MEMBER2, off, indirection2);
        return gpu_detail::ok(rsbd8g_radixsort(&d, count, input, gpu_detail::stream_slot()));
    } else {
        rsbd8g_desc d = gpu_detail::makedesc<direction, mode, M>(RSBD8G_MEMBER, off);
        return gpu_detail::ok(rsbd8g_radixsort(&d, count, input, gpu_detail::stream_slot()));
    }
}

// ---- getter member function (evaluated on the host), with optional extra arguments ----------------

template <auto indirection1, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V, typename... vararguments>
[[nodiscard]] inline std::enable_if_t<std::is_member_function_pointer_v<decltype(indirection1)>, bool>
radixsortcopy(std::size_t count, V *const *input, V **output, int mmapflags = 0, vararguments &&...varparameters) {
    static_assert(indirection2 == 0 && !isindexed2, "getter results are the keys themselves on the GPU path");
    static_cast<void>(mmapflags);
    using T = std::remove_cv_t<std::remove_reference_t<decltype((std::declval<V *>()->*indirection1)(varparameters...))>>;
    static_assert(gpu_detail::iskeytype<T>, "unsupported getter result type");
    if (count < 2) {
        if (count == 1) return cudaMemcpy(output, input, sizeof(V *), cudaMemcpyDefault) == cudaSuccess;
        return true;
    }
    std::vector<V *> ptrs(count);
    if (cudaMemcpy(ptrs.data(), input, count * sizeof(V *), cudaMemcpyDefault) != cudaSuccess) return false;
    std::vector<T> keys(count);
    for (std::size_t i = 0; i < count; ++i) keys[i] = (ptrs[i]->*indirection1)(varparameters...);
    void *dkeys = nullptr;
    if (cudaMalloc(&dkeys, count * sizeof(T)) != cudaSuccess) return false;
    bool good = cudaMemcpy(dkeys, keys.data(), count * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
    if (good) {
        rsbd8g_desc d = gpu_detail::makedesc<direction, mode, T>(RSBD8G_KEYED);
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

// ---- type + offset: <T, indirection1, direction, mode, indirection2> -----------------------------
// T not a pointer: the key of type T sits at byte indirection1 of each object.
// T a pointer type U *: each object holds a pointer at byte indirection1 and the key of type U sits
// at byte indirection2 behind it.

template <typename T, std::ptrdiff_t indirection1 = 0, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<std::remove_pointer_t<T>>>, bool>
radixsortcopy(std::size_t count, V *const *input, V **output, int mmapflags = 0) noexcept {
    static_assert(!isindexed2, "indexed second-level indirection is not available on the GPU path");
    static_cast<void>(mmapflags);
    using K = std::remove_cv_t<std::remove_pointer_t<T>>;
    rsbd8g_desc d = std::is_pointer_v<T> ? gpu_detail::makedesc<direction, mode, K>(RSBD8G_MEMBER2, indirection1,
                                                                                    indirection2)
                                         : gpu_detail::makedesc<direction, mode, K>(RSBD8G_MEMBER, indirection1);
    return gpu_detail::ok(rsbd8g_radixsortcopy(&d, count, input, output, gpu_detail::stream_slot()));
}

template <typename T, std::ptrdiff_t indirection1 = 0, sortingdirection direction = sortingdirection::ascfwdorder,
          sortingmode mode = sortingmode::native, std::ptrdiff_t indirection2 = 0, bool isindexed2 = false,
          typename V>
[[nodiscard]] inline std::enable_if_t<gpu_detail::iskeytype<std::remove_cv_t<std::remove_pointer_t<T>>>, bool>
radixsort(std::size_t count, V **input, int mmapflags = 0) noexcept {
    static_assert(!isindexed2, "indexed second-level indirection is not available on the GPU path");
    static_cast<void>(mmapflags);
    using K = std::remove_cv_t<std::remove_pointer_t<T>>;
    rsbd8g_desc d = std::is_pointer_v<T> ? gpu_detail::makedesc<direction, mode, K>(RSBD8G_MEMBER2, indirection1,
                                                                                    indirection2)
                                         : gpu_detail::makedesc<direction, mode, K>(RSBD8G_MEMBER, indirection1);
    return gpu_detail::ok(rsbd8g_radixsort(&d, count, input, gpu_detail::stream_slot()));
}

}  // namespace rsbd8
