"""Python host mirror of the rsbd8 sorting API over the C ABI of ``librsbd8g.so``.

The functions keep the reference's names and argument meaning (Radixsortbidi8.hpp,
namespace rsbd8): ``radixsortcopy`` / ``radixsort`` (allocate, block until sorted,
return True, or False when the device allocation fails, :60398 / :60476) and
``radixsortcopynoalloc`` / ``radixsortnoalloc`` (caller-provided buffer and scratch,
stream-ordered, :60129 / :60163), with ``direction`` a ``sortingdirection`` name or
value and ``mode`` a ``sortingmode`` name or value.  Arrays are CUDA tensors (any
PyTorch dtype of the key's width; ``key_dtype`` names the key type when the tensor
dtype does not, e.g. int32 storage holding uint32 keys).  The member-pointer and
type+offset indirection forms take tensors of object addresses (uint64/int64) and the
key's byte offset.

There is no CPU path: without the CUDA library every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

MODES = {
    "native": 64, "nativeabs": 65, "nativetieredabs": 66,
    "forceunsigned": 0, "specialsigned": 0, "forcesigned": 2, "forceabssigned": 3,
    "forcefloatingp": 6, "forceabsfloatingp": 7, "specialunsigned": 7,
    "specialfloatingp": 4, "forcetieredabsfloatingp": 5, "forcetieredabssigned": 1,
}
DIRECTIONS = {"ascfwdorder": 0, "dscfwdorder": 1, "ascrevorder": 2, "dscrevorder": 3}

KIND_UNSIGNED, KIND_SIGNED, KIND_FLOAT, KIND_X87 = 0, 1, 2, 3
# 16-byte keys (arrays of two little-endian 64-bit words per key, 16-byte aligned): named by string
WIDE_KEY_KINDS = {"u128": KIND_UNSIGNED, "i128": KIND_SIGNED, "f128": KIND_FLOAT, "x87": KIND_X87}
DIRECT, MEMBER, MEMBER2 = 0, 1, 2
FLAG_DIAG_STALL = 1
FLAG_DIAG_NOMEM = 2
FLAG_DEVICE_ARRAYS = 4        # every array is device memory (include/rsbd8g.h)

STATUS = {0: "ok", 1: "bad argument", 2: "device allocation failed", 3: "CUDA runtime error",
          4: "device-side wait timed out", 5: "device-side fault flag", 6: "count too large",
          7: "admission refused: memory budget exhausted"}
OK, ERR_BAD_ARG, ERR_NO_MEMORY, ERR_CUDA, ERR_TIMEOUT, ERR_DEVICE_FAULT, ERR_TOO_LARGE, ERR_BUSY = range(8)


class RSBD8GError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} ({status})" if what else STATUS.get(status, str(status)))


class Desc(ctypes.Structure):
    """rsbd8g_desc of include/rsbd8g.h"""
    _fields_ = [("key_bytes", ctypes.c_uint32), ("key_kind", ctypes.c_uint32),
                ("mode", ctypes.c_uint32), ("direction", ctypes.c_uint32),
                ("indirection", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("offset1", ctypes.c_int64), ("offset2", ctypes.c_int64)]


_lib = None

# every symbol the C header declares (checked by the CPU test suite)
EXPORTS = ["rsbd8g_scratch_bytes", "rsbd8g_radixsortcopy", "rsbd8g_radixsort",
           "rsbd8g_radixsortcopynoalloc", "rsbd8g_radixsortnoalloc", "rsbd8g_scratch_status",
           "rsbd8g_status_string", "rsbd8g_version", "rsbd8g_profile_enable", "rsbd8g_profile_collect"]

KERNEL_NAMES = {0: "memset", 1: "histogram", 2: "plan", 3: "onesweep", 4: "copy", 5: "segmented", 6: "merge"}


class LaunchRecord(ctypes.Structure):
    """rsbd8g_launch_record of include/rsbd8g.h"""
    _fields_ = [("kernel", ctypes.c_uint32), ("key_bytes", ctypes.c_uint32), ("pass_", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("count", ctypes.c_uint64), ("ms", ctypes.c_double)]


def library_path() -> str:
    return _build.LIB


def lib():
    """Load librsbd8g.so (building it first if it is missing or stale); raises if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    L = ctypes.CDLL(path)
    P, S, U32, I32, VP = ctypes.POINTER(Desc), ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p
    sigs = {
        "rsbd8g_scratch_bytes": ([P, S, ctypes.POINTER(ctypes.c_size_t)], I32),
        "rsbd8g_radixsortcopy": ([P, S, VP, VP, VP], I32),
        "rsbd8g_radixsort": ([P, S, VP, VP], I32),
        "rsbd8g_radixsortcopynoalloc": ([P, S, VP, S, VP, VP, VP, VP], I32),
        "rsbd8g_radixsortnoalloc": ([P, S, VP, S, VP, VP, I32, VP], I32),
        "rsbd8g_scratch_status": ([VP, VP], I32),
        "rsbd8g_status_string": ([I32], ctypes.c_char_p),
        "rsbd8g_version": ([], I32),
        "rsbd8g_profile_enable": ([I32], I32),
        "rsbd8g_profile_collect": ([ctypes.POINTER(LaunchRecord), S, ctypes.POINTER(ctypes.c_size_t)], I32),
        "rsbd8g_radixsortcopy_static": ([P, S, VP, VP, VP], I32),
        "rsbd8g_static_status": ([VP], I32),
        "rsbd8g_binary_version": ([ctypes.POINTER(I32)], I32),
        "rsbd8g_prepare": ([ctypes.POINTER(Desc)], I32),
        "rsbd8g_merge_runs": ([P, S, ctypes.POINTER(ctypes.c_size_t), VP, VP, VP, VP], I32),
        "rsbd8g_radixsortcopy_chunked": ([P, S, VP, VP, S, VP], I32),
    }
    for name, (args, res) in sigs.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    _lib = L
    return L


# ---- descriptors ------------------------------------------------------------------------

_TORCH_TO_NP = {}


def _np_dtype(dt) -> np.dtype:
    """numpy dtype for a numpy or torch dtype."""
    if isinstance(dt, np.dtype):
        return dt
    try:
        return np.dtype(dt)
    except TypeError:
        pass
    import torch
    if not _TORCH_TO_NP:
        for t, n in [("bool", np.bool_), ("uint8", np.uint8), ("int8", np.int8), ("int16", np.int16),
                     ("uint16", np.uint16), ("int32", np.int32), ("uint32", np.uint32),
                     ("float32", np.float32), ("int64", np.int64), ("uint64", np.uint64),
                     ("float64", np.float64)]:
            if hasattr(torch, t):
                _TORCH_TO_NP[getattr(torch, t)] = np.dtype(n)
    if dt in _TORCH_TO_NP:
        return _TORCH_TO_NP[dt]
    raise TypeError(f"unsupported key type {dt}")


def key_kind(dtype) -> tuple[int, int]:
    """(kind, key bytes): what std::is_signed_v / is_floating_point_v say of the key type.
    16-byte keys are named "u128", "i128", "f128" (a 128-bit float word) or "x87" (x87 extended
    precision in 16-byte storage)."""
    if isinstance(dtype, str) and dtype in WIDE_KEY_KINDS:
        return WIDE_KEY_KINDS[dtype], 16
    dt = _np_dtype(dtype)
    if dt == np.bool_:
        return KIND_UNSIGNED, 1
    if dt.kind == "u":
        return KIND_UNSIGNED, dt.itemsize
    if dt.kind == "i":
        return KIND_SIGNED, dt.itemsize
    if dt.kind == "f" and dt.itemsize in (4, 8):
        return KIND_FLOAT, dt.itemsize
    raise TypeError(f"unsupported key type {dt}")


def _mode(m) -> int:
    return MODES[m] if isinstance(m, str) else int(m)


def _direction(d) -> int:
    return DIRECTIONS[d] if isinstance(d, str) else int(d)


def make_desc(key_dtype, direction="ascfwdorder", mode="native", indirection=DIRECT,
              offset1: int = 0, offset2: int = 0, flags: int = 0) -> Desc:
    kind, kb = key_kind(key_dtype)
    return Desc(kb, kind, _mode(mode), _direction(direction), indirection, flags, offset1, offset2)


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("arrays must be CUDA tensors (device-resident)")
        if not x.is_contiguous():
            raise ValueError("arrays must be contiguous")
        return x.data_ptr()
    raise TypeError(f"expected a CUDA tensor or a device address, got {type(x)}")


def _stream(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _check(st: int, what: str) -> None:
    if st != OK:
        raise RSBD8GError(st, what)


def _count(x, count, desc=None):
    if count is not None:
        return int(count)
    if desc is not None and desc.indirection == DIRECT and desc.key_bytes == 16:
        return int(x.numel() * x.element_size() // 16)       # 16-byte keys held in a wider-typed tensor
    return int(x.numel())


# ---- the rsbd8 entry points ---------------------------------------------------------------

def scratch_bytes(key_dtype, count: int, direction="ascfwdorder", mode="native", indirection=DIRECT,
                  offset1: int = 0, offset2: int = 0) -> int:
    """Scratch bytes a noalloc call needs (rsbd8::allocatearray sizing, Radixsortbidi8.hpp:59928)."""
    d = make_desc(key_dtype, direction, mode, indirection, offset1, offset2)
    out = ctypes.c_size_t(0)
    _check(lib().rsbd8g_scratch_bytes(ctypes.byref(d), count, ctypes.byref(out)), "rsbd8g_scratch_bytes")
    return out.value


def radixsortcopy(input, output, direction="ascfwdorder", mode="native", key_dtype=None, count=None,
                  stream=None, flags: int = 0) -> bool:
    """rsbd8::radixsortcopy<direction, mode>(count, input, output): True when sorted, False when
    the device allocation failed (the reference's only false return)."""
    d = make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode, flags=flags)
    st = lib().rsbd8g_radixsortcopy(ctypes.byref(d), _count(input, count, d), _ptr(input), _ptr(output),
                                    _stream(stream))
    if st == ERR_NO_MEMORY:
        return False
    _check(st, "radixsortcopy")
    return True


def radixsort(input, direction="ascfwdorder", mode="native", key_dtype=None, count=None, stream=None,
              flags: int = 0) -> bool:
    """rsbd8::radixsort<direction, mode>(count, input): in-place sort."""
    d = make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode, flags=flags)
    st = lib().rsbd8g_radixsort(ctypes.byref(d), _count(input, count, d), _ptr(input), _stream(stream))
    if st == ERR_NO_MEMORY:
        return False
    _check(st, "radixsort")
    return True


def radixsortcopynoalloc(input, output, buffer, scratch, direction="ascfwdorder", mode="native",
                         key_dtype=None, count=None, scratch_bytes_=None, stream=None, flags: int = 0) -> None:
    """rsbd8::radixsortcopynoalloc: caller buffer + scratch (a uint8 CUDA tensor), stream-ordered."""
    d = make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode, flags=flags)
    nbytes = scratch_bytes_ if scratch_bytes_ is not None else scratch.numel() * scratch.element_size()
    _check(lib().rsbd8g_radixsortcopynoalloc(ctypes.byref(d), _count(input, count, d), _ptr(scratch), nbytes,
                                             _ptr(input), _ptr(output), _ptr(buffer), _stream(stream)),
           "radixsortcopynoalloc")


def radixsortnoalloc(input, buffer, scratch, movetobuffer: bool = False, direction="ascfwdorder",
                     mode="native", key_dtype=None, count=None, scratch_bytes_=None, stream=None,
                     flags: int = 0) -> None:
    """rsbd8::radixsortnoalloc: in place (or into buffer with movetobuffer), stream-ordered."""
    d = make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode, flags=flags)
    nbytes = scratch_bytes_ if scratch_bytes_ is not None else scratch.numel() * scratch.element_size()
    _check(lib().rsbd8g_radixsortnoalloc(ctypes.byref(d), _count(input, count, d), _ptr(scratch), nbytes,
                                         _ptr(input), _ptr(buffer), int(bool(movetobuffer)), _stream(stream)),
           "radixsortnoalloc")


def scratch_status(scratch, stream=None) -> int:
    """Wait for the stream and read (and clear) the device status word of a scratch area."""
    return int(lib().rsbd8g_scratch_status(_ptr(scratch), _stream(stream)))


def merge_runs(input, output, run_counts, buffer=None, direction="ascfwdorder", mode="native", key_dtype=None,
               stream=None) -> None:
    """Stable merge of sorted runs lying back to back in `input` (lengths run_counts) into `output`
    (the reference's mergehalves* / mergethirds* for its halves / thirds split); `buffer` (as long
    as the runs together) when there are more than two runs.  Stream-ordered."""
    d = make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode)
    counts = (ctypes.c_size_t * max(1, len(run_counts)))(*[int(c) for c in run_counts])
    _check(lib().rsbd8g_merge_runs(ctypes.byref(d), len(run_counts), counts, _ptr(input), _ptr(output), _ptr(buffer),
                                   _stream(stream)), "rsbd8g_merge_runs")


def halves(count: int) -> list[int]:
    """The reference's split of an array into two parts (mergehalves*)."""
    return [count // 2, count - count // 2]


def thirds(count: int) -> list[int]:
    """The reference's split of an array into three parts (mergethirds*)."""
    return [count // 3, (count + 1) // 3, count - count // 3 - (count + 1) // 3]


def radixsortcopy_chunked(input, output, direction="ascfwdorder", mode="native", key_dtype=None,
                          device_bytes: int = 0, stream=None) -> bool:
    """rsbd8::radixsortcopy for keys in HOST memory (numpy arrays or CPU tensors) that need not fit
    the device: sorted in chunks within device_bytes (0: most of the free memory) and merged.
    Blocks until done; False when the device allocation failed."""
    def hptr(x):
        if isinstance(x, np.ndarray):
            if not x.flags["C_CONTIGUOUS"]:
                raise ValueError("arrays must be contiguous")
            return x.ctypes.data
        if hasattr(x, "data_ptr"):
            if x.is_cuda or not x.is_contiguous():
                raise ValueError("arrays must be contiguous host tensors")
            return x.data_ptr()
        raise TypeError(f"expected a host array, got {type(x)}")
    kd = key_dtype if key_dtype is not None else input.dtype
    d = make_desc(kd, direction, mode)
    n = int(input.size if isinstance(input, np.ndarray) else input.numel())
    if d.key_bytes == 16:
        n = n * (input.itemsize if isinstance(input, np.ndarray) else input.element_size()) // 16
    st = lib().rsbd8g_radixsortcopy_chunked(ctypes.byref(d), n, hptr(input), hptr(output), int(device_bytes),
                                            _stream(stream))
    if st == ERR_NO_MEMORY:
        return False
    _check(st, "radixsortcopy_chunked")
    return True


def binary_version() -> int:
    """The architecture the loaded kernels were compiled for, as the CUDA runtime reports it
    (103 for sm_103a); needs a device."""
    v = ctypes.c_int(0)
    _check(lib().rsbd8g_binary_version(ctypes.byref(v)), "rsbd8g_binary_version")
    return v.value


def prepare(key_dtype, direction="ascfwdorder", mode="native", indirection=DIRECT, offset1: int = 0,
            offset2: int = 0) -> None:
    """Load every kernel that sorts of this key type, mode and indirection can launch (rsbd8g_prepare),
    so that the first sort does not wait for the CUDA runtime to load them."""
    d = make_desc(key_dtype, direction, mode, indirection, offset1, offset2)
    _check(lib().rsbd8g_prepare(ctypes.byref(d)), "rsbd8g_prepare")


# ---- indirection --------------------------------------------------------------------------

def radixsortcopy_member(input, output, key_dtype, offset: int, direction="ascfwdorder", mode="native",
                         offset2: int | None = None, count=None, stream=None, flags: int = 0) -> bool:
    """rsbd8::radixsortcopy<T, offset, direction, mode> (type+offset) or <&V::member, ...>:
    sort an array of object addresses by the key of type key_dtype at byte `offset` of each object
    (with offset2: second level, the object holds a pointer at `offset`, the key is at offset2
    behind it).  input/output are uint64/int64 CUDA tensors of device addresses."""
    ind = MEMBER if offset2 is None else MEMBER2
    d = make_desc(key_dtype, direction, mode, ind, offset, offset2 or 0, flags)
    st = lib().rsbd8g_radixsortcopy(ctypes.byref(d), _count(input, count, d), _ptr(input), _ptr(output),
                                    _stream(stream))
    if st == ERR_NO_MEMORY:
        return False
    _check(st, "radixsortcopy (indirection)")
    return True


def radixsort_member(input, key_dtype, offset: int, direction="ascfwdorder", mode="native",
                     offset2: int | None = None, count=None, stream=None) -> bool:
    """rsbd8::radixsort<T, offset, direction, mode>: in-place sort of object addresses."""
    ind = MEMBER if offset2 is None else MEMBER2
    d = make_desc(key_dtype, direction, mode, ind, offset, offset2 or 0)
    st = lib().rsbd8g_radixsort(ctypes.byref(d), _count(input, count, d), _ptr(input), _stream(stream))
    if st == ERR_NO_MEMORY:
        return False
    _check(st, "radixsort (indirection)")
    return True


def radixsortcopynoalloc_member(input, output, buffer, scratch, key_dtype, offset: int, direction="ascfwdorder",
                                mode="native", offset2: int | None = None, count=None, stream=None) -> None:
    ind = MEMBER if offset2 is None else MEMBER2
    d = make_desc(key_dtype, direction, mode, ind, offset, offset2 or 0)
    nbytes = scratch.numel() * scratch.element_size()
    _check(lib().rsbd8g_radixsortcopynoalloc(ctypes.byref(d), _count(input, count, d), _ptr(scratch), nbytes,
                                             _ptr(input), _ptr(output), _ptr(buffer), _stream(stream)),
           "radixsortcopynoalloc (indirection)")


def profile_enable(on: bool = True) -> None:
    """Bracket every library kernel launch with CUDA events on its own stream."""
    _check(lib().rsbd8g_profile_enable(int(bool(on))), "rsbd8g_profile_enable")


def profile_collect(capacity: int = 1 << 16) -> list[dict]:
    """Wait for and return the recorded launches: dicts {kernel, key_bytes, pass, count, ms}."""
    recs = (LaunchRecord * capacity)()
    n = ctypes.c_size_t(0)
    _check(lib().rsbd8g_profile_collect(recs, capacity, ctypes.byref(n)), "rsbd8g_profile_collect")
    return [dict(kernel=KERNEL_NAMES.get(r.kernel, str(r.kernel)), key_bytes=r.key_bytes, pass_=r.pass_,
                 count=r.count, ms=r.ms) for r in recs[:min(n.value, capacity)]]


def loaded_library_path() -> str | None:
    """Path of the loaded CUDA library (None until first use)."""
    return os.path.abspath(_build.LIB) if _lib is not None else None
