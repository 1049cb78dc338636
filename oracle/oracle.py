"""The oracle: the CPU restatement that verifies the GB300 radix sort (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only to verify results (or as the timed
CPU stand-in of the reference).  The product path never calls it.

Three independent CPU opinions live here:

* ``sortcopy`` / ``sortcopy_indirect`` -- the plain-C restatement of the
  reference's stable LSD radix sort (``rsbd8_oracle.c``, every part citing the
  Radixsortbidi8.hpp lines it follows), multithreaded with pthreads;
* ``numpy_sortcopy`` -- the same sort key K(b) fed to numpy's stable argsort,
  a second restatement that shares no code with the C one;
* ``ref_sortcopy`` / ``ref_indirect`` / ``ref_inplace`` -- the reference's own
  ``rsbd8::radixsortcopy`` / ``radixsort``, compiled from the reference header
  into ``_ref/librsbd8ref.so`` by ``make ref`` where the reference tree exists.
  Only the modes that are sound at the pinned snapshot are compiled in.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "librsbd8_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "librsbd8ref.so")

# rsbd8::sortingmode (Radixsortbidi8.hpp:212-250)
MODES = {
    "native": 64, "nativeabs": 65, "nativetieredabs": 66,
    "forceunsigned": 0, "specialsigned": 0, "forcesigned": 2, "forceabssigned": 3,
    "forcefloatingp": 6, "forceabsfloatingp": 7, "specialunsigned": 7,
    "specialfloatingp": 4, "forcetieredabsfloatingp": 5, "forcetieredabssigned": 1,
}
# rsbd8::sortingdirection (Radixsortbidi8.hpp:252-265)
DIRECTIONS = {"ascfwdorder": 0, "dscfwdorder": 1, "ascrevorder": 2, "dscrevorder": 3}

KIND_UNSIGNED, KIND_SIGNED, KIND_FLOAT = 0, 1, 2

_TYPE_NAMES = {
    np.dtype(np.uint8): "u8", np.dtype(np.int8): "i8", np.dtype(np.uint16): "u16",
    np.dtype(np.int16): "i16", np.dtype(np.uint32): "u32", np.dtype(np.int32): "i32",
    np.dtype(np.float32): "f32", np.dtype(np.uint64): "u64", np.dtype(np.int64): "i64",
    np.dtype(np.float64): "f64",
}


class Desc(ctypes.Structure):
    _fields_ = [("key_bytes", ctypes.c_uint32), ("absv", ctypes.c_uint32),
                ("sign", ctypes.c_uint32), ("fltp", ctypes.c_uint32),
                ("desc", ctypes.c_uint32), ("rev", ctypes.c_uint32),
                ("indirect", ctypes.c_uint32), ("pad_", ctypes.c_uint32),
                ("offset1", ctypes.c_int64), ("offset2", ctypes.c_int64)]


def kind_of(dtype) -> tuple[int, int]:
    """(kind, key bytes) of a numpy dtype, as std::is_signed_v / is_floating_point_v see it."""
    dt = np.dtype(dtype)
    if dt == np.bool_:
        return KIND_UNSIGNED, 1
    if dt.kind == "u":
        return KIND_UNSIGNED, dt.itemsize
    if dt.kind == "i":
        return KIND_SIGNED, dt.itemsize
    if dt.kind == "f" and dt.itemsize in (4, 8):
        return KIND_FLOAT, dt.itemsize
    raise TypeError(f"unsupported key type {dt}")


def _mode(m):
    return MODES[m] if isinstance(m, str) else int(m)


def _dir(d):
    return DIRECTIONS[d] if isinstance(d, str) else int(d)


def build(ref: bool = False) -> None:
    """Compile the C restatement (and, with ref=True, the reference adapter)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, "-j8"] + targets, check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        L.rsbd8o_resolve.argtypes = [ctypes.c_uint32] * 4 + [ctypes.POINTER(Desc)]
        L.rsbd8o_resolve.restype = ctypes.c_int
        L.rsbd8o_sortcopy.argtypes = [ctypes.POINTER(Desc), ctypes.c_uint64, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_uint]
        L.rsbd8o_sortcopy.restype = ctypes.c_int
        L.rsbd8o_sortkey.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(Desc)]
        L.rsbd8o_sortkey.restype = ctypes.c_uint64
        L.rsbd8o_skipmask.argtypes = [ctypes.POINTER(Desc), ctypes.c_uint64, ctypes.c_void_p,
                                      ctypes.c_uint32]
        L.rsbd8o_skipmask.restype = ctypes.c_uint32
        L.rsbd8o_sortcopy_batch.argtypes = [ctypes.c_uint64, ctypes.POINTER(Job), ctypes.c_uint]
        L.rsbd8o_sortcopy_batch.restype = ctypes.c_int
        _lib = L
    return _lib


def resolve(dtype, mode="native", direction="ascfwdorder", indirect: int = 0) -> Desc:
    kind, kb = kind_of(dtype)
    d = Desc()
    if lib().rsbd8o_resolve(kind, _mode(mode), _dir(direction), indirect, ctypes.byref(d)) != 0:
        raise ValueError(f"bad mode/direction {mode!r}/{direction!r}")
    d.key_bytes = kb
    return d


def sortcopy(a: np.ndarray, mode="native", direction="ascfwdorder", threads: int = 1) -> np.ndarray:
    """Stable sort of a plain key array, as rsbd8::radixsortcopy<direction, mode>."""
    a = np.ascontiguousarray(a)
    d = resolve(a.dtype, mode, direction)
    out = np.empty_like(a)
    rc = lib().rsbd8o_sortcopy(ctypes.byref(d), a.size, a.ctypes.data, out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"oracle sort failed ({rc})")
    return out


def sortcopy_indirect(ptrs: np.ndarray, key_dtype, offset1: int, mode="native",
                      direction="ascfwdorder", threads: int = 1, offset2: int | None = None) -> np.ndarray:
    """Stable sort of an array of object addresses by the key at byte offset1 of each object
    (second level when offset2 is given: the object holds a pointer at offset1 and the
    key sits at offset2 behind it), as rsbd8::radixsortcopy<T, offset1, ...>."""
    ptrs = np.ascontiguousarray(ptrs, dtype=np.uint64)
    d = resolve(key_dtype, mode, direction, indirect=2 if offset2 is not None else 1)
    d.offset1 = offset1
    d.offset2 = offset2 or 0
    out = np.empty_like(ptrs)
    rc = lib().rsbd8o_sortcopy(ctypes.byref(d), ptrs.size, ptrs.ctypes.data, out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"oracle sort failed ({rc})")
    return out


class Job(ctypes.Structure):
    """rsbd8o_job of rsbd8_oracle.h"""
    _fields_ = [("d", ctypes.POINTER(Desc)), ("n", ctypes.c_uint64), ("inp", ctypes.c_void_p),
                ("out", ctypes.c_void_p)]


def sortcopy_batch(items, threads: int = 1) -> list:
    """Independent stable sorts, `threads` at a time: items are (array, mode, direction);
    returns the sorted arrays (the reference's callers loop over radixsortcopy per array)."""
    arrays = [np.ascontiguousarray(a) for a, _, _ in items]
    outs = [np.empty_like(a) for a in arrays]
    descs = [resolve(a.dtype, m, d) for a, (_, m, d) in zip(arrays, items)]
    jobs = (Job * max(1, len(arrays)))()
    for i, (a, o, d) in enumerate(zip(arrays, outs, descs)):
        jobs[i].d = ctypes.pointer(d)
        jobs[i].n = a.size
        jobs[i].inp = a.ctypes.data
        jobs[i].out = o.ctypes.data
    rc = lib().rsbd8o_sortcopy_batch(len(arrays), jobs, threads)
    if rc != 0:
        raise RuntimeError(f"oracle batch sort failed ({rc})")
    return outs


def sortcopy_segments(a: np.ndarray, offsets: np.ndarray, mode="native", direction="ascfwdorder",
                      threads: int = 1) -> np.ndarray:
    """Every segment [offsets[s], offsets[s+1]) of `a` sorted on its own, as one
    rsbd8::radixsortcopy per segment; returns the concatenated result."""
    a = np.ascontiguousarray(a)
    out = np.empty_like(a)
    d = resolve(a.dtype, mode, direction)
    offs = np.asarray(offsets, dtype=np.int64)
    nseg = offs.size - 1
    jobs = (Job * max(1, nseg))()
    dp = ctypes.pointer(d)
    es = a.dtype.itemsize
    for s in range(nseg):
        jobs[s].d = dp
        jobs[s].n = int(offs[s + 1] - offs[s])
        jobs[s].inp = a.ctypes.data + int(offs[s]) * es
        jobs[s].out = out.ctypes.data + int(offs[s]) * es
    rc = lib().rsbd8o_sortcopy_batch(nseg, jobs, threads)
    if rc != 0:
        raise RuntimeError(f"oracle segmented sort failed ({rc})")
    return out


def skipmask(a: np.ndarray, mode="native", direction="ascfwdorder", digit_bits: int = 0) -> int:
    """Digits the pass-skip test drops (bit g = digit g of digit_bits bits; 0 = the reference's width)."""
    a = np.ascontiguousarray(a)
    d = resolve(a.dtype, mode, direction)
    return int(lib().rsbd8o_skipmask(ctypes.byref(d), a.size, a.ctypes.data, digit_bits))


# ---- the numpy restatement (independent of the C code) ----------------------------

def sortkeys(bits: np.ndarray, key_bytes: int, d: Desc) -> np.ndarray:
    """K(b) of raw bits (unsigned numpy array), vectorised; mirrors rsbd8_oracle.c sortkey."""
    w = key_bytes * 8
    ut = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[key_bytes]
    b = bits.astype(ut, copy=False)
    sb = ut(1 << (w - 1))
    mask = ut((1 << w) - 1)
    s = (b & sb) != 0
    m = b & ~sb
    zero = ut(0)
    one = ut(1)
    with np.errstate(over="ignore"):
        if d.absv != d.fltp:
            if d.absv:
                if d.sign:
                    k = np.where(s, zero - b, b)
                else:
                    k = (b << one) ^ np.where(s, mask, zero)
            else:
                if d.sign:
                    k = np.where(s, zero - m, m) ^ sb
                else:
                    k = np.where(s, mask ^ m, m)
        elif d.absv:
            if d.sign:
                k = m
            else:
                k = ((b << one) | (b >> ut(w - 1))) ^ one
        else:
            k = (b ^ sb) if d.sign else b.copy()
        if d.desc:
            k = ~k
    return k.astype(ut, copy=False)


def numpy_sortcopy(a: np.ndarray, mode="native", direction="ascfwdorder") -> np.ndarray:
    """Stable sort by K(b) with numpy's stable argsort (a second, independent restatement)."""
    a = np.ascontiguousarray(a)
    d = resolve(a.dtype, mode, direction)
    ut = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    src = a[::-1] if d.rev else a
    k = sortkeys(src.view(ut), a.dtype.itemsize, d)
    return src[np.argsort(k, kind="stable")]


def numpy_sort_indices(keys: np.ndarray, mode="native", direction="ascfwdorder", indirect=True) -> np.ndarray:
    """Permutation (source indices) the indirect sort applies, for keys gathered in pointer order."""
    keys = np.ascontiguousarray(keys)
    d = resolve(keys.dtype, mode, direction, indirect=1 if indirect else 0)
    ut = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[keys.dtype.itemsize]
    n = keys.size
    idx = np.arange(n)[::-1] if d.rev else np.arange(n)
    k = sortkeys(keys.view(ut)[idx], keys.dtype.itemsize, d)
    return idx[np.argsort(k, kind="stable")]


# ---- 16-byte keys -------------------------------------------------------------------
# Arrays of 16-byte keys are (n, 2) uint64 arrays of little-endian words [lo, hi].  Kinds:
#   "u128" / "i128"  128-bit integers (the reference's test128 without / with the sign flag),
#   "f128"           a 128-bit float word, sign in bit 127 (test128 with the float flags),
#   "x87"            x87 extended precision in 16-byte storage: 80-bit key, sign in bit 79; the
#                    upper 48 bits of `hi` are padding (longdoubletest128, Radixsortbidi8.hpp:1061-1100).

WIDE_KINDS = {"u128": (KIND_UNSIGNED, 64), "i128": (KIND_SIGNED, 64), "f128": (KIND_FLOAT, 64),
              "x87": (KIND_FLOAT, 16)}


def resolve_wide(kind: str, mode="native", direction="ascfwdorder", indirect: int = 0) -> Desc:
    k, _ = WIDE_KINDS[kind]
    d = Desc()
    if lib().rsbd8o_resolve(k, _mode(mode), _dir(direction), indirect, ctypes.byref(d)) != 0:
        raise ValueError(f"bad mode/direction {mode!r}/{direction!r}")
    d.key_bytes = 16
    return d


def sortkeys_wide(words: np.ndarray, kind: str, d: Desc) -> tuple[np.ndarray, np.ndarray]:
    """K(b) of 16-byte keys as (lo, hi) uint64 arrays: the 8 filter combinations of the
    (64 + HB)-bit key, the same formulas as sortkeys on narrower keys, with a carry between words."""
    hb = WIDE_KINDS[kind][1]
    u = np.uint64
    hm = u((1 << hb) - 1) if hb < 64 else u(0xFFFFFFFFFFFFFFFF)
    sb = u(1 << (hb - 1))
    lo = words[:, 0].astype(u)
    hi = words[:, 1].astype(u) & hm
    s = (hi & sb) != 0
    sm = np.where(s, u(0xFFFFFFFFFFFFFFFF), u(0))

    def add_s(l, h):                      # (l, h) + (sm, sm): subtract 1 where negative
        r = l + sm
        c = (r < l).astype(u)
        return r, (h + sm + c) & hm

    def shl1(l, h):
        return l << u(1), ((h << u(1)) | (l >> u(63))) & hm

    with np.errstate(over="ignore"):
        if d.absv != d.fltp:
            if d.absv:
                kl, kh = add_s(lo, hi) if d.sign else shl1(lo, hi)
                kl, kh = kl ^ sm, (kh ^ sm) & hm
            else:
                mh = hi & ~sb
                if d.sign:
                    kl, kh = add_s(lo, mh)
                    kl, kh = kl ^ sm, ((kh ^ sm) & hm) ^ sb
                else:
                    kl, kh = lo ^ sm, (mh ^ sm) & hm
        elif d.absv:
            if d.sign:
                kl, kh = lo, hi & ~sb
            else:
                kl, kh = shl1(lo, hi)
                kl = (kl | (hi >> u(hb - 1))) ^ u(1)
        else:
            kl, kh = (lo, hi ^ sb) if d.sign else (lo, hi)
        if d.desc:
            kl, kh = ~kl, ~kh & hm
    return kl, kh


def sortcopy_wide(words: np.ndarray, kind: str, mode="native", direction="ascfwdorder") -> np.ndarray:
    """Stable sort of 16-byte keys ((n, 2) uint64 words), as rsbd8::radixsortcopy<direction, mode>."""
    words = np.ascontiguousarray(words, dtype=np.uint64).reshape(-1, 2)
    d = resolve_wide(kind, mode, direction)
    src = words[::-1] if d.rev else words
    kl, kh = sortkeys_wide(src, kind, d)
    return src[np.lexsort((kl, kh))]            # lexsort is stable; the last key is the primary one


def sort_indices_wide(words: np.ndarray, kind: str, mode="native", direction="ascfwdorder") -> np.ndarray:
    """Permutation the indirect sort applies to objects whose 16-byte keys are `words` (pointer order)."""
    words = np.ascontiguousarray(words, dtype=np.uint64).reshape(-1, 2)
    d = resolve_wide(kind, mode, direction, indirect=1)
    n = words.shape[0]
    idx = np.arange(n)[::-1] if d.rev else np.arange(n)
    kl, kh = sortkeys_wide(words[idx], kind, d)
    return idx[np.lexsort((kl, kh))]


def ref_sortcopy_wide(words: np.ndarray, kind: str, mode, direction) -> np.ndarray:
    """The reference's own radixsortcopy on 16-byte keys (16-byte class under a forced mode, or
    long double as x87); KeyError where that combination is not instantiated."""
    words = np.ascontiguousarray(words, dtype=np.uint64).reshape(-1, 2)
    tn = "x87" if kind == "x87" else "w128"
    f = _reffn(f"rsbd8ref_copy_{tn}_m{_mode(mode)}_d{_dir(direction)}")
    out = np.zeros_like(words)
    rc = f(ctypes.c_uint64(words.shape[0]), ctypes.c_void_p(words.ctypes.data), ctypes.c_void_p(out.ctypes.data))
    if rc != 0:
        raise RuntimeError(f"reference sort failed ({rc})")
    return out


# ---- the reference's own sort (only where it was compiled) -------------------------

def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _reflib():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_SO)
    return _ref


def _reffn(name):
    try:
        f = getattr(_reflib(), name)
    except AttributeError:
        raise KeyError(name) from None
    f.restype = ctypes.c_int
    return f


def ref_sortcopy(a: np.ndarray, mode="native", direction="ascfwdorder") -> np.ndarray:
    """rsbd8::radixsortcopy<direction, mode> from the reference itself (KeyError if not compiled in)."""
    a = np.ascontiguousarray(a)
    f = _reffn(f"rsbd8ref_copy_{_TYPE_NAMES[a.dtype]}_m{_mode(mode)}_d{_dir(direction)}")
    f.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    out = np.empty_like(a)
    if f(a.size, a.ctypes.data, out.ctypes.data) != 0:
        raise RuntimeError("reference sort failed")
    return out


def ref_inplace(a: np.ndarray, mode="native", direction="ascfwdorder") -> np.ndarray:
    """rsbd8::radixsort<direction, mode> (in place) from the reference; returns the sorted copy."""
    a = np.ascontiguousarray(a).copy()
    f = _reffn(f"rsbd8ref_inplace_{_TYPE_NAMES[a.dtype]}_m{_mode(mode)}_d{_dir(direction)}")
    f.argtypes = [ctypes.c_uint64, ctypes.c_void_p]
    if f(a.size, a.ctypes.data) != 0:
        raise RuntimeError("reference sort failed")
    return a


def ref_indirect(ptrs: np.ndarray, key_dtype, mode="native", direction="ascfwdorder",
                 member: bool = False) -> np.ndarray:
    """rsbd8::radixsortcopy<T, 8, direction, mode> over pointers to 24-byte records holding the
    key at byte 8 (member=True: the <&rec24::key, direction> member-pointer form, double keys)."""
    ptrs = np.ascontiguousarray(ptrs, dtype=np.uint64)
    if member:
        f = _reffn(f"rsbd8ref_member_key_d{_dir(direction)}")
    else:
        f = _reffn(f"rsbd8ref_indirect8_{_TYPE_NAMES[np.dtype(key_dtype)]}_m{_mode(mode)}_d{_dir(direction)}")
    f.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    out = np.empty_like(ptrs)
    if f(ptrs.size, ptrs.ctypes.data, out.ctypes.data) != 0:
        raise RuntimeError("reference sort failed")
    return out
