"""The C-ABI library without a GPU: it loads, exports every function include/*.h declares,
sizes scratch, and rejects bad descriptors before touching the device."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import radixsortbidi8_gb300 as rs
from radixsortbidi8_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"RSBD8G_API\s+[\w\s\*]+?\b(rsbd8g_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("rsbd8g_radixsortcopy", "rsbd8g_radixsort", "rsbd8g_radixsortcopynoalloc",
                 "rsbd8g_radixsortnoalloc", "rsbd8g_scratch_bytes"):
        assert must in names


def test_library_loads_and_exports_every_declared_symbol():
    L = rs.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name
    assert L.rsbd8g_version() >= 100
    assert L.rsbd8g_status_string(4) == b"device-side wait timed out"


def test_library_is_built_for_sm103a_only():
    """Every translation unit is compiled with exactly one -gencode, for sm_103a (the GPU side
    checks what the runtime reports for the loaded module: test_gpu_parity.py)."""
    from radixsortbidi8_gb300 import build as B
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert not any("gencode" in f or "arch" in f for f in B.NVCC_FLAGS)


def test_scratch_sizes():
    s20 = rs.scratch_bytes(np.uint32, 1 << 20)
    s28 = rs.scratch_bytes(np.uint32, 1 << 28)
    assert 0 < s20 < s28
    # look-back state: one 4-byte word per (tile, bucket, digit) below 2^30 keys, 8 bytes above
    assert s28 < 300 << 20
    assert rs.scratch_bytes(np.uint64, 1 << 30) > 2 * rs.scratch_bytes(np.uint64, (1 << 30) - 1) * 0.9
    # indirection also holds the gathered keys twice
    assert rs.scratch_bytes(np.float64, 1 << 20, indirection=api.MEMBER, offset1=8) > 2 * 8 * (1 << 20)


def test_bad_descriptors_rejected_without_a_device():
    L = rs.lib()
    out = ctypes.c_size_t()
    for kb, kind, mode, d in [(3, 0, 64, 0), (4, 0, 9, 0), (4, 0, 64, 4), (2, 2, 64, 0), (4, 7, 64, 0)]:
        desc = api.Desc(kb, kind, mode, d, 0, 0, 0, 0)
        assert L.rsbd8g_scratch_bytes(ctypes.byref(desc), 10, ctypes.byref(out)) == api.ERR_BAD_ARG
        assert L.rsbd8g_radixsortcopy(ctypes.byref(desc), 10, 1, 2, None) == api.ERR_BAD_ARG
    good = api.make_desc(np.uint32)
    assert L.rsbd8g_scratch_bytes(ctypes.byref(good), 1 << 41, ctypes.byref(out)) == api.ERR_TOO_LARGE
    # count 0 is sorted already (the reference returns true without touching the arrays)
    assert L.rsbd8g_radixsortcopy(ctypes.byref(good), 0, None, None, None) == api.OK
    assert L.rsbd8g_radixsortcopy(ctypes.byref(good), 5, 4096, 4096, None) == api.ERR_BAD_ARG   # aliasing


def test_key_kinds_follow_std_type_traits():
    assert rs.key_kind(np.uint16) == (0, 2)
    assert rs.key_kind(np.int64) == (1, 8)
    assert rs.key_kind(np.float32) == (2, 4)
    assert rs.key_kind(np.bool_) == (0, 1)


def test_no_cpu_fallback_in_product_path():
    """The product package never imports the oracle."""
    for f in glob.glob(os.path.join(ROOT, "radixsortbidi8_gb300", "**", "*.py"), recursive=True):
        src = open(f).read()
        assert not re.search(r"^\s*(from|import)\s+oracle", src, re.M), f


def test_sixteen_byte_key_descriptors():
    """16-byte keys: 128-bit integer / float words and x87 extended precision; x87 only in 16 bytes."""
    import radixsortbidi8_gb300 as rs
    from radixsortbidi8_gb300 import api
    assert api.key_kind("u128") == (api.KIND_UNSIGNED, 16) and api.key_kind("x87") == (api.KIND_X87, 16)
    s16 = rs.scratch_bytes("u128", 1 << 20)
    s10 = rs.scratch_bytes("x87", 1 << 20)
    assert s16 > s10 > 0               # 16 digit passes of look-back words against 10
    L = api.lib()
    out = ctypes.c_size_t(0)
    for kb, kind in ((8, api.KIND_X87), (2, api.KIND_X87), (12, api.KIND_UNSIGNED), (16, 4)):
        d = api.Desc(kb, kind, 64, 0, 0, 0, 0, 0)
        assert L.rsbd8g_scratch_bytes(ctypes.byref(d), 1000, ctypes.byref(out)) == api.ERR_BAD_ARG, (kb, kind)


def test_tile_tiers_follow_the_count():
    """Keys of up to 4 bytes take 512 x 16 tiles below 2^23 keys, 512 x 24 up to 2^25 and 512 x 32
    from there on; the scratch size (look-back words: one per tile, digit pass and bucket) shows it."""
    kib = 1024
    for dt, passes in ((np.uint32, 4), (np.uint16, 2)):
        for n, tile in (((1 << 23) - 1, 8192), (1 << 23, 12288), ((1 << 25) - 1, 12288), (1 << 25, 16384)):
            tiles = -(-n // tile)
            body = tiles * passes * kib               # 256 buckets x 4 bytes per tile and pass
            s = rs.scratch_bytes(dt, n)
            assert body <= s < body + 128 * kib, (dt, n, s, body)
    # 8-byte keys keep 512 x 16 at every count below 2^30
    for n in ((1 << 23) - 1, 1 << 25):
        body = -(-n // 8192) * 8 * kib
        assert body <= rs.scratch_bytes(np.int64, n) < body + 128 * kib


def test_sort_array_lookup_of_the_control_block_indices(tmp_path):
    """The scatter and copy kernels find their arrays by index (rsbd8g::sort_array): valid indices,
    the 'none' index, and indices that name no array (fallback + fault flag), checked on the host."""
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    src = os.path.join(ROOT, "tests", "cpp", "sort_array_test.cu")
    exe = str(tmp_path / "sort_array_test")
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "radixsortbidi8_gb300", "csrc"),
                        src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_prepare_and_tuning_refusals_without_a_device():
    """rsbd8g_prepare refuses a bad descriptor before touching the device; the segmented scratch
    sizing refuses a small shape or large-segment tile that was not compiled."""
    L = rs.lib()
    L.rsbd8g_prepare.argtypes = [ctypes.POINTER(api.Desc)]
    L.rsbd8g_prepare.restype = ctypes.c_int
    assert L.rsbd8g_prepare(None) == api.ERR_BAD_ARG
    for kb, kind, mode in [(3, 0, 64), (4, 0, 9), (2, 2, 64), (4, 7, 64)]:
        assert L.rsbd8g_prepare(ctypes.byref(api.Desc(kb, kind, mode, 0, 0, 0, 0, 0))) == api.ERR_BAD_ARG
    from radixsortbidi8_gb300 import batched as B
    for t in (B.SegTuning(3, 0, 0), B.SegTuning(1, 0, 2), B.SegTuning(1, 1 << 20, 0)):
        with pytest.raises(api.RSBD8GError) as e:
            B.segmented_scratch_bytes(np.uint32, 100000, 20, tuning=t)
        assert e.value.status == api.ERR_BAD_ARG
    assert B.segmented_scratch_bytes(np.uint32, 100000, 20, tuning=B.SegTuning(1, 0, 1)) > 0
