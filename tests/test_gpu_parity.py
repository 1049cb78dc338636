"""GPU parity: the sm_103a sort through the C ABI against the oracle, bit for bit.

Every case sorts the same seeded input on the GPU and with the oracle's C restatement
(oracle/rsbd8_oracle.c) and compares the bytes: keys, tie order (stability, -0.0/+0.0,
NaN placement) and, for indirection, the exact pointer order.
"""
import os

import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev
from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = pytest.mark.gpu

DIRS = ["ascfwdorder", "dscfwdorder", "ascrevorder", "dscrevorder"]
TYPES = [np.uint8, np.int8, np.uint16, np.int16, np.uint32, np.int32, np.float32,
         np.uint64, np.int64, np.float64]
# around the scatter tiles: 12288 keys up to 4 bytes, 8192 for 8-byte keys, 4096 with a pointer payload
EDGE_SIZES = [2, 3, 31, 32, 33, 255, 256, 257, 4095, 4096, 4097, 8191, 8192, 8193, 12287, 12288, 12289,
              16385, 24575, 24577, 65543]
ALL_MODES = ["native", "nativeabs", "nativetieredabs", "forceunsigned", "forcesigned", "forceabssigned",
             "forcefloatingp", "forceabsfloatingp", "specialfloatingp", "forcetieredabsfloatingp",
             "forcetieredabssigned"]


def R():
    import radixsortbidi8_gb300 as rs
    return rs


def gpu_copy(a, mode="native", direction="ascfwdorder"):
    inp = to_dev(a)
    out = empty_dev(a.size, a.dtype)
    assert R().radixsortcopy(inp, out, direction, mode, key_dtype=a.dtype)
    # the input must be untouched
    assert same_bits(from_dev(inp, a.dtype), a)
    return from_dev(out, a.dtype)


def gpu_inplace(a, mode="native", direction="ascfwdorder"):
    t = to_dev(a)
    assert R().radixsort(t, direction, mode, key_dtype=a.dtype)
    return from_dev(t, a.dtype)


def mixed_input(dt, n, seed):
    """uniform bits, with specials for floats and duplicates for everyone"""
    dt = np.dtype(dt)
    if dt.kind == "f":
        a = S.float_specials(seed, n, dt)
    else:
        a = S.uniform_bits(seed, n, dt)
    if n > 8:
        a[:: 7] = a[3]      # duplicates
    return a


@pytest.mark.parametrize("dt", TYPES, ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("direction", DIRS)
def test_native_modes_all_types(dt, direction):
    for n in (0, 1, 2, 1000, 40009):
        a = mixed_input(dt, n, 100 + n)
        assert same_bits(gpu_copy(a, "native", direction), O.sortcopy(a, "native", direction)), (n,)


@pytest.mark.parametrize("mode", ALL_MODES)
@pytest.mark.parametrize("dt", [np.int16, np.int32, np.float32, np.int64, np.float64], ids=lambda t: np.dtype(t).name)
def test_every_mode_and_direction(mode, dt):
    if np.dtype(dt).itemsize == 2 and mode in ("forcefloatingp", "forceabsfloatingp",
                                             "specialfloatingp", "forcetieredabsfloatingp"):
        pass  # forced float modes on 16-bit keys are still defined (the mode bits pick the filter)
    a = mixed_input(dt, 30011, 7)
    for d in DIRS:
        assert same_bits(gpu_copy(a, mode, d), O.sortcopy(a, mode, d)), d


@pytest.mark.parametrize("n", EDGE_SIZES)
def test_edge_sizes_u32_f32(n):
    for dt, mode, d in [(np.uint32, "native", "ascfwdorder"), (np.float32, "native", "dscrevorder"),
                        (np.float32, "nativeabs", "dscfwdorder"), (np.int64, "native", "ascfwdorder")]:
        a = mixed_input(dt, n, n)
        assert same_bits(gpu_copy(a, mode, d), O.sortcopy(a, mode, d)), (dt, mode, d)


def test_pass_skip_low12_and_all_equal():
    # only the low 12 bits random: digits 2 and 3 skipped
    a = S.low_bits_u32(4, 1 << 20)
    assert O.skipmask(a, digit_bits=8) == 0b1100
    assert same_bits(gpu_copy(a), O.sortcopy(a))
    # every digit skipped: plain copy, reversed copy under isrevorder, in place too
    for dt, mode in [(np.uint32, "native"), (np.float32, "native"), (np.float32, "nativeabs")]:
        b = np.full(50000, 3, dtype=dt)
        if dt == np.float32:
            # -0.0 and +0.0 share one sort key; under the absolute filter so do -2.5 and 2.5
            b = np.where(np.arange(b.size) % 3 == 0, np.float32(-0.0), np.float32(0.0))
            if mode == "nativeabs":
                b = np.where(np.arange(b.size) % 3 == 0, np.float32(-2.5), np.float32(2.5))
        for d in DIRS:
            assert same_bits(gpu_copy(b, mode, d), O.sortcopy(b, mode, d)), (dt, mode, d)
            assert same_bits(gpu_inplace(b, mode, d), O.sortcopy(b, mode, d)), (dt, mode, d)


def test_two_keys_sorted_reversed():
    for a in (np.tile(np.array([5, 1], np.uint32), 30000), np.arange(100000, dtype=np.uint32),
              np.arange(100000, dtype=np.int32)[::-1].copy(), np.arange(-50000, 50000, dtype=np.int64)):
        for d in DIRS:
            assert same_bits(gpu_copy(a, "native", d), O.sortcopy(a, "native", d))


def test_float_lattice_and_int_extremes():
    f = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 1e-45, -1e-45, 1.0, -1.0,
                  3.4028235e38, -3.4028235e38, 1.1754944e-38, -1.1754944e-38], dtype=np.float32)
    f = np.tile(f, 997)
    f.view(np.uint32)[::13] ^= 0x00000001  # NaN payload / subnormal variants
    for mode in ALL_MODES:
        for d in DIRS:
            assert same_bits(gpu_copy(f, mode, d), O.sortcopy(f, mode, d)), (mode, d)
    i = np.tile(np.array([0, -1, 1, -2, 2, np.iinfo(np.int32).min, np.iinfo(np.int32).max, -3, 5, -5],
                         np.int32), 3001)
    for mode in ALL_MODES:
        for d in DIRS:
            assert same_bits(gpu_copy(i, mode, d), O.sortcopy(i, mode, d)), (mode, d)


def test_inplace_and_noalloc_forms():
    import torch
    rs = R()
    for dt, mode, d in [(np.uint32, "native", "ascfwdorder"), (np.float64, "native", "dscrevorder"),
                        (np.int16, "nativetieredabs", "ascfwdorder"), (np.float32, "nativeabs", "ascrevorder")]:
        for n in (5, 8193, 70001):
            a = mixed_input(dt, n, n + 1)
            want = O.sortcopy(a, mode, d)
            assert same_bits(gpu_inplace(a, mode, d), want)
            nbytes = rs.scratch_bytes(dt, n, d, mode)
            scratch = torch.full((nbytes,), 0x5A, dtype=torch.uint8, device="cuda")  # garbage content
            inp, out, buf = to_dev(a), empty_dev(n, dt), empty_dev(n, dt)
            rs.radixsortcopynoalloc(inp, out, buf, scratch, d, mode, key_dtype=dt)
            assert rs.scratch_status(scratch) == 0
            assert same_bits(from_dev(out, dt), want)
            for mtb in (False, True):
                x, b2 = to_dev(a), empty_dev(n, dt)
                rs.radixsortnoalloc(x, b2, scratch, mtb, d, mode, key_dtype=dt)
                assert rs.scratch_status(scratch) == 0
                assert same_bits(from_dev(b2 if mtb else x, dt), want), (dt, n, mtb)


def test_graph_capture_of_noalloc():
    import torch
    rs = R()
    n = 100003
    a = mixed_input(np.float32, n, 77)
    inp, out, buf = to_dev(a), empty_dev(n, np.float32), empty_dev(n, np.float32)
    scratch = torch.empty(rs.scratch_bytes(np.float32, n, "dscfwdorder"), dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())      # the arrays were made on the current stream
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        rs.radixsortcopynoalloc(inp, out, buf, scratch, "dscfwdorder", key_dtype=np.float32, stream=s)
        s.synchronize()
        with torch.cuda.graph(g, stream=s):
            rs.radixsortcopynoalloc(inp, out, buf, scratch, "dscfwdorder", key_dtype=np.float32, stream=s)
    want = O.sortcopy(a, "native", "dscfwdorder")
    for seed in (1, 2):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert same_bits(from_dev(out, np.float32), want)
    # new input bytes in the same buffers
    b = mixed_input(np.float32, n, 78)
    inp.copy_(to_dev(b))
    g.replay()
    torch.cuda.synchronize()
    assert same_bits(from_dev(out, np.float32), O.sortcopy(b, "native", "dscfwdorder"))


def test_lookback_timeout_is_reported_and_device_recovers():
    """A tile that never publishes makes its successors' bounded waits run out: the call
    reports a timeout instead of hanging, and the device keeps working."""
    rs = R()
    a = S.uniform_bits(9, 8192 * 6, np.uint32)
    inp, out = to_dev(a), empty_dev(a.size, np.uint32)
    with pytest.raises(rs.RSBD8GError) as e:
        rs.radixsortcopy(inp, out, key_dtype=np.uint32, flags=1)
    assert e.value.status == 4
    assert same_bits(gpu_copy(a), O.sortcopy(a))


def test_bad_arguments_rejected():
    import torch
    rs = R()
    a = to_dev(np.arange(100, dtype=np.uint32))
    with pytest.raises(rs.RSBD8GError):
        rs.radixsortcopy(a, a, key_dtype=np.uint32)          # aliasing
    with pytest.raises(rs.RSBD8GError):
        rs.radixsortcopy(a, empty_dev(100, np.uint32), mode=9, key_dtype=np.uint32)
    small = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(rs.RSBD8GError):
        rs.radixsortcopynoalloc(a, empty_dev(100, np.uint32), empty_dev(100, np.uint32), small, key_dtype=np.uint32)


@pytest.mark.parametrize("n", [2 ** 20, 2 ** 20 + 12345])
def test_config1_u32_uniform_bit_exact(n):
    a = S.uniform_bits(0x5EED0001, n, np.uint32)
    got = gpu_copy(a)
    assert same_bits(got, O.sortcopy(a, threads=8))
    assert same_bits(got, np.sort(a, kind="stable"))


# ---- indirection ----------------------------------------------------------------------------

def _records_dev(rec: np.ndarray):
    import torch
    raw = torch.from_numpy(rec.view(np.uint8).copy()).cuda()
    return raw, raw.data_ptr()


@pytest.mark.parametrize("direction", DIRS)
def test_indirect_records_f64_bit_exact(direction):
    import torch
    rs = R()
    n = 200003
    rec = S.records24(0x5EED0003, n)
    raw, base = _records_dev(rec)
    ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 24 + base
    out = torch.empty_like(ptrs)
    assert rs.radixsortcopy_member(ptrs, out, np.float64, 8, direction)
    idx = (out.cpu().numpy() - base) // 24
    # oracle on host copies of the same records
    host_ptrs = np.uint64(rec.ctypes.data) + np.arange(n, dtype=np.uint64) * np.uint64(24)
    want = (O.sortcopy_indirect(host_ptrs, np.float64, 8, "native", direction, threads=8)
            - np.uint64(rec.ctypes.data)) // np.uint64(24)
    assert np.array_equal(idx, want.astype(np.int64))
    assert np.array_equal(idx, O.numpy_sort_indices(rec["key"].copy(), "native", direction))


@pytest.mark.parametrize("kt,off", [(np.uint32, 8), (np.float32, 12), (np.int64, 0), (np.uint16, 16),
                                    (np.int32, 9), (np.uint64, 9), (np.float64, 17)])
def test_indirect_key_types_and_unaligned_offsets(kt, off):
    import torch
    rs = R()
    n, size = 50021, 25          # packed 25-byte objects: offsets 9 and 17 are unaligned
    bytes_ = S.uniform_bits(31, n * size, np.uint8)
    keys = mixed_input(kt, n, 5)
    kb = np.dtype(kt).itemsize
    obj = bytes_.reshape(n, size).copy()
    obj[:, off:off + kb] = keys.view(np.uint8).reshape(n, kb)
    raw = torch.from_numpy(obj.reshape(-1).copy()).cuda()
    base = raw.data_ptr()
    perm = np.argsort(S.splitmix64(3, n))  # shuffled pointer order
    ptrs = torch.from_numpy((perm * size).astype(np.int64)).cuda() + base
    for d in DIRS:
        out = torch.empty_like(ptrs)
        assert rs.radixsortcopy_member(ptrs, out, kt, off, d)
        idx = (out.cpu().numpy() - base) // size
        hobj = obj.reshape(-1)
        hp = np.uint64(hobj.ctypes.data) + (perm * size).astype(np.uint64)
        want = (O.sortcopy_indirect(hp, kt, off, "native", d) - np.uint64(hobj.ctypes.data)) // np.uint64(size)
        assert np.array_equal(idx, want.astype(np.int64)), d


def test_indirect_second_level_and_inplace():
    import torch
    rs = R()
    n = 30011
    keys = mixed_input(np.float32, n, 12)
    kdev = to_dev(keys)                                   # the keys, 4 bytes each
    # first-level objects: 16 bytes {u64 pad, u64 pointer to a key}
    holders = np.zeros((n, 2), dtype=np.uint64)
    holders[:, 1] = np.uint64(kdev.data_ptr()) + np.arange(n, dtype=np.uint64) * np.uint64(4)
    hdev = torch.from_numpy(holders.view(np.int64).reshape(-1).copy()).cuda()
    ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 16 + hdev.data_ptr()
    for d in DIRS:
        out = torch.empty_like(ptrs)
        assert rs.radixsortcopy_member(ptrs, out, np.float32, 8, d, offset2=0)
        idx = (out.cpu().numpy() - hdev.data_ptr()) // 16
        assert np.array_equal(idx, O.numpy_sort_indices(keys, "native", d)), d
        # in place
        p2 = ptrs.clone()
        assert rs.radixsort_member(p2, np.float32, 8, d, offset2=0)
        assert np.array_equal((p2.cpu().numpy() - hdev.data_ptr()) // 16, idx)


@pytest.mark.parametrize("n", [2, 33, 4095, 4096, 4097, 8193])
def test_indirect_tile_edges(n):
    """Pointer-payload sorts around their 4096-key tiles, against the oracle."""
    import torch
    rs = R()
    rec = S.records24(0x5EED0011, n)
    raw, base = _records_dev(rec)
    ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 24 + base
    host_ptrs = np.uint64(rec.ctypes.data) + np.arange(n, dtype=np.uint64) * np.uint64(24)
    for d in DIRS:
        out = torch.empty_like(ptrs)
        assert rs.radixsortcopy_member(ptrs, out, np.float64, 8, d)
        idx = (out.cpu().numpy() - base) // 24
        want = (O.sortcopy_indirect(host_ptrs, np.float64, 8, "native", d) - np.uint64(rec.ctypes.data)) // 24
        assert np.array_equal(idx, want.astype(np.int64)), d


def test_concurrent_calls_from_host_threads():
    """Calls on disjoint data from several host threads, each on its own stream, are independent
    (the reference's functions hold no shared mutable state either)."""
    import threading
    import torch
    rs = R()
    arrays = [mixed_input(dt, 200003 + 17 * i, 40 + i) for i, dt in
              enumerate([np.uint32, np.float32, np.int64, np.float64, np.uint16, np.int32])]
    results = [None] * len(arrays)
    errors = []

    def work(i):
        try:
            a = arrays[i]
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                x = to_dev(a)
                y = empty_dev(a.size, a.dtype)
                for _ in range(3):
                    assert rs.radixsortcopy(x, y, "dscrevorder", "native", key_dtype=a.dtype, stream=s)
                results[i] = from_dev(y, a.dtype)
        except Exception as e:      # reported below, on the main thread
            errors.append(e)

    th = [threading.Thread(target=work, args=(i,)) for i in range(len(arrays))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for a, got in zip(arrays, results):
        assert same_bits(got, O.sortcopy(a, "native", "dscrevorder")), a.dtype


def test_allocation_failure_returns_false_and_leaves_arrays():
    """The reference's only failure: the allocation of its scratch fails and radixsort /
    radixsortcopy return false.  Injected on the host with a diagnostics flag."""
    import torch
    from radixsortbidi8_gb300 import api
    rs = R()
    a = mixed_input(np.uint32, 10007, 3)
    x = to_dev(a)
    y = torch.full_like(x, 7)
    assert rs.radixsortcopy(x, y, key_dtype=np.uint32, flags=api.FLAG_DIAG_NOMEM) is False
    assert rs.radixsort(x, key_dtype=np.uint32, flags=api.FLAG_DIAG_NOMEM) is False
    assert same_bits(from_dev(x, np.uint32), a)
    assert bool((y == 7).all())
    assert rs.radixsortcopy(x, y, key_dtype=np.uint32)          # and the next call sorts
    assert same_bits(from_dev(y, np.uint32), O.sortcopy(a))


def test_lookback_timeout_in_the_pipelined_passes():
    """The same bounded wait in the pipelined scatter pass (enough tiles to fill its pipeline) and
    in the pipelined segmented pass: a timeout is reported, nothing hangs, the device keeps working."""
    import torch
    from radixsortbidi8_gb300 import api, batched
    rs = R()
    a = S.uniform_bits(19, 1 << 23, np.uint32)           # 683 tiles of 12288 keys
    inp, out = to_dev(a), empty_dev(a.size, np.uint32)
    with pytest.raises(rs.RSBD8GError) as e:
        rs.radixsortcopy(inp, out, key_dtype=np.uint32, flags=api.FLAG_DIAG_STALL)
    assert e.value.status == api.ERR_TIMEOUT
    offs = torch.arange(0, (1 << 23) + 1, 1 << 20, dtype=torch.int64, device="cuda")   # 8 segments of 2^20
    nb = batched.segmented_scratch_bytes(np.uint32, a.size, 8)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    buf = empty_dev(a.size, np.uint32)
    batched.segmented_sortcopy(inp, out, buf, offs, scratch, key_dtype=np.uint32, flags=api.FLAG_DIAG_STALL)
    assert api.scratch_status(scratch) == api.ERR_TIMEOUT
    assert same_bits(gpu_copy(a[:100003]), O.sortcopy(a[:100003]))


# sizes that fill the pipelined scatter pass (at least two tiles per resident CTA on a 152-SM GB300:
# 683 tiles of 12288 keys up to 4 bytes, 1025 of 8192 8-byte keys), every key size, filters,
# directions, in place
PIPE_CASES = [(np.uint8, 1 << 23, "native", "ascrevorder"), (np.int16, (1 << 23) + 5, "nativeabs", "dscfwdorder"),
              (np.uint32, (1 << 23) + 7, "native", "dscrevorder"), (np.float32, (1 << 23) + 1, "nativeabs", "dscrevorder"),
              (np.float32, 1 << 23, "nativetieredabs", "ascrevorder"), (np.int32, 1 << 23, "nativetieredabs", "dscfwdorder"),
              (np.int64, (1 << 23) + 3, "native", "ascfwdorder"), (np.float64, (1 << 23) + 9, "native", "dscrevorder"),
              (np.uint64, 1 << 23, 4, "ascrevorder"),
              # the 512 x 16 tiles of keys up to 4 bytes below 2^23 keys, pipelined from 608 tiles on
              (np.uint32, 6_000_011, "native", "ascrevorder"), (np.float32, (3 << 21) + 9, "nativeabs", "dscfwdorder")]


@pytest.mark.parametrize("dt,n,mode,direction", PIPE_CASES, ids=lambda v: str(v))
def test_pipelined_pass_matches_oracle(dt, n, mode, direction):
    a = mixed_input(dt, n, n % 1000)
    want = O.sortcopy(a, mode, direction, threads=8)
    assert same_bits(gpu_copy(a, mode, direction), want)
    assert same_bits(gpu_inplace(a, mode, direction), want)


def test_pipelined_pass_sixteen_byte_keys():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import torch
    from make_ref_wide import wide_input
    rs = R()
    for kind, gen, mode, d in (("x87", "x87", "native", "dscrevorder"), ("i128", "w128", "native", "ascfwdorder")):
        a = wide_input(gen, (1 << 21) + 11, 77)
        x = torch.from_numpy(a.view(np.int64).reshape(-1).copy()).cuda()
        y = torch.empty_like(x)
        assert rs.radixsortcopy(x, y, d, mode, key_dtype=kind)
        assert np.array_equal(y.cpu().numpy().view(np.uint64).reshape(-1, 2), O.sortcopy_wide(a, kind, mode, d)), kind


@pytest.mark.parametrize("direction", DIRS)
def test_pipelined_pass_pointer_payloads(direction):
    """Indirect sorts with enough 4096-pointer tiles to run the pipelined pass (2.6 M objects: at
    least two tiles per resident CTA), float64 keys in 24-byte records, against the oracle; and
    uint32 keys at an unaligned offset of packed 13-byte objects, copy and in place."""
    import torch
    rs = R()
    n = 2_600_017
    rec = S.records24(0x5EED0021, n)
    raw, base = _records_dev(rec)
    ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 24 + base
    out = torch.empty_like(ptrs)
    assert rs.radixsortcopy_member(ptrs, out, np.float64, 8, direction)
    idx = (out.cpu().numpy() - base) // 24
    host_ptrs = np.uint64(rec.ctypes.data) + np.arange(n, dtype=np.uint64) * np.uint64(24)
    want = (O.sortcopy_indirect(host_ptrs, np.float64, 8, "native", direction, threads=8)
            - np.uint64(rec.ctypes.data)) // np.uint64(24)
    assert np.array_equal(idx, want.astype(np.int64))
    size, off = 13, 5
    keys = mixed_input(np.uint32, n, 21)
    obj = S.uniform_bits(41, n * size, np.uint8).reshape(n, size).copy()
    obj[:, off:off + 4] = keys.view(np.uint8).reshape(n, 4)
    odev = torch.from_numpy(obj.reshape(-1).copy()).cuda()
    perm = np.argsort(S.splitmix64(5, n))
    p = torch.from_numpy((perm * size).astype(np.int64)).cuda() + odev.data_ptr()
    want_u = perm[O.numpy_sort_indices(keys[perm], "native", direction)]
    o2 = torch.empty_like(p)
    assert rs.radixsortcopy_member(p, o2, np.uint32, off, direction)
    assert np.array_equal((o2.cpu().numpy() - odev.data_ptr()) // size, want_u)
    assert rs.radixsort_member(p, np.uint32, off, direction)
    assert np.array_equal((p.cpu().numpy() - odev.data_ptr()) // size, want_u)


def _crowded(dt, n, seed):
    """Keys whose digit 1 is 0x5A for about 70 % of them (a crowded pass: most lanes of a ranking
    unit share one digit word) and uniform elsewhere, plus a run of equal keys."""
    a = S.uniform_bits(seed, n, dt)
    u = a.view(np.dtype(f"u{np.dtype(dt).itemsize}"))
    pick = (S.splitmix64(seed + 1, n) % np.uint64(10)) < np.uint64(7)
    u[pick] = (u[pick] & ~u.dtype.type(0xFF00)) | u.dtype.type(0x5A00)
    a[n // 3:n // 3 + 5000] = a[7]
    return a


@pytest.mark.parametrize("dt,n", [(np.uint32, 100003), (np.uint32, (1 << 23) + 3), (np.int64, 70001),
                                  (np.int64, (1 << 23) + 1), (np.float32, (1 << 23) + 5)])
def test_crowded_pass_matches_oracle(dt, n):
    """A pass whose histogram has a bucket with most of the keys: the plain and the pipelined scatter
    pass, every direction, copy and in place."""
    a = _crowded(dt, n, n % 977)
    for d in DIRS:
        want = O.sortcopy(a, "native", d, threads=8)
        assert same_bits(gpu_copy(a, "native", d), want), d
    assert same_bits(gpu_inplace(a, "native", "dscrevorder"), O.sortcopy(a, "native", "dscrevorder", threads=8))


def test_crowded_pass_pointer_payloads():
    """Warp ranking units under a crowded pass: an indirect sort whose float64 keys crowd one bucket
    (75 % equal keys), at a size that runs the pipelined pass."""
    import torch
    rs = R()
    n = 2_600_017
    rec = S.records24(0x5EED0031, n)
    k = rec["key"].copy()
    pick = (S.splitmix64(9, n) % np.uint64(4)) != np.uint64(0)
    k[pick] = 1.5                                  # 75 % equal keys: every digit crowded
    rec["key"] = k
    raw, base = _records_dev(rec)
    ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 24 + base
    for d in ("ascfwdorder", "dscrevorder"):
        out = torch.empty_like(ptrs)
        assert rs.radixsortcopy_member(ptrs, out, np.float64, 8, d)
        idx = (out.cpu().numpy() - base) // 24
        assert np.array_equal(idx, O.numpy_sort_indices(k, "native", d)), d


# counts from 2^25 up run keys of up to 4 bytes in 512 x 32 tiles
LARGE_TILE_CASES = [(np.uint32, (1 << 25) + 7, "native", "dscrevorder"), (np.float32, 1 << 25, "nativeabs", "ascrevorder"),
                    (np.int16, (1 << 25) + 3, "nativetieredabs", "dscfwdorder"), (np.uint8, (1 << 25) + 1, "native", "ascfwdorder"),
                    (np.int32, (1 << 25) + 11, "native", "ascfwdorder")]


@pytest.mark.parametrize("dt,n,mode,direction", LARGE_TILE_CASES, ids=lambda v: str(v))
def test_large_tile_pass_matches_oracle(dt, n, mode, direction):
    a = mixed_input(dt, n, n % 1013)
    want = O.sortcopy(a, mode, direction, threads=8)
    assert same_bits(gpu_copy(a, mode, direction), want)
    assert same_bits(gpu_inplace(a, mode, direction), want)


def test_loaded_module_is_sm103a():
    """The CUDA runtime reports the library's kernels as compiled for sm_103a."""
    assert R().api.binary_version() == 103


@pytest.mark.parametrize("n", [12345, (1 << 23) + 17, (1 << 25) + 3])
def test_crowded_digit_that_also_pads_the_last_tile(n):
    """A descending sort whose fullest bucket (60 % of the keys: top byte 0) becomes ranked digit 255,
    the digit the padding slots of a partial last tile take: the ballot-ranked digit and the padding
    must rank exactly as the table would."""
    a = S.uniform_bits(n % 991, n, np.uint32)
    pick = (S.splitmix64(n, n) % np.uint64(10)) < np.uint64(6)
    a[pick] &= np.uint32(0x00FFFFFF)
    for d in ("dscfwdorder", "ascfwdorder"):
        assert same_bits(gpu_copy(a, "native", d), O.sortcopy(a, "native", d, threads=8)), d
