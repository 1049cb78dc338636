"""The allocation-free entry point, rsbd8g_radixsortcopy_static, called through the C ABI.

Some callers cannot call cudaMalloc (their framework owns all device memory, or the
implicit synchronisation is not acceptable); this entry point serves them from one
file-scope device array.  Its results must equal the allocating rsbd8g_radixsortcopy and
the oracle bit for bit, on two calls in a row (the array is shared and keeps the previous
call's bytes), at the largest counts the array takes and at count 1; counts beyond the
array are refused; and a device-side failure is reported by rsbd8g_static_status.  This
file is collected last on purpose.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu

STATIC_BYTES = 64 << 20          # the library's array
FLAG_DIAG_STALL = 1
ERR_TIMEOUT, ERR_TOO_LARGE = 4, 6


def _entries():
    import radixsortbidi8_gb300 as rs
    L = rs.lib()
    f = L.rsbd8g_radixsortcopy_static
    f.argtypes = [ctypes.POINTER(rs.Desc), ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    g = L.rsbd8g_static_status
    g.argtypes = [ctypes.c_void_p]
    g.restype = ctypes.c_int
    return f, g


CASES = [(np.uint32, "native", "ascfwdorder"), (np.float32, "nativeabs", "dscrevorder"),
         (np.int64, "native", "dscfwdorder"), (np.float64, "native", "ascrevorder"),
         (np.int16, "nativetieredabs", "ascfwdorder"), (np.uint8, "native", "dscrevorder")]


def _input(dt, n, seed):
    from radixsortbidi8_gb300 import synth as S
    a = S.float_specials(seed, n, dt) if np.dtype(dt).kind == "f" else S.uniform_bits(seed, n, dt)
    a[::11] = a[5]
    return a


def _oracle(a, mode, direction):
    from oracle import oracle as O
    return O.sortcopy(a, mode, direction, threads=os.cpu_count() or 1)


@pytest.mark.parametrize("dt,mode,direction", CASES, ids=lambda x: str(getattr(x, "__name__", x)))
def test_static_entry_matches_allocating_entry_and_oracle_twice(dt, mode, direction):
    import torch
    import radixsortbidi8_gb300 as rs
    f, status = _entries()
    desc = rs.make_desc(dt, direction, mode)
    stream = torch.cuda.current_stream().cuda_stream
    for call, n in enumerate((1 << 20, (1 << 20) + 54321)):    # two calls in a row, sizes differ
        a = _input(dt, n, 40 + call)
        inp = to_dev(a)
        got, want = empty_dev(n, dt), empty_dev(n, dt)
        assert f(ctypes.byref(desc), n, inp.data_ptr(), got.data_ptr(), stream) == 0, call
        assert status(stream) == 0, call
        assert rs.radixsortcopy(inp, want, direction, mode, key_dtype=dt)
        g = from_dev(got, dt)
        assert same_bits(g, from_dev(want, dt)), call
        assert same_bits(g, _oracle(a, mode, direction)), call
        assert same_bits(from_dev(inp, dt), a)


def _largest_count(dt) -> int:
    """The largest count whose scratch plus ping-pong buffer fits the array, found from
    rsbd8g_scratch_bytes (monotonic within one tile-size tier)."""
    import radixsortbidi8_gb300 as rs
    kb = np.dtype(dt).itemsize

    def fits(n):
        return rs.scratch_bytes(dt, n) + ((n * kb + 255) & ~255) <= STATIC_BYTES

    lo = 1 << 20 if kb == 8 else 1 << 23
    hi = STATIC_BYTES // kb + 1
    assert fits(lo) and not fits(hi)
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if fits(mid):
            lo = mid
        else:
            hi = mid
    return lo


@pytest.mark.parametrize("dt", [np.uint32, np.int64], ids=["uint32", "int64"])
def test_static_entry_at_the_largest_count_and_one_beyond(dt):
    import torch
    import radixsortbidi8_gb300 as rs
    f, status = _entries()
    n = _largest_count(dt)
    desc = rs.make_desc(dt, "dscfwdorder")
    stream = torch.cuda.current_stream().cuda_stream
    a = _input(dt, n, 77)
    inp, out = to_dev(a), empty_dev(n, dt)
    assert f(ctypes.byref(desc), n + 1, inp.data_ptr(), out.data_ptr(), stream) == ERR_TOO_LARGE
    assert f(ctypes.byref(desc), n, inp.data_ptr(), out.data_ptr(), stream) == 0
    assert status(stream) == 0
    assert same_bits(from_dev(out, dt), _oracle(a, "native", "dscfwdorder"))


def test_static_entry_count_one_and_refusals():
    import torch
    import radixsortbidi8_gb300 as rs
    f, status = _entries()
    desc = rs.make_desc(np.uint32)
    x = torch.tensor([7, 8, 9, 10], dtype=torch.int32, device="cuda")
    y = torch.full((4,), -1, dtype=torch.int32, device="cuda")
    # 2^24 four-byte keys need more than the 64 MiB array; nothing is launched
    assert f(ctypes.byref(desc), 1 << 24, x.data_ptr(), y.data_ptr(), None) == ERR_TOO_LARGE
    ind = rs.make_desc(np.uint32, indirection=1, offset1=0)
    assert f(ctypes.byref(ind), 100, x.data_ptr(), y.data_ptr(), None) == 1
    assert f(ctypes.byref(desc), 1, x.data_ptr(), y.data_ptr(), None) == 0       # one element: copied
    torch.cuda.synchronize()
    assert y.tolist() == [7, -1, -1, -1]
    # still usable afterwards
    a = _input(np.uint32, 5000, 3)
    inp, out = to_dev(a), empty_dev(5000, np.uint32)
    assert f(ctypes.byref(desc), 5000, inp.data_ptr(), out.data_ptr(), None) == 0
    assert status(None) == 0
    assert same_bits(from_dev(out, np.uint32), np.sort(a, kind="stable"))


def test_static_entry_reports_a_device_timeout_and_recovers():
    """RSBD8G_FLAG_DIAG_STALL: tile 1 of every scatter pass never publishes, so the tiles after it
    run into the bounded look-back wait (200 ms); the enqueue succeeds, rsbd8g_static_status
    returns RSBD8G_ERR_TIMEOUT (and clears it), and the next call sorts correctly."""
    import torch
    import radixsortbidi8_gb300 as rs
    f, status = _entries()
    n = 1 << 20
    a = _input(np.uint32, n, 5)
    inp, out = to_dev(a), empty_dev(n, np.uint32)
    stream = torch.cuda.current_stream().cuda_stream
    stall = rs.make_desc(np.uint32, flags=FLAG_DIAG_STALL)
    assert f(ctypes.byref(stall), n, inp.data_ptr(), out.data_ptr(), stream) == 0
    assert status(stream) == ERR_TIMEOUT
    assert status(stream) == 0                      # read and cleared
    desc = rs.make_desc(np.uint32)
    assert f(ctypes.byref(desc), n, inp.data_ptr(), out.data_ptr(), stream) == 0
    assert status(stream) == 0
    assert same_bits(from_dev(out, np.uint32), np.sort(a, kind="stable"))
