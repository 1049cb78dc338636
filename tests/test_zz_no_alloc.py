"""The allocation-free entry point, rsbd8g_radixsortcopy_static, called through the C ABI.

Some callers cannot call cudaMalloc (their framework owns all device memory, or the
implicit synchronisation is not acceptable); this entry point serves them from one
file-scope device array.  Its results must equal the allocating rsbd8g_radixsortcopy bit
for bit, on two calls in a row (the array is shared and keeps the previous call's bytes),
and counts beyond the array are refused.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu


def _static_entry():
    import radixsortbidi8_gb300 as rs
    f = rs.lib().rsbd8g_radixsortcopy_static
    f.argtypes = [ctypes.POINTER(rs.Desc), ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


CASES = [(np.uint32, "native", "ascfwdorder"), (np.float32, "nativeabs", "dscrevorder"),
         (np.int64, "native", "dscfwdorder"), (np.float64, "native", "ascrevorder"),
         (np.int16, "nativetieredabs", "ascfwdorder"), (np.uint8, "native", "dscrevorder")]


def _input(dt, n, seed):
    from radixsortbidi8_gb300 import synth as S
    a = S.float_specials(seed, n, dt) if np.dtype(dt).kind == "f" else S.uniform_bits(seed, n, dt)
    a[::11] = a[5]
    return a


@pytest.mark.parametrize("dt,mode,direction", CASES, ids=lambda x: str(getattr(x, "__name__", x)))
def test_static_entry_matches_allocating_entry_twice(dt, mode, direction):
    import torch
    import radixsortbidi8_gb300 as rs
    f = _static_entry()
    desc = rs.make_desc(dt, direction, mode)
    stream = torch.cuda.current_stream().cuda_stream
    for call, n in enumerate((1 << 20, (1 << 20) + 54321)):    # two calls in a row, sizes differ
        a = _input(dt, n, 40 + call)
        inp = to_dev(a)
        got, want = empty_dev(n, dt), empty_dev(n, dt)
        assert f(ctypes.byref(desc), n, inp.data_ptr(), got.data_ptr(), stream) == 0, call
        torch.cuda.synchronize()
        assert rs.radixsortcopy(inp, want, direction, mode, key_dtype=dt)
        assert same_bits(from_dev(got, dt), from_dev(want, dt)), call
        assert same_bits(from_dev(inp, dt), a)


def test_static_entry_refuses_counts_beyond_its_array():
    import torch
    import radixsortbidi8_gb300 as rs
    f = _static_entry()
    desc = rs.make_desc(np.uint32)
    x = torch.empty(4, dtype=torch.int32, device="cuda")
    y = torch.empty(4, dtype=torch.int32, device="cuda")
    # 2^24 four-byte keys need more than the 64 MiB array; nothing is launched
    assert f(ctypes.byref(desc), 1 << 24, x.data_ptr(), y.data_ptr(), None) == 6
    ind = rs.make_desc(np.uint32, indirection=1, offset1=0)
    assert f(ctypes.byref(ind), 100, x.data_ptr(), y.data_ptr(), None) == 1
    # still usable afterwards
    a = _input(np.uint32, 5000, 3)
    inp, out = to_dev(a), empty_dev(5000, np.uint32)
    assert f(ctypes.byref(desc), 5000, inp.data_ptr(), out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert same_bits(from_dev(out, np.uint32), np.sort(a, kind="stable"))
