"""Sorts whose arrays are managed memory or mapped pinned host memory rather than cudaMalloc memory.

The scatter passes prefetch tiles into L2 with bulk copies only when every array is device memory
(the library checks with cudaPointerGetAttributes); other memory the GPU can reach is read and
written with plain loads and stores.  These tests run both scatter kernels (the plain pass at 2^16
keys, the pipelined pass at 9 M keys) on such arrays and compare with numpy's stable sort.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    found = ctypes.util.find_library("cudart")
    if found:
        return ctypes.CDLL(found)
    pytest.skip("the CUDA runtime library is not loadable")


class _Alloc:
    """cudaMallocManaged / cudaHostAlloc(mapped) arrays, freed at the end of the test."""

    def __init__(self, kind):
        self.rt = _cudart()
        self.kind = kind
        self.ptrs = []

    def array(self, n, dtype):
        p = ctypes.c_void_p()
        nbytes = max(1, n * np.dtype(dtype).itemsize)
        if self.kind == "managed":
            assert self.rt.cudaMallocManaged(ctypes.byref(p), ctypes.c_size_t(nbytes), ctypes.c_uint(1)) == 0
        else:
            assert self.rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(nbytes), ctypes.c_uint(2)) == 0
        self.ptrs.append(p)
        buf = (ctypes.c_char * nbytes).from_address(p.value)
        return p.value, np.frombuffer(buf, dtype=dtype, count=n)

    def free(self):
        for p in self.ptrs:
            if self.kind == "managed":
                self.rt.cudaFree(p)
            else:
                self.rt.cudaFreeHost(p)


@pytest.mark.parametrize("kind", ["managed", "host_mapped"])
@pytest.mark.parametrize("n", [1 << 16, 9_000_000])
@pytest.mark.parametrize("dtype", [np.uint32, np.int64])
def test_sort_in_managed_and_host_memory(kind, n, dtype):
    import torch
    import radixsortbidi8_gb300 as rs
    from radixsortbidi8_gb300 import api
    torch.cuda.init()
    L = api.lib()
    a = _Alloc(kind)
    try:
        pin, vin = a.array(n, dtype)
        pout, vout = a.array(n, dtype)
        pbuf, _ = a.array(n, dtype)
        rng = np.random.default_rng(0x5EED00A1 + n)
        vin[:] = rng.integers(np.iinfo(dtype).min, np.iinfo(dtype).max, size=n, dtype=dtype, endpoint=True)
        want = np.sort(vin.copy(), kind="stable")
        desc = rs.make_desc(dtype)
        # allocating form: the scratch and buffer come from the library's pool, in/out are not device memory
        assert L.rsbd8g_radixsortcopy(ctypes.byref(desc), n, pin, pout, None) == 0
        assert a.rt.cudaDeviceSynchronize() == 0
        assert np.array_equal(vout, want)
        # noalloc form with the buffer in the same kind of memory
        vout[:] = 0
        nb = ctypes.c_size_t()
        assert L.rsbd8g_scratch_bytes(ctypes.byref(desc), n, ctypes.byref(nb)) == 0
        scr = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
        assert L.rsbd8g_radixsortcopynoalloc(ctypes.byref(desc), n, scr.data_ptr(), nb.value, pin, pout, pbuf,
                                             None) == 0
        assert a.rt.cudaDeviceSynchronize() == 0
        assert L.rsbd8g_scratch_status(scr.data_ptr(), None) == 0
        assert np.array_equal(vout, want)
    finally:
        a.rt.cudaDeviceSynchronize()
        a.free()
