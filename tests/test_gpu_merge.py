"""Stable merges of sorted runs (rsbd8g_merge_runs) and the chunked sort of host arrays
(rsbd8g_radixsortcopy_chunked) on the GPU, against the oracle.

Merging the parts of an array that were each sorted stably gives the stable sort of the whole
array: on equal keys the earlier part goes first (its elements came first), or the later part
when the direction reverses tie order -- the order the reference's mergehalves* / mergethirds*
produce for the halves and thirds its threads sort.  So every merge is checked against the
oracle's sort of the concatenated input, bit for bit."""
import os

import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev
from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = pytest.mark.gpu
DIRS = ["ascfwdorder", "dscfwdorder", "ascrevorder", "dscrevorder"]
THREADS = os.cpu_count() or 1


def _input(dt, n, seed, ties=True):
    dt = np.dtype(dt)
    a = S.float_specials(seed, n, dt) if dt.kind == "f" else S.uniform_bits(seed, n, dt)
    if ties and n > 8:
        a[::5] = a[3]                 # equal keys inside and across the parts
        a[1::7] = a[2]
    return a


def _sorted_parts(a, counts, mode, direction):
    """each part sorted on its own (by the oracle), back to back"""
    out, o = [], 0
    for c in counts:
        out.append(O.sortcopy(a[o:o + c], mode, direction))
        o += c
    return np.concatenate(out) if out else a[:0].copy()


def _merge(parts, counts, dt, mode, direction):
    from radixsortbidi8_gb300 import api
    n = parts.size
    inp, out = to_dev(parts), empty_dev(n, dt)
    buf = empty_dev(n, dt) if len(counts) > 2 else None
    api.merge_runs(inp, out, counts, buf, direction, mode, key_dtype=dt)
    import torch
    torch.cuda.synchronize()
    assert same_bits(from_dev(inp, dt), parts)          # the input is not written
    return from_dev(out, dt)


CASES = [(np.uint32, "native"), (np.float32, "nativeabs"), (np.float64, "native"), (np.int64, "native"),
         (np.int16, "nativetieredabs"), (np.uint8, "native"), (np.float32, "forcetieredabsfloatingp"),
         (np.int32, "forceabssigned")]


@pytest.mark.parametrize("dt,mode", CASES, ids=lambda x: str(getattr(x, "__name__", x)))
@pytest.mark.parametrize("split", ["halves", "thirds"])
def test_merge_of_sorted_parts_is_the_stable_sort(dt, mode, split):
    from radixsortbidi8_gb300 import api
    for n in (2, 3, 7, 4095, 4096, 4097, 100003, (1 << 20) + 17):
        a = _input(dt, n, n % 977 + 5)
        counts = api.halves(n) if split == "halves" else api.thirds(n)
        for d in DIRS:
            got = _merge(_sorted_parts(a, counts, mode, d), counts, dt, mode, d)
            assert same_bits(got, O.sortcopy(a, mode, d, threads=THREADS)), (n, d)


@pytest.mark.parametrize("counts", [[0, 5], [5, 0], [1, 1], [0, 0, 9], [3, 0, 4, 0, 2], [1000, 1, 1, 1, 70000, 5, 6],
                                    [8191] * 9, [12, 40000, 3, 3, 3, 50000, 1, 77, 65536, 2, 2]])
def test_merge_of_many_and_empty_runs(counts):
    n = sum(counts)
    for dt, mode in ((np.float32, "native"), (np.uint16, "native"), (np.int64, "nativeabs")):
        a = _input(dt, n, len(counts) + n % 101)
        for d in DIRS:
            got = _merge(_sorted_parts(a, counts, mode, d), counts, dt, mode, d)
            assert same_bits(got, O.sortcopy(a, mode, d)), (dt, d)


def test_merge_of_sixteen_byte_keys():
    from radixsortbidi8_gb300 import api
    import torch
    n = 30001
    words = S.uniform_bits(71, 2 * n, np.uint64)
    words[2::6] = words[0]
    words[3::6] = words[1]                          # repeated 128-bit keys
    counts = api.thirds(n)
    for kind in ("u128", "i128", "x87"):
        for d in DIRS:
            parts, o = [], 0
            for c in counts:
                parts.append(O.sortcopy_wide(words[2 * o:2 * (o + c)], kind, "native", d))
                o += c
            parts = np.concatenate(parts)
            inp = torch.from_numpy(parts.view(np.int64).copy()).cuda()
            out, buf = torch.empty_like(inp), torch.empty_like(inp)
            api.merge_runs(inp, out, counts, buf, d, "native", key_dtype=kind)
            torch.cuda.synchronize()
            got = out.cpu().numpy().view(np.uint64)
            assert same_bits(got, O.sortcopy_wide(words, kind, "native", d)), (kind, d)


def test_merge_rejects_bad_arguments():
    import ctypes
    import torch
    from radixsortbidi8_gb300 import api
    L = api.lib()
    d = api.make_desc(np.uint32)
    x = torch.empty(10, dtype=torch.int32, device="cuda")
    y = torch.empty(10, dtype=torch.int32, device="cuda")
    c3 = (ctypes.c_size_t * 3)(3, 3, 4)
    assert L.rsbd8g_merge_runs(ctypes.byref(d), 3, c3, x.data_ptr(), y.data_ptr(), None, None) == api.ERR_BAD_ARG
    assert L.rsbd8g_merge_runs(ctypes.byref(d), 3, c3, x.data_ptr(), x.data_ptr(), None, None) == api.ERR_BAD_ARG
    ind = api.make_desc(np.uint32, indirection=api.MEMBER, offset1=0)
    c2 = (ctypes.c_size_t * 2)(5, 5)
    assert L.rsbd8g_merge_runs(ctypes.byref(ind), 2, c2, x.data_ptr(), y.data_ptr(), None, None) == api.ERR_BAD_ARG
    assert L.rsbd8g_merge_runs(ctypes.byref(d), 0, None, None, None, None, None) == api.OK


# ---- the chunked sort of host arrays -----------------------------------------------------------

@pytest.mark.parametrize("dt,mode,direction", [(np.uint32, "native", "ascfwdorder"), (np.float32, "nativeabs", "dscrevorder"),
                                               (np.int64, "native", "dscfwdorder"), (np.float64, "native", "ascrevorder"),
                                               (np.uint16, "native", "ascfwdorder"), (np.int8, "nativetieredabs", "dscrevorder")],
                         ids=lambda x: str(getattr(x, "__name__", x)))
def test_chunked_sort_of_host_arrays_matches_oracle(dt, mode, direction):
    from radixsortbidi8_gb300 import api
    for n, budget in ((1 << 20, 0), ((1 << 20) + 3, 3 << 20), (300007, 1 << 20), (50000, 200000)):
        a = _input(dt, n, n % 89 + 1)
        out = np.empty_like(a)
        assert api.radixsortcopy_chunked(a, out, direction, mode, key_dtype=dt, device_bytes=budget)
        assert same_bits(out, O.sortcopy(a, mode, direction, threads=THREADS)), (n, budget)


def test_chunked_sort_with_many_chunks_at_2p26():
    """2^26 int32 keys with a 64 MiB device budget: dozens of chunks merged block by block."""
    from radixsortbidi8_gb300 import api
    n = 1 << 26
    a = _input(np.int32, n, 1234)
    out = np.empty_like(a)
    assert api.radixsortcopy_chunked(a, out, "dscrevorder", "nativeabs", key_dtype=np.int32, device_bytes=64 << 20)
    assert same_bits(out, O.sortcopy(a, "nativeabs", "dscrevorder", threads=THREADS))


def test_chunked_sort_refuses_a_budget_too_small_for_two_keys():
    from radixsortbidi8_gb300 import api
    a = _input(np.uint32, 1000, 3)
    out = np.empty_like(a)
    with pytest.raises(api.RSBD8GError) as e:
        api.radixsortcopy_chunked(a, out, key_dtype=np.uint32, device_bytes=1024)
    assert e.value.status == api.ERR_TOO_LARGE


def test_chunked_sort_of_sixteen_byte_keys():
    """128-bit integer keys in host memory, sorted in chunks within a small device budget."""
    from radixsortbidi8_gb300 import api
    n = 200003
    words = S.uniform_bits(17, 2 * n, np.uint64)
    words[6::14] = words[0]
    words[7::14] = words[1]
    out = np.empty_like(words)
    for d in ("ascfwdorder", "dscfwdorder"):
        assert api.radixsortcopy_chunked(words, out, d, "native", key_dtype="i128", device_bytes=2 << 20)
        want = O.sortcopy_wide(words, "i128", "native", d).reshape(-1)
        assert same_bits(out, want), d
