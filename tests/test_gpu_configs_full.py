"""Bit-exact parity at the benchmark configurations' full sizes, through the C ABI.

Every output is copied to the host and compared byte for byte with the oracle's C restatement
run on the host copy of the same input:
  * the mode/dtype sweep, 2^28 keys per array (float32 descending with the absolute filter, in
    forward and in reverse tie order; int64 ascending; uint32 with 12 random low bits);
  * indirection: 2^26 records of 24 bytes sorted through their pointers by the double at byte 8,
    ascending, the exact pointer order (ties included);
  * the batched sort: every segment of the 2^28-key uint32 batch and of the float64 batch;
  * the serving loop: every request of a run of the serving configuration's request stream.
Inputs are built on the device with the generators the benchmark uses (synth.py).  Two more cases
sort 2^30 + 12345 keys, past the size where the look-back words widen to 8 bytes."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(1200)]

THREADS = os.cpu_count() or 1
SWEEP_SEED_WIDE = 0x5EED0030


def _host(t, dtype) -> np.ndarray:
    """Host copy of a device tensor, viewed as `dtype`."""
    return t.cpu().numpy().view(np.dtype(dtype))


def _bytes_equal(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


SWEEP = [("float32_abs_dscfwdorder", None), ("float32_abs_dscfwdorder", "dscrevorder"),
         ("int64_ascfwdorder", None), ("uint32_low12_ascfwdorder", None)]


@pytest.mark.parametrize("name,direction_override", SWEEP, ids=[f"{n}-{d or 'as-configured'}" for n, d in SWEEP])
def test_sweep_arrays_at_2p28_match_oracle(name, direction_override):
    import torch
    import radixsortbidi8_gb300 as rs
    n = 1 << 28
    arrays = {a[0]: a for a in S.sweep_arrays_torch(n)} if name != "int64_ascfwdorder" else None
    if arrays is None:                       # build only the array this case needs (2 GiB)
        bits = S.uniform_bits_torch(S.SWEEP_SEEDS["i64"], n, 8)
        kdt, direction, mode = np.int64, "ascfwdorder", "native"
    else:
        _, bits, kdt, direction, mode = arrays.pop(name)
        del arrays
    torch.cuda.empty_cache()
    direction = direction_override or direction
    out, buf = torch.empty_like(bits), torch.empty_like(bits)
    scr = torch.empty(rs.scratch_bytes(kdt, n, direction, mode), dtype=torch.uint8, device=bits.device)
    rs.radixsortcopynoalloc(bits, out, buf, scr, direction, mode, key_dtype=kdt)
    assert rs.scratch_status(scr) == 0
    a = _host(bits, kdt)
    got = _host(out, kdt)
    del bits, out, buf, scr
    torch.cuda.empty_cache()
    want = O.sortcopy(a, mode, direction, threads=THREADS)
    assert _bytes_equal(got, want)


def test_records_at_2p26_pointer_order_matches_oracle():
    import torch
    import radixsortbidi8_gb300 as rs
    n = 1 << 26
    rec = S.records24_torch(S.RECORDS_SEED, n)          # (n, 3) int64: 24-byte records
    base = rec.data_ptr()
    ptrs = torch.arange(n, dtype=torch.int64, device=rec.device) * 24 + base
    out = torch.empty_like(ptrs)
    assert rs.radixsortcopy_member(ptrs, out, np.float64, 8, "ascfwdorder")
    got = (out.cpu().numpy() - base) // 24
    rec_h = np.ascontiguousarray(rec.cpu().numpy())
    del rec, ptrs, out
    torch.cuda.empty_cache()
    hbase = rec_h.ctypes.data
    host_ptrs = np.uint64(hbase) + np.arange(n, dtype=np.uint64) * np.uint64(24)
    want = (O.sortcopy_indirect(host_ptrs, np.float64, 8, "native", "ascfwdorder", threads=THREADS)
            - np.uint64(hbase)) // np.uint64(24)
    assert np.array_equal(got, want.astype(np.int64))
    # the 10% duplicated keys: ties exist and kept input order (the index rises within a run)
    keys = rec_h[:, 1].view(np.float64)[got]
    tie = keys[1:] == keys[:-1]
    assert tie.sum() > n // 20
    assert bool(np.all(got[1:][tie] > got[:-1][tie]))


@pytest.mark.parametrize("which", ["A_2p28", "B"])
def test_batched_every_segment_matches_oracle(which):
    import torch
    from radixsortbidi8_gb300 import batched as B
    lens = S.batch_lengths(which)
    offs = np.zeros(lens.size + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    total = int(offs[-1])
    kdt = np.uint32 if which.startswith("A") else np.float64
    keys = S.batch_keys_torch(which, total)
    sorter = B.SegmentedSorter(keys, torch.from_numpy(offs).cuda(), key_dtype=kdt).capture()
    sorter.replay()
    sorter.replay()                  # a replay over the previous replay's buffers
    assert sorter.status() == 0
    got = _host(sorter.output, kdt)
    a = _host(keys, kdt)
    del sorter, keys
    torch.cuda.empty_cache()
    want = O.sortcopy_segments(a, offs, "native", "ascfwdorder", threads=THREADS)
    assert _bytes_equal(got, want)


def test_served_requests_of_the_serving_stream_match_oracle():
    """The first ~200 requests of the serving configuration (lengths log-uniform in [2^10, 2^26],
    uint16 / int32 / float32 / float64, ascending or descending, absolute filter half of the time)
    submitted at once to the serving loop; every result equals the oracle's sort of its input."""
    import torch
    from radixsortbidi8_gb300 import serving
    arr, lens, kind, desc, absf = S.serving_requests(2000.0, 0.1)
    nreq = arr.size
    tdt = {np.uint16: torch.int16, np.int32: torch.int32, np.float32: torch.int32, np.float64: torch.int64}
    ins, outs, metas = [], [], []
    for i in range(nreq):
        kd = S.SERVING_KINDS[kind[i]]
        m = int(lens[i])
        kb = np.dtype(kd).itemsize
        bits = S.float_specials_torch(S.SERVING_SEED + i, m, kb) if kd in (np.float32, np.float64) else \
            S.uniform_bits_torch(S.SERVING_SEED + i, m, kb)
        ins.append(bits.view(tdt[kd]))
        outs.append(torch.empty_like(ins[-1]))
        metas.append((kd, "dscfwdorder" if desc[i] else "ascfwdorder", "nativeabs" if absf[i] else "native"))
    with serving.Server(budget_bytes=64 << 30, max_inflight=4) as srv:
        ids = [srv.submit(ins[i], outs[i], metas[i][1], metas[i][2], key_dtype=metas[i][0]) for i in range(nreq)]
        srv.drain()
        infos = [srv.wait(r) for r in ids]
    assert all(x.status == 0 for x in infos)
    host_in = [_host(ins[i], metas[i][0]) for i in range(nreq)]
    got = [_host(outs[i], metas[i][0]) for i in range(nreq)]
    del ins, outs
    torch.cuda.empty_cache()
    want = O.sortcopy_batch([(host_in[i], metas[i][2], metas[i][1]) for i in range(nreq)], threads=THREADS)
    bad = [i for i in range(nreq) if not _bytes_equal(got[i], want[i])]
    assert not bad, bad[:10]


@pytest.mark.parametrize("name,kdt,mode,direction", [("uint32", np.uint32, "native", "ascfwdorder"),
                                                     ("float32_abs", np.float32, "nativeabs", "dscrevorder"),
                                                     ("int64", np.int64, "native", "dscfwdorder")])
def test_past_2p30_keys_with_wide_lookback_words_matches_oracle(name, kdt, mode, direction):
    """2^30 + 12345 keys: at 2^30 keys and more the look-back words widen to 8 bytes (62-bit counts)
    and the offsets of the write-out to 64 bits; the last tile is partly empty.  The float32 case
    also reads its first pass back to front (dscrevorder under the absolute filter)."""
    import torch
    import radixsortbidi8_gb300 as rs
    n = (1 << 30) + 12345
    kb = np.dtype(kdt).itemsize
    bits = (S.float_specials_torch(SWEEP_SEED_WIDE, n, kb) if kdt == np.float32
            else S.uniform_bits_torch(SWEEP_SEED_WIDE, n, kb))
    out, buf = torch.empty_like(bits), torch.empty_like(bits)
    scr = torch.empty(rs.scratch_bytes(kdt, n, direction, mode), dtype=torch.uint8, device=bits.device)
    rs.radixsortcopynoalloc(bits, out, buf, scr, direction, mode, key_dtype=kdt)
    assert rs.scratch_status(scr) == 0
    a = _host(bits, kdt)
    got = _host(out, kdt)
    del bits, out, buf, scr
    torch.cuda.empty_cache()
    assert _bytes_equal(got, O.sortcopy(a, mode, direction, threads=THREADS))
