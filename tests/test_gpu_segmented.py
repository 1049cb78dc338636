"""Batched (segmented) sort on the GPU: every segment bit-exact against the oracle sorting that
segment alone, for segment lists with empty, single, small, cutoff-boundary and multi-tile
segments, all modes that matter and all directions; graph capture and replay; and the
per-array loop giving the same bytes."""
import numpy as np
import pytest

from conftest import from_dev, same_bits, to_dev
from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = pytest.mark.gpu
DIRS = ["ascfwdorder", "dscfwdorder", "ascrevorder", "dscrevorder"]


def _segments(lens, dt, seed):
    lens = np.asarray(lens, dtype=np.int64)
    offs = np.zeros(lens.size + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    n = int(offs[-1])
    dt = np.dtype(dt)
    a = S.float_specials(seed, n, dt) if dt.kind == "f" else S.uniform_bits(seed, n, dt)
    if n > 10:
        a[::9] = a[4]
    return a, offs


def _check(a, offs, dt, mode, direction, tuning=None):
    import torch
    from radixsortbidi8_gb300 import batched as B
    inp = to_dev(a)
    off_t = torch.from_numpy(offs).cuda()
    s = B.SegmentedSorter(inp, off_t, direction, mode, key_dtype=dt, tuning=tuning)
    with torch.cuda.stream(s.stream):
        s.run()
    assert s.status() == 0
    got = from_dev(s.output, dt)
    for i in range(offs.size - 1):
        seg = a[offs[i]:offs[i + 1]]
        assert same_bits(got[offs[i]:offs[i + 1]], O.sortcopy(seg, mode, direction)), (i, offs[i + 1] - offs[i])
    return s


def _lens_mixed(cutoff, tile):
    return [0, 1, 2, 17, 0, cutoff - 1, cutoff, cutoff + 1, 3 * tile + 5, 1000, 7, 2 * tile, tile - 1,
            tile + 1, 50000, 31, 32, 33]


@pytest.mark.parametrize("dt,mode", [(np.uint32, "native"), (np.float32, "nativeabs"), (np.int64, "native"),
                                     (np.float64, "native"), (np.uint16, "native"), (np.int32, "nativetieredabs"),
                                     (np.uint8, "native")], ids=lambda x: str(getattr(x, "__name__", x)))
def test_segmented_matches_oracle_per_segment(dt, mode):
    from radixsortbidi8_gb300 import batched as B
    kb = np.dtype(dt).itemsize
    th, it = B.SMALL_SHAPES[kb][1]
    cutoff = th * it
    tile = 512 * (12 if kb == 8 else 16)
    a, offs = _segments(_lens_mixed(cutoff, tile), dt, 7 + kb)
    for d in DIRS:
        _check(a, offs, dt, mode, d)


def test_segmented_every_small_shape_and_cutoff():
    from radixsortbidi8_gb300 import batched as B
    lens = S.log_uniform_lengths(3, 400, 1, 20000)
    a, offs = _segments(lens, np.float32, 11)
    for v, (th, it) in enumerate(B.SMALL_SHAPES[4]):
        for cutoff in (0, th * it // 3):
            _check(a, offs, np.float32, "native", "dscrevorder", B.SegTuning(v, cutoff))


def test_segmented_pass_skip_and_all_equal_segments():
    lens = [5000, 40000, 3, 70000]
    a = np.concatenate([np.full(5000, 7, np.uint32), S.low_bits_u32(2, 40000), np.array([1, 1, 1], np.uint32),
                        np.full(70000, 123456, np.uint32)])
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    for d in DIRS:
        _check(a, offs, np.uint32, "native", d)
    f = np.where(np.arange(70000) % 3 == 0, np.float32(-0.0), np.float32(0.0))   # all keys tie
    offs2 = np.array([0, 20000, 70000], np.int64)
    for d in DIRS:
        _check(f, offs2, np.float32, "native", d)


def test_segmented_graph_replay_and_loop_agree():
    import torch
    from radixsortbidi8_gb300 import batched as B
    lens = S.log_uniform_lengths(5, 2000, 16, 1 << 16)
    a, offs = _segments(lens, np.uint32, 21)
    inp = to_dev(a)
    off_t = torch.from_numpy(offs).cuda()
    s = B.SegmentedSorter(inp, off_t, key_dtype=np.uint32).capture()
    s.output.zero_()
    s.replay()
    torch.cuda.synchronize()
    assert s.status() == 0
    got = from_dev(s.output, np.uint32)
    loop_out = torch.empty_like(inp)
    B.sort_each(inp, loop_out, offs, key_dtype=np.uint32)
    torch.cuda.synchronize()
    assert same_bits(got, from_dev(loop_out, np.uint32))
    want = np.concatenate([np.sort(a[offs[i]:offs[i + 1]], kind="stable") for i in range(offs.size - 1)])
    assert same_bits(got, want)
    # new data in the same buffers, same graph
    b = S.uniform_bits(22, a.size, np.uint32)
    inp.copy_(to_dev(b))
    s.replay()
    torch.cuda.synchronize()
    want = np.concatenate([np.sort(b[offs[i]:offs[i + 1]], kind="stable") for i in range(offs.size - 1)])
    assert same_bits(from_dev(s.output, np.uint32), want)


def test_segmented_lookback_timeout_reported():
    import torch
    from radixsortbidi8_gb300 import batched as B
    a, offs = _segments([200000, 300000], np.uint32, 3)
    inp = to_dev(a)
    out, buf = torch.empty_like(inp), torch.empty_like(inp)
    off_t = torch.from_numpy(offs).cuda()
    scratch = torch.empty(B.segmented_scratch_bytes(np.uint32, a.size, 2), dtype=torch.uint8, device="cuda")
    B.segmented_sortcopy(inp, out, buf, off_t, scratch, key_dtype=np.uint32, flags=1)
    from radixsortbidi8_gb300 import api
    assert api.scratch_status(scratch) == api.ERR_TIMEOUT
    _check(a, offs, np.uint32, "native", "ascfwdorder")


@pytest.mark.parametrize("large_variant", [0, 1])
@pytest.mark.parametrize("dt,mode,direction", [(np.uint32, "native", "dscrevorder"), (np.float64, "nativeabs", "ascrevorder")])
def test_segmented_pipelined_pass_matches_oracle(dt, mode, direction, large_variant):
    """A batch with tiles enough for the pipelined segmented pass (more than two per resident CTA):
    large segments of uneven sizes, small ones between them, consecutive tiles of one CTA crossing
    segment boundaries; both compiled tiles of the large segments."""
    from radixsortbidi8_gb300 import batched as B
    rng_lens = [1 << 20, 3, 700001, 0, 5000, (1 << 20) + 77, 12289, 1, 900007, 65536, 2 ** 19 + 5, 44444]
    lens = rng_lens * 2
    a, offs = _segments(lens, dt, 31)
    _check(a, offs, dt, mode, direction, B.SegTuning(1, 0, large_variant))


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.float64], ids=lambda x: x.__name__)
def test_segmented_second_large_tile_matches_oracle(dt):
    """large_variant 1 (512 x 20 keys up to 4 bytes, 512 x 16 for 8-byte keys) at its tile edges"""
    from radixsortbidi8_gb300 import batched as B
    kb = np.dtype(dt).itemsize
    th, it = B.SMALL_SHAPES[kb][1]
    lth, lit = B.LARGE_SHAPES[kb][1]
    a, offs = _segments(_lens_mixed(th * it, lth * lit), dt, 50 + kb)
    for d in DIRS:
        _check(a, offs, dt, "native", d, B.SegTuning(1, 0, 1))


@pytest.mark.parametrize("flags", [0, 4])
def test_segmented_pointer_tables_match_oracle(flags):
    """The pointer-table form (one separate device array per segment) with and without
    RSBD8G_FLAG_DEVICE_ARRAYS (= 4, which lets the pipelined pass prefetch tiles into L2), with
    arrays enough for the pipelined pass, against the oracle per array."""
    import torch
    from radixsortbidi8_gb300 import api, batched as B
    assert api.FLAG_DEVICE_ARRAYS == 4
    lens = [1 << 20, 3, 700001, 0, 5000, (1 << 20) + 77, 12289, 1, 900007, 65536, 2 ** 19 + 5, 44444] * 2
    arrays = [S.uniform_bits(101 + i, m, np.uint32) for i, m in enumerate(lens)]
    ins = [to_dev(x) if x.size else torch.empty(0, dtype=torch.int32, device="cuda") for x in arrays]
    outs = [torch.empty_like(x) for x in ins]
    bufs = [torch.empty_like(x) for x in ins]
    for direction in ("ascfwdorder", "dscrevorder"):
        scratch = torch.empty(B.segmented_scratch_bytes(np.uint32, sum(lens), len(lens)), dtype=torch.uint8,
                              device="cuda")
        keep = B.segmented_sortcopy_ptrs(ins, outs, bufs, scratch, direction, key_dtype=np.uint32, flags=flags)
        assert api.scratch_status(scratch) == 0
        del keep
        for x, o in zip(arrays, outs):
            assert same_bits(from_dev(o, np.uint32), O.sortcopy(x, "native", direction)), x.size


@pytest.mark.parametrize("dt,mode", [(np.float32, "nativeabs"), (np.int32, "native"), (np.float64, "native"),
                                     (np.uint16, "nativeabs")], ids=lambda x: str(getattr(x, "__name__", x)))
def test_segmented_per_segment_directions_match_oracle(dt, mode):
    """rsbd8g_segmented_sortcopy_ptrs_dirs: one launch sorts every array in its own direction --
    small, cutoff-sized and multi-tile arrays, reverse tie order where the mode honours it."""
    import torch
    from radixsortbidi8_gb300 import api, batched as B
    lens = [5, 0, 3000, 70001, 1, 40000, 9000, 250000, 33, 123457, 2, 16384]
    dirs = [DIRS[i % 4] for i in range(len(lens))]
    arrays = []
    for i, n in enumerate(lens):
        a, _ = _segments([n], dt, 300 + i)
        arrays.append(a)
    ins = [to_dev(a) if a.size else torch.empty(0, dtype=torch.int32, device="cuda") for a in arrays]
    outs = [torch.empty_like(x) for x in ins]
    bufs = [torch.empty_like(x) for x in ins]
    total = sum(lens)
    scratch = torch.empty(B.segmented_scratch_bytes(dt, total, len(lens), "ascfwdorder", mode), dtype=torch.uint8,
                          device="cuda")
    keep = B.segmented_sortcopy_ptrs(ins, outs, bufs, scratch, mode=mode, key_dtype=dt, directions=dirs)
    assert api.scratch_status(scratch) == 0
    del keep
    for a, o, d in zip(arrays, outs, dirs):
        if a.size:
            assert same_bits(from_dev(o, dt), O.sortcopy(a, mode, d)), (a.size, d)


def test_segmented_sixteen_byte_keys_match_oracle():
    """128-bit integer keys (two 64-bit words each) in the contiguous segmented form: small,
    cutoff-sized and multi-tile segments, every direction, against the oracle per segment; and the
    serving loop on the same kind of keys."""
    import torch
    from radixsortbidi8_gb300 import batched as B, serving
    lens = [0, 1, 2, 700, 1024, 1025, 5000, 3 * 3072 + 5, 70001, 12, 3072, 40000]
    offs = np.zeros(len(lens) + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    n = int(offs[-1])
    words = S.uniform_bits(61, 2 * n, np.uint64)
    words[4::10] = words[0]
    words[5::10] = words[1]                        # repeated keys
    inp = torch.from_numpy(words.view(np.int64).copy()).cuda()
    off_t = torch.from_numpy(offs).cuda()
    for kind in ("u128", "i128"):
        for d in DIRS:
            s = B.SegmentedSorter(inp, off_t, d, "native", key_dtype=kind)
            with torch.cuda.stream(s.stream):
                s.run()
            assert s.status() == 0
            got = s.output.cpu().numpy().view(np.uint64)
            for i in range(len(lens)):
                seg = words[2 * offs[i]:2 * offs[i + 1]]
                want = O.sortcopy_wide(seg, kind, "native", d).reshape(-1)
                assert same_bits(got[2 * offs[i]:2 * offs[i + 1]], want), (kind, d, i)
    outs = [torch.empty(2 * m, dtype=torch.int64, device="cuda") for m in lens]
    ins = [inp[2 * offs[i]:2 * offs[i + 1]] for i in range(len(lens))]
    with serving.Server(budget_bytes=1 << 30, max_inflight=2) as srv:
        ids = [srv.submit(ins[i], outs[i], DIRS[i % 4], "native", key_dtype="u128") for i in range(len(lens))]
        srv.drain()
        assert all(srv.wait(r).status == 0 for r in ids)
    for i in range(len(lens)):
        seg = words[2 * offs[i]:2 * offs[i + 1]]
        want = O.sortcopy_wide(seg, "u128", "native", DIRS[i % 4]).reshape(-1)
        assert same_bits(outs[i].cpu().numpy().view(np.uint64), want), i
