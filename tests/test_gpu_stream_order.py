"""Work on the caller's stream is finished before a sort on another stream reads its arrays.

Each test keeps the current stream busy (torch.cuda._sleep, a bounded spin of about 20 ms), queues
the write of the input behind it, and calls the API at once: the batched sorter (its own stream),
the per-array loop on an explicit side stream, and the serving loop (the server's streams).  A sort
that did not wait would read the stale input (zeros) and differ from the oracle."""
import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev
from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = pytest.mark.gpu

SPIN_CYCLES = 40_000_000          # about 20 ms at 2 GHz


def _late_input(a: np.ndarray):
    """a device array that holds zeros now and `a` once the spin ahead of it on the current stream ends"""
    import torch
    src = to_dev(a)
    dst = torch.zeros_like(src)
    torch.cuda.synchronize()
    torch.cuda._sleep(SPIN_CYCLES)
    dst.copy_(src)                 # queued behind the spin
    return dst


def test_segmented_sorter_waits_for_the_callers_stream():
    import torch
    from radixsortbidi8_gb300 import batched as B
    lens = S.log_uniform_lengths(5, 300, 16, 1 << 14)
    offs = np.zeros(lens.size + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    a = S.uniform_bits(6, int(offs[-1]), np.uint32)
    off_t = torch.from_numpy(offs).cuda()
    keys = _late_input(a)
    sorter = B.SegmentedSorter(keys, off_t, "dscfwdorder", key_dtype=np.uint32)
    out = sorter.run()
    got = from_dev(out, np.uint32)            # read on the caller's stream, after the sort
    assert same_bits(got, O.sortcopy_segments(a, offs, "native", "dscfwdorder"))
    # a captured graph, replayed behind new input
    b = S.uniform_bits(7, int(offs[-1]), np.uint32)
    sorter.capture()
    src_b = to_dev(b)
    torch.cuda.synchronize()
    torch.cuda._sleep(SPIN_CYCLES)
    keys.copy_(src_b)              # queued behind the spin
    sorter.replay()
    assert same_bits(from_dev(sorter.output, np.uint32), O.sortcopy_segments(b, offs, "native", "dscfwdorder"))


def test_per_array_loop_on_a_side_stream_waits_for_the_callers_stream():
    import torch
    from radixsortbidi8_gb300 import batched as B
    lens = np.array([1000, 70000, 3, 4096], dtype=np.int64)
    offs = np.zeros(lens.size + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    a = S.uniform_bits(8, int(offs[-1]), np.int32)
    keys = _late_input(a)
    out = torch.empty_like(keys)
    side = torch.cuda.Stream()
    B.sort_each(keys, out, offs, key_dtype=np.int32, stream=side)
    side.synchronize()
    assert same_bits(from_dev(out, np.int32), O.sortcopy_segments(a, offs, "native", "ascfwdorder"))


def test_server_submit_waits_for_the_callers_stream():
    from radixsortbidi8_gb300 import serving
    a = S.float_specials(9, 300001, np.float32)
    x = _late_input(a)
    y = empty_dev(a.size, np.float32)
    with serving.Server(budget_bytes=256 << 20, max_inflight=2) as srv:
        rid = srv.submit(x, y, "dscfwdorder", "nativeabs", key_dtype=np.float32)
        assert srv.wait(rid).status == 0
    assert same_bits(from_dev(y, np.float32), O.sortcopy(a, "nativeabs", "dscfwdorder"))
